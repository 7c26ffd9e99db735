"""Python handle on the GB300 engine (thin wrapper over the C ABI).

Method names follow the reference's per-step wrappers (bond_force_cuda,
isspa_force_cuda, ... in src/*_force_cuda.cu); each adds into the engine's
force accumulator exactly as the reference kernels add into for_d.
"""
from __future__ import annotations

import ctypes as C
import weakref
from typing import Iterable, Optional, Sequence

import numpy as np

from . import abi
from .system import System


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Engine:
    def __init__(self, windows: "System | Sequence[System]", isspa_terms: int = 7,
                 nonbond_terms: int = 7, use_graph: bool = True, field_split: int = 0,
                 force_chunk: int = 0, mem_cap: int = 0, force_atoms_per_thread: int = 0,
                 force_tail_chunk: int = 0, field_vote: int = 0, force_vote: int = 0, integrator: int = 0,
                 nonbond_chunk: int = 0, field_tma: int = 0, nonbond_cutoff: float = 0.0,
                 nonbond_skin: float = 0.0, nonbond_list_max: int = 0, step_pdl: int = 0,
                 isspa_fused: int = 0, force_overlap: int = 0):
        if isinstance(windows, System):
            windows = [windows]
        self.windows = list(windows)
        L = abi.lib()
        descs = (abi.SystemDesc * len(self.windows))()
        keep = []
        for k, w in enumerate(self.windows):
            d, kp = w.to_desc()
            descs[k] = d
            keep.append(kp)
        opt = abi.EngineOptions()
        L.isspa_default_options(C.byref(opt))
        opt.isspa_terms, opt.nonbond_terms = int(isspa_terms), int(nonbond_terms)
        opt.use_graph, opt.field_split, opt.force_chunk = int(use_graph), int(field_split), int(force_chunk)
        opt.mem_cap = int(mem_cap)
        opt.force_atoms_per_thread = int(force_atoms_per_thread)
        opt.force_tail_chunk = int(force_tail_chunk)
        opt.field_vote = int(field_vote)
        opt.force_vote = int(force_vote)
        opt.integrator = int(integrator)
        opt.nonbond_chunk = int(nonbond_chunk)
        opt.field_tma = int(field_tma)
        opt.nonbond_cutoff = float(nonbond_cutoff)
        opt.nonbond_skin = float(nonbond_skin)
        opt.nonbond_list_max = int(nonbond_list_max)
        opt.step_pdl = int(step_pdl)
        opt.isspa_fused = int(isspa_fused)
        opt.force_overlap = int(force_overlap)
        h = C.c_void_p()
        abi.check(L.isspa_engine_create(descs, len(self.windows), C.byref(opt), C.byref(h)), "engine create")
        self._h = h
        nw, na, npt = C.c_int(), C.c_int(), C.c_longlong()
        L.isspa_engine_info(h, C.byref(nw), C.byref(na), C.byref(npt))
        self.n_windows, self.n_atoms, self.n_points = nw.value, na.value, npt.value

    def shapes(self) -> dict:
        """Launch shapes chosen for the work lists (recorded with every benchmark)."""
        v = (C.c_int * abi.SHAPE_COUNT)()
        abi.check(abi.lib().isspa_engine_shapes(self._h, v), "shapes")
        keys = ("field_split", "field_tiles", "force_chunk", "force_items", "nonbond_items",
                "nonbond_partners_per_item", "sms", "force_atoms_per_thread", "force_tail_chunk",
                "field_vote", "force_vote", "integrator", "field_tma", "nonbond_list_rows", "nonbond_list_cells",
                "step_pdl", "isspa_fused", "force_overlap")
        return dict(zip(keys, list(v)))

    def nonbond_list_stats(self) -> dict:
        """Cutoff mode: list builds so far and the fullest row of the last build."""
        b, m = C.c_int(), C.c_int()
        abi.check(abi.lib().isspa_nonbond_list_stats(self._h, C.byref(b), C.byref(m)), "list stats")
        return {"builds": b.value, "fullest_row": m.value}

    def autotune(self, reps: int = 3) -> dict:
        """Time candidate launch shapes on this workload and keep the fastest."""
        v = (C.c_int * abi.SHAPE_COUNT)()
        abi.check(abi.lib().isspa_autotune(self._h, int(reps), v), "autotune")
        return self.shapes()

    # -------------------------------------------------------------- lifetime
    def close(self):
        if getattr(self, "_h", None):
            abi.lib().isspa_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -------------------------------------------------- per-step force calls
    def _call(self, name: str, timed: bool):
        ms = C.c_float(0.0)
        fn = getattr(abi.lib(), name)
        abi.check(fn(self._h, C.byref(ms) if timed else None), name)
        return ms.value if timed else None

    def zero_forces(self):
        abi.check(abi.lib().isspa_zero_forces(self._h), "zero")

    def bond_force(self, timed=False):
        return self._call("bond_force_cuda", timed)

    def angle_force(self, timed=False):
        return self._call("angle_force_cuda", timed)

    def dih_force(self, timed=False):
        return self._call("dih_force_cuda", timed)

    def isspa_force(self, timed=False):
        return self._call("isspa_force_cuda", timed)

    def nonbond_force(self, timed=False):
        return self._call("nonbond_force_cuda", timed)

    def us_force(self, timed=False):
        return self._call("us_force_cuda", timed)

    def leapfrog(self, timed=False):
        return self._call("leapfrog_cuda", timed)

    def compute_forces(self):
        """All force terms of one step in the reference order (total_force_cuda.cpp:109-129)."""
        self.zero_forces()
        self.bond_force()
        self.angle_force()
        self.dih_force()
        self.isspa_force()
        self.nonbond_force()
        self.us_force()
        return self.forces()

    def step(self, nsteps: int = 1):
        abi.check(abi.lib().isspa_step(self._h, int(nsteps)), "step")

    def time_steps(self, nsteps: int, flush_bytes: int = 0) -> float:
        ms = C.c_double(0.0)
        abi.check(abi.lib().isspa_time_steps(self._h, int(nsteps), int(flush_bytes), C.byref(ms)), "time")
        return ms.value

    KERNELS = ("field", "force", "nonbond", "bonded", "umbrella", "leapfrog", "integrator", "step")

    def time_steps_detailed(self, nsteps: int, flush_bytes: int = 0):
        """Device time of `nsteps` graph-replayed steps and of every kernel in them."""
        tot = C.c_double(0.0)
        kms = (C.c_double * len(self.KERNELS))()
        kn = (C.c_int * len(self.KERNELS))()
        abi.check(abi.lib().isspa_time_steps_detailed(self._h, int(nsteps), int(flush_bytes), C.byref(tot),
                                                       kms, kn), "time detailed")
        return tot.value, {k: (kms[i], kn[i]) for i, k in enumerate(self.KERNELS)}

    def synchronize(self):
        abi.check(abi.lib().isspa_synchronize(self._h), "synchronize")

    def device_status(self, reset: bool = False) -> int:
        return abi.lib().isspa_device_status(self._h, int(reset))

    # ------------------------------------------------------------ state I/O
    def _get4(self, name: str) -> np.ndarray:
        out = np.zeros((self.n_atoms, 4), np.float32)
        abi.check(getattr(abi.lib(), name)(self._h, _ptr(out), self.n_atoms), name)
        return out

    def positions(self):
        return self._get4("isspa_get_positions")

    def velocities(self):
        return self._get4("isspa_get_velocities")

    def forces(self) -> np.ndarray:
        return self._get4("isspa_get_forces")[:, :3]

    def set_positions(self, pos4):
        a = np.ascontiguousarray(pos4, np.float32).reshape(self.n_atoms, 4)
        abi.check(abi.lib().isspa_set_positions(self._h, _ptr(a), self.n_atoms), "set positions")

    def set_velocities(self, vel4):
        a = np.ascontiguousarray(vel4, np.float32).reshape(self.n_atoms, 4)
        abi.check(abi.lib().isspa_set_velocities(self._h, _ptr(a), self.n_atoms), "set velocities")

    def set_step(self, step: int):
        abi.check(abi.lib().isspa_set_step(self._h, int(step)), "set step")

    def get_step(self) -> int:
        s = C.c_uint32()
        abi.check(abi.lib().isspa_get_step(self._h, C.byref(s)), "get step")
        return s.value

    def us_com(self):
        com = np.zeros((self.n_windows, 2, 3))
        cv = np.zeros(self.n_windows)
        abi.check(abi.lib().isspa_get_us_com(self._h, _ptr(com), _ptr(cv)), "us com")
        return com, cv

    def step_host(self, pos_in, vel_in, pos_out, vel_out, force_out):
        """One step through isspa_step_host.  Each argument is None or a
        C-contiguous float32 array of n_atoms x 4 (outputs writeable); arrays
        from host_array are read and written by the GPU directly."""
        args = []
        for k, a in enumerate((pos_in, vel_in, pos_out, vel_out, force_out)):
            if a is None:
                args.append(None)
                continue
            if (a.dtype != np.float32 or a.size != 4 * self.n_atoms or not a.flags.c_contiguous
                    or (k >= 2 and not a.flags.writeable)):
                raise ValueError("step_host buffers: C-contiguous float32 arrays of n_atoms x 4, outputs writeable")
            args.append(a.ctypes.data)
        abi.check(abi.lib().isspa_step_host(self._h, *args), "step_host")

    # ----------------------------------------------------------- MC points
    def set_mc_points(self, xyz):
        a = np.ascontiguousarray(xyz, np.float32).reshape(self.n_points, 3)
        abi.check(abi.lib().isspa_set_mc_points(self._h, _ptr(a), self.n_points), "set points")

    def clear_mc_points(self):
        abi.check(abi.lib().isspa_clear_mc_points(self._h), "clear points")

    def point_fields(self):
        P = self.n_points
        xyz = np.zeros((P, 3), np.float32)
        w = np.zeros(P, np.float32)
        n = np.zeros(P, np.int32)
        E = np.zeros((P, 3), np.float32)
        E0 = np.zeros((P, 3), np.float32)
        abi.check(abi.lib().isspa_get_point_fields(self._h, _ptr(xyz), _ptr(w), _ptr(n), _ptr(E), _ptr(E0), P),
                  "point fields")
        return xyz, w, n, E, E0

    # ------------------------------------------------ force field and gradient
    def set_tables(self, g_table=None, e_table=None, f_table=None, lj_ab=None):
        """Replace force-field tables (same shapes as the System's)."""
        arrs = [None if t is None else np.ascontiguousarray(t, np.float32) for t in (g_table, e_table, f_table, lj_ab)]
        abi.check(abi.lib().isspa_set_tables(self._h, *[None if a is None else _ptr(a) for a in arrs]), "set tables")

    def adjoint_mean_force(self, steps, frames=None):
        """Mean COM-axis force J per window and dJ/d(ISSPA_FORCES, ISSPA_DENSITIES,
        LJ A, LJ B), averaged over frames (positions [F][Ntot][4] or None for the
        current positions) whose MC points come from the Philox keys `steps`."""
        w0 = self.windows[0]
        W = self.n_windows
        nt = len(w0.rmax)
        nF, nG = nt * w0.f_table.shape[1], nt * w0.g_table.shape[1]
        ntt = int(w0.n_lj_types) * (int(w0.n_lj_types) + 1) // 2
        st = np.ascontiguousarray(steps, np.uint32)
        fr = None if frames is None else np.ascontiguousarray(frames, np.float32).reshape(len(st), self.n_atoms, 4)
        J = np.zeros(W)
        df = np.zeros((W, nt, w0.f_table.shape[1]))
        dg = np.zeros((W, nt, w0.g_table.shape[1]))
        dA = np.zeros((W, ntt))
        dB = np.zeros((W, ntt))
        abi.check(abi.lib().isspa_adjoint_mean_force(self._h, len(st), None if fr is None else _ptr(fr), _ptr(st),
                                                     _ptr(J), _ptr(df), _ptr(dg), _ptr(dA), _ptr(dB)), "adjoint")
        return J, df, dg, dA, dB

    def energies(self) -> np.ndarray:
        """Energy components of the current state per window, FP64 kcal/mol,
        [n_windows][len(abi.ENERGY_NAMES)] (state unchanged)."""
        out = np.zeros((self.n_windows, len(abi.ENERGY_NAMES)))
        abi.check(abi.lib().isspa_energies(self._h, _ptr(out)), "energies")
        return out

    # --------------------------------------------------------------- lists
    def neighbor_list(self, rnn: float, max_per_atom: int = 576):
        n = self.windows[0].n_atoms
        rows = np.zeros((n, max_per_atom), np.int32)
        counts = np.zeros(n, np.int32)
        abi.check(abi.lib().isspa_neighbor_list(self._h, float(rnn), int(max_per_atom), _ptr(rows), _ptr(counts)),
                  "neighbor list")
        return rows, counts

    def cell_list(self, rc: float, ncell: Iterable[int]):
        nc = np.ascontiguousarray(list(ncell), np.int32)
        cell = np.zeros(self.windows[0].n_atoms, np.int32)
        abi.check(abi.lib().isspa_cell_list(self._h, float(rc), _ptr(nc), _ptr(cell)), "cell list")
        return cell


def host_array(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked, device-mapped memory (isspa_host_alloc),
    released through isspa_host_free once no view of it is left.  Engine.step_host
    with such arrays lets the GPU read and write them directly."""
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    p = C.c_void_p()
    abi.check(abi.lib().isspa_host_alloc(nbytes, C.byref(p)), "host alloc")
    buf = (C.c_char * nbytes).from_address(p.value)
    weakref.finalize(buf, abi.lib().isspa_host_free, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dt).reshape(shape)


def measure_fp32_peak() -> float:
    v = C.c_double()
    abi.check(abi.lib().isspa_measure_fp32_peak(C.byref(v)), "fp32 peak")
    return v.value
