"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is the checker for the GPU engine: tests, the smoke check and the
CPU-baseline leg of bench.py load it.  The product never imports this module.
Every function here forwards to ``isspa_oracle.c``, which restates the
reference kernels of mccullaghlab/ISSPA-Force-Cuda (file:line citations there).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")

MULTIPOLE, LJ_TAB, CDD = 1, 2, 4          # IS-SPA force terms (Csolv, LJsolv, Csolv_CDD)
NB_LJ, NB_COUL, NB_CORR = 1, 2, 4         # nonbond terms (LJsolu, Csolu, Csolv_pair)


def build(force: bool = False) -> str:
    """Compile liborc.so from isspa_oracle.c with gcc (OpenMP, no FP contraction)."""
    src = os.path.join(HERE, "isspa_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
               "-o", LIB_PATH, src, "-lm"]
        subprocess.check_call(cmd)
    return LIB_PATH


class _IsspaSys(C.Structure):
    _fields_ = [("n_atoms", C.c_int), ("pos", C.c_void_p), ("isspa_type", C.c_void_p),
                ("n_itypes", C.c_int), ("rmax", C.c_void_p), ("vtot", C.c_void_p),
                ("n_g", C.c_int), ("n_e", C.c_int), ("n_f", C.c_int),
                ("g_table", C.c_void_p), ("e_table", C.c_void_p), ("f_table", C.c_void_p),
                ("g_r0", C.c_float), ("g_dr", C.c_float), ("e_r0", C.c_float),
                ("e_dr", C.c_float), ("f_r0", C.c_float), ("f_dr", C.c_float),
                ("box", C.c_float)]


class _NbSys(C.Structure):
    _fields_ = [("n_atoms", C.c_int), ("pos", C.c_void_p), ("n_types", C.c_int),
                ("lj_type", C.c_void_p), ("nb_parm_index", C.c_void_p), ("lj_ab", C.c_void_p),
                ("n_excl_cum", C.c_void_p), ("excl_list", C.c_void_p),
                ("isspa_type", C.c_void_p), ("rmax", C.c_void_p), ("box", C.c_float), ("cut2", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _pad(t, extra):
    t = _f64(t).ravel()
    return np.concatenate([t, np.zeros(extra, np.float64)])


class Oracle:
    """Oracle bound to one system (a ``isspa_gb300.System``-like object).

    Table values (ISSPA_DENSITIES / _EFIELD / _FORCES, LJ A and B) are held in
    FP64; `tables` may supply FP64 values that override the system's float ones
    (finite differences in the force-field parameters).  `nonbond_cutoff` > 0
    truncates the nonbond pairs and their energies at that distance (the
    engine's optional cutoff mode; every pair counts otherwise)."""

    def __init__(self, system, threads: int = 0, tables=None, nonbond_cutoff: float = 0.0):
        s = system
        self.s = s
        self.n = int(s.n_atoms)
        self.n_mc = int(s.n_mc)
        self._keep = []
        k = self._keep
        tables = tables or {}
        pos = _f32(s.pos).reshape(-1, 4)
        k.append(pos)
        self.pos = pos
        ityp = _i32(s.isspa_type); k.append(ityp)
        rmax = _f32(s.rmax); k.append(rmax)
        vtot = _f32(s.vtot()); k.append(vtot)
        gt = tables.get("g", s.g_table); et = tables.get("e", s.e_table); ft = tables.get("f", s.f_table)
        pad = max(gt.shape[1], et.shape[1], ft.shape[1]) + 1
        g = _pad(gt, pad); e = _pad(et, pad); f = _pad(ft, pad)
        k.extend([g, e, f])
        self.isys = _IsspaSys(self.n, _p(pos), _p(ityp), int(len(rmax)), _p(rmax), _p(vtot),
                              gt.shape[1], et.shape[1], ft.shape[1],
                              _p(g), _p(e), _p(f), s.g_r0, s.g_dr, s.e_r0, s.e_dr,
                              s.f_r0, s.f_dr, s.box)
        ljt = _i32(s.lj_type); nbp = _i32(s.nb_parm_index); lj = _f64(tables.get("lj_ab", s.lj_ab))
        self.lj = lj
        exc = _i32(s.n_excl_cum); exl = _i32(s.excl_list if len(s.excl_list) else [-1])
        k.extend([ljt, nbp, lj, exc, exl])
        rc = np.float32(nonbond_cutoff)
        self.nsys = _NbSys(self.n, _p(pos), int(s.n_lj_types), _p(ljt), _p(nbp), _p(lj),
                           _p(exc), _p(exl), _p(ityp), _p(rmax), s.box, float(rc * rc) if rc > 0 else 0.0)
        L = lib()
        L.orc_set_threads(int(threads))

    # -- IS-SPA ------------------------------------------------------------
    def mc_points(self, seed: int, step: int, window: int = 0) -> np.ndarray:
        out = np.zeros((self.n * self.n_mc, 3), np.float32)
        lib().orc_mc_points(C.byref(self.isys), self.n_mc, C.c_uint64(seed), C.c_uint32(step),
                            C.c_uint32(window), _p(out))
        return out

    def field(self, pts):
        pts = _f32(pts).reshape(-1, 3)
        P = pts.shape[0]
        w = np.zeros(P); cnt = np.zeros(P, np.int32)
        E = np.zeros((P, 3)); E0 = np.zeros((P, 3))
        lib().orc_field(C.byref(self.isys), self.n_mc, _p(pts), _p(w), _p(cnt), _p(E), _p(E0))
        return w, cnt, E, E0

    def isspa_force(self, pts, field=None, terms: int = 7) -> np.ndarray:
        pts = _f32(pts).reshape(-1, 3)
        if field is None:
            field = self.field(pts)
        w, cnt, E, E0 = field
        f = np.zeros((self.n, 3))
        lib().orc_isspa_force(C.byref(self.isys), self.n_mc, _p(pts), _p(np.ascontiguousarray(w)),
                              _p(_i32(cnt)), _p(np.ascontiguousarray(E)),
                              _p(np.ascontiguousarray(E0)), int(terms), _p(f))
        return f

    # -- subsets (large systems) -------------------------------------------
    def field_at(self, pts, idx):
        """Field pass at the point indices `idx` only (pts: all points)."""
        pts = _f32(pts).reshape(-1, 3)
        idx = np.ascontiguousarray(idx, np.int64)
        n = len(idx)
        w = np.zeros(n); cnt = np.zeros(n, np.int32); E = np.zeros((n, 3)); E0 = np.zeros((n, 3))
        lib().orc_field_at(C.byref(self.isys), self.n_mc, _p(pts), _p(idx), C.c_long(n), _p(w), _p(cnt),
                           _p(E), _p(E0))
        return w, cnt, E, E0

    def isspa_force_atoms(self, pts, field, atoms, terms: int = 7):
        """IS-SPA force on `atoms` from all points, given the field of all points."""
        pts = _f32(pts).reshape(-1, 3)
        w, cnt, E, E0 = field
        at = _i32(atoms)
        f = np.zeros((len(at), 3))
        lib().orc_isspa_force_atoms(C.byref(self.isys), self.n_mc, _p(pts), _p(np.ascontiguousarray(w, np.float64)),
                                    _p(_i32(cnt)), _p(np.ascontiguousarray(E, np.float64)),
                                    _p(np.ascontiguousarray(E0, np.float64)), int(terms), _p(at), len(at), _p(f))
        return f

    def nonbond_atoms(self, atoms, terms: int = 7):
        at = _i32(atoms)
        f = np.zeros((len(at), 3))
        lib().orc_nonbond_atoms(C.byref(self.nsys), int(terms), _p(at), len(at), _p(f))
        return f

    # -- pair / bonded terms ---------------------------------------------------
    def nonbond(self, terms: int = 7) -> np.ndarray:
        f = np.zeros((self.n, 3))
        lib().orc_nonbond(C.byref(self.nsys), int(terms), _p(f))
        return f

    def bonded(self, with_14: bool = True, bonds: bool = True, angles: bool = True,
               dihedrals: bool = True) -> np.ndarray:
        s = self.s
        f = np.zeros((self.n, 3))
        L = lib()
        ba = _i32(s.bond_atoms); bp = _f32(s.bond_params)
        aa = _i32(s.angle_atoms); ap = _f32(s.angle_params)
        da = _i32(s.dih_atoms); dt = _i32(s.dih_types); dp = _f32(s.dih_params)
        sc = _f32(s.scaled14)
        ljt = _i32(s.lj_type); nbp = _i32(s.nb_parm_index); lj = self.lj
        if bonds and len(ba):
            L.orc_bonds(len(ba), _p(ba), _p(bp), _p(self.pos), C.c_float(s.box), _p(f))
        if angles and len(aa):
            L.orc_angles(len(aa), _p(aa), _p(ap), _p(self.pos), C.c_float(s.box), _p(f))
        if dihedrals and len(da):
            L.orc_dihedrals(len(da), _p(da), _p(dt), _p(dp), _p(sc), _p(ljt), _p(nbp),
                            int(s.n_lj_types), _p(lj), _p(self.pos), C.c_float(s.box),
                            int(with_14), _p(f))
        return f

    ENERGY_NAMES = ("kin_before", "kin_after", "bond", "angle", "dihedral", "lj14", "coul14", "lj", "coul",
                    "corr", "umbrella", "virial")

    def energies(self, force, nb_terms: int = 7, with_us: bool = True) -> np.ndarray:
        """FP64 energy components (ENERGY_NAMES order) of the system's state;
        `force` [N][3] is the step's total force (for the kinetic energy after
        the kick)."""
        s = self.s
        out = np.zeros(12)
        ba = _i32(s.bond_atoms if len(s.bond_atoms) else np.zeros((1, 3))); bp = _f32(s.bond_params)
        aa = _i32(s.angle_atoms if len(s.angle_atoms) else np.zeros((1, 4))); ap = _f32(s.angle_params)
        da = _i32(s.dih_atoms if len(s.dih_atoms) else np.zeros((1, 4)))
        dt = _i32(s.dih_types if len(s.dih_types) else np.zeros(1))
        dp = _f32(s.dih_params if len(s.dih_params) else np.zeros((1, 4)))
        sc = _f32(s.scaled14 if len(s.scaled14) else np.ones((1, 2)))
        us = with_us and bool(s.us_on)
        bl = _i32(s.bias_list if us else np.zeros((1, 2)))
        mf = _f32(s.bias_mass_fraction() if us else np.zeros(1))
        vel = _f32(s.vel).reshape(-1, 4)
        fo = np.ascontiguousarray(force, dtype=np.float64).reshape(-1, 3)
        lib().orc_energies(C.byref(self.nsys), int(nb_terms), len(s.bond_atoms), _p(ba), _p(bp),
                           len(s.angle_atoms), _p(aa), _p(ap), len(s.dih_atoms), _p(da), _p(dt), _p(dp),
                           _p(sc), len(bl) if us else 0, _p(bl), _p(mf), C.c_double(float(s.us_k) if us else 0.0),
                           C.c_double(float(s.us_x0) if us else 0.0), _p(vel), _p(fo), C.c_float(s.dt), _p(out))
        return out

    def us(self):
        s = self.s
        f = np.zeros((self.n, 3))
        com = np.zeros((2, 3))
        if not s.us_on:
            return f, com
        lst = _i32(s.bias_list); mf = _f32(s.bias_mass_fraction())
        lib().orc_us(len(lst), _p(lst), _p(mf), C.c_double(s.us_k), C.c_double(s.us_x0),
                     _p(self.pos), C.c_float(s.box), _p(f), _p(com))
        return f, com

    def leapfrog(self, force, seed: int, step: int, window: int = 0):
        s = self.s
        vel = _f32(s.vel).reshape(-1, 4)
        po = np.zeros((self.n, 3)); vo = np.zeros((self.n, 3)); res = np.zeros(self.n, np.int32)
        fo = np.ascontiguousarray(force, dtype=np.float64)
        lib().orc_leapfrog(self.n, _p(self.pos), _p(vel), _p(fo), C.c_float(s.kT), C.c_float(s.dt),
                           C.c_float(s.pnu), C.c_float(s.box), C.c_uint64(seed), C.c_uint32(step),
                           C.c_uint32(window), _p(po), _p(vo), _p(res))
        return po, vo, res

    def neighbor_list(self, rnn: float, max_per_atom: int = 576):
        rows = np.full((self.n, max_per_atom), -1, np.int32)
        counts = np.zeros(self.n, np.int32)
        lib().orc_neighbor_list.restype = C.c_long
        lib().orc_neighbor_list(C.byref(self.nsys), C.c_float(rnn * rnn), int(max_per_atom),
                                _p(rows), _p(counts))
        return rows, counts

    def cell_index(self, rc: float, ncell):
        nc = _i32(ncell)
        cell = np.zeros(self.n, np.int32)
        lib().orc_cell_index(self.n, _p(self.pos), C.c_float(rc), _p(nc), _p(cell))
        return cell

    def com_axis_weights(self):
        """Per-atom weights c_i of the mean COM-axis force J = sum_i c_i . F_i:
        +n/2 on restraint group 0, -n/2 on group 1, n the unit vector from the
        group-1 to the group-0 centre of mass (mass fractions, minimum image as
        us_force_cuda.cu:30-31)."""
        s = self.s
        c = np.zeros((self.n, 3))
        if not s.us_on:
            return c
        _, com = self.us()
        d = com[0] - com[1]
        d -= s.box * np.where(d > 0.5 * s.box, 1.0, np.where(d < -0.5 * s.box, -1.0, 0.0))
        nh = d / np.linalg.norm(d)
        for a, g in np.asarray(s.bias_list).reshape(-1, 2):
            c[a] += (0.5 if g == 0 else -0.5) * nh
        return c

    def adjoint(self, pts, c=None):
        """FP64 adjoint of J = sum_i c_i . F_i (IS-SPA + nonbond + 1-4) for one
        frame: returns J and dJ/d(ISSPA_FORCES, ISSPA_DENSITIES, LJ A, LJ B)."""
        s = self.s
        c = self.com_axis_weights() if c is None else np.ascontiguousarray(c, np.float64)
        pts = _f32(pts).reshape(-1, 3)
        nt = len(s.rmax)
        df = np.zeros(nt * s.f_table.shape[1])
        dg = np.zeros(nt * s.g_table.shape[1])
        ntt = int(s.n_lj_types) * (int(s.n_lj_types) + 1) // 2
        dA = np.zeros(ntt)
        dB = np.zeros(ntt)
        da = _i32(s.dih_atoms if len(s.dih_atoms) else np.zeros((1, 4)))
        dt = _i32(s.dih_types if len(s.dih_types) else np.zeros(1))
        sc = _f32(s.scaled14 if len(s.scaled14) else np.ones((1, 2)))
        cc = np.ascontiguousarray(c, np.float64)
        L = lib()
        L.orc_adjoint.restype = C.c_double
        J = L.orc_adjoint(C.byref(self.isys), C.byref(self.nsys), self.n_mc, _p(pts), _p(cc),
                          int(len(s.dih_atoms)), _p(da), _p(dt), _p(sc), _p(df), _p(dg), _p(dA), _p(dB))
        return J, df.reshape(nt, -1), dg.reshape(nt, -1), dA, dB

    def mean_force(self, pts, c=None):
        """J = sum_i c_i . F_i over every non-restraint force term of one frame."""
        c = self.com_axis_weights() if c is None else c
        J = self.adjoint(pts, c)[0]
        s = self.s
        f = np.zeros((self.n, 3))
        L = lib()
        ba = _i32(s.bond_atoms); bp = _f32(s.bond_params)
        aa = _i32(s.angle_atoms); ap = _f32(s.angle_params)
        if len(ba):
            L.orc_bonds(len(ba), _p(ba), _p(bp), _p(self.pos), C.c_float(s.box), _p(f))
        if len(aa):
            L.orc_angles(len(aa), _p(aa), _p(ap), _p(self.pos), C.c_float(s.box), _p(f))
        if len(s.dih_atoms):
            L.orc_dihedrals(len(s.dih_atoms), _p(_i32(s.dih_atoms)), _p(_i32(s.dih_types)),
                            _p(_f32(s.dih_params)), _p(_f32(s.scaled14)), _p(_i32(s.lj_type)),
                            _p(_i32(s.nb_parm_index)), int(s.n_lj_types), _p(self.lj), _p(self.pos),
                            C.c_float(s.box), 0, _p(f))
        return J + float(np.sum(np.asarray(c) * f))

    def total_force(self, seed: int, step: int, window: int = 0, pts=None):
        """Forces of one full step, in the reference's call order
        (total_force_cuda.cpp:109-129): bonded, IS-SPA, nonbond, umbrella."""
        if pts is None:
            pts = self.mc_points(seed, step, window)
        f = self.bonded()
        f += self.isspa_force(pts)
        f += self.nonbond()
        fu, com = self.us()
        return f + fu, pts, com


def philox(ctr, key):
    out = (C.c_uint32 * 4)()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    lib().orc_philox4x32_10(c, k, out)
    return list(out)


def set_langevin_float_closed_forms(on: bool) -> None:
    """Diagnostic: evaluate <P1>, <P2>, <P3> with the reference's float closed
    forms (isspa_force_cuda.cu:270-287) instead of the accurate evaluation
    (process-wide until switched back)."""
    lib().orc_set_langevin_mode(1 if on else 0)


def langevin(x: float):
    out = (C.c_double * 3)()
    lib().orc_langevin(C.c_double(x), out)
    return list(out)
