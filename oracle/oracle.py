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
                ("isspa_type", C.c_void_p), ("rmax", C.c_void_p), ("box", C.c_float)]


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


def _pad(t, extra):
    t = _f32(t).ravel()
    return np.concatenate([t, np.zeros(extra, np.float32)])


class Oracle:
    """Oracle bound to one system (a ``isspa_gb300.System``-like object)."""

    def __init__(self, system, threads: int = 0):
        s = system
        self.s = s
        self.n = int(s.n_atoms)
        self.n_mc = int(s.n_mc)
        self._keep = []
        k = self._keep
        pos = _f32(s.pos).reshape(-1, 4)
        k.append(pos)
        self.pos = pos
        ityp = _i32(s.isspa_type); k.append(ityp)
        rmax = _f32(s.rmax); k.append(rmax)
        vtot = _f32(s.vtot()); k.append(vtot)
        pad = max(s.g_table.shape[1], s.e_table.shape[1], s.f_table.shape[1]) + 1
        g = _pad(s.g_table, pad); e = _pad(s.e_table, pad); f = _pad(s.f_table, pad)
        k.extend([g, e, f])
        self.isys = _IsspaSys(self.n, _p(pos), _p(ityp), int(len(rmax)), _p(rmax), _p(vtot),
                              s.g_table.shape[1], s.e_table.shape[1], s.f_table.shape[1],
                              _p(g), _p(e), _p(f), s.g_r0, s.g_dr, s.e_r0, s.e_dr,
                              s.f_r0, s.f_dr, s.box)
        ljt = _i32(s.lj_type); nbp = _i32(s.nb_parm_index); lj = _f32(s.lj_ab)
        exc = _i32(s.n_excl_cum); exl = _i32(s.excl_list if len(s.excl_list) else [-1])
        k.extend([ljt, nbp, lj, exc, exl])
        self.nsys = _NbSys(self.n, _p(pos), int(s.n_lj_types), _p(ljt), _p(nbp), _p(lj),
                           _p(exc), _p(exl), _p(ityp), _p(rmax), s.box)
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

    # -- pair / bonded terms ---------------------------------------------------
    def nonbond(self, terms: int = 7) -> np.ndarray:
        f = np.zeros((self.n, 3))
        lib().orc_nonbond(C.byref(self.nsys), int(terms), _p(f))
        return f

    def bonded(self, with_14: bool = True) -> np.ndarray:
        s = self.s
        f = np.zeros((self.n, 3))
        L = lib()
        ba = _i32(s.bond_atoms); bp = _f32(s.bond_params)
        aa = _i32(s.angle_atoms); ap = _f32(s.angle_params)
        da = _i32(s.dih_atoms); dt = _i32(s.dih_types); dp = _f32(s.dih_params)
        sc = _f32(s.scaled14)
        ljt = _i32(s.lj_type); nbp = _i32(s.nb_parm_index); lj = _f32(s.lj_ab)
        if len(ba):
            L.orc_bonds(len(ba), _p(ba), _p(bp), _p(self.pos), C.c_float(s.box), _p(f))
        if len(aa):
            L.orc_angles(len(aa), _p(aa), _p(ap), _p(self.pos), C.c_float(s.box), _p(f))
        if len(da):
            L.orc_dihedrals(len(da), _p(da), _p(dt), _p(dp), _p(sc), _p(ljt), _p(nbp),
                            int(s.n_lj_types), _p(lj), _p(self.pos), C.c_float(s.box),
                            int(with_14), _p(f))
        return f

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


def langevin(x: float):
    out = (C.c_double * 3)()
    lib().orc_langevin(C.c_double(x), out)
    return list(out)
