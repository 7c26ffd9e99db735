"""Host-side description of one simulation window as numpy arrays.

Field names and layouts follow ``isspa_system_desc`` (include/isspa_gb300.h),
which in turn follows the reference's atom/bond/angle/dih/isspa/us objects.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import abi

PI_F = np.float32(3.1415926535)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape is not None else a


def _i32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a.reshape(shape) if shape is not None else a


@dataclass
class System:
    pos: np.ndarray                    # [N,4] x y z q/sqrt(eps)
    vel: np.ndarray                    # [N,4] vx vy vz mass(H->12)
    raw_mass: np.ndarray               # [N]
    n_lj_types: int
    lj_type: np.ndarray                # [N]
    nb_parm_index: np.ndarray          # [nt*nt]
    lj_ab: np.ndarray                  # [nt(nt+1)/2, 2]
    n_excl_cum: np.ndarray             # [N]
    excl_list: np.ndarray              # [L]
    bond_atoms: np.ndarray             # [nb,3]
    bond_params: np.ndarray            # [nbt,2]
    angle_atoms: np.ndarray            # [na,4]
    angle_params: np.ndarray           # [nat,2]
    dih_atoms: np.ndarray              # [nd,4]
    dih_types: np.ndarray              # [nd]
    dih_params: np.ndarray             # [ndt,4]
    scaled14: np.ndarray               # [ndt,2]
    isspa_type: np.ndarray             # [N]
    rmax: np.ndarray                   # [nit]
    g_table: np.ndarray                # [nit, nG]
    e_table: np.ndarray                # [nit, nE]
    f_table: np.ndarray                # [nit, nF]
    g_r0: float
    g_dr: float
    e_r0: float
    e_dr: float
    f_r0: float
    f_dr: float
    n_mc: int
    box: float
    kT: float
    dt: float
    pnu: float
    seed: int
    us_on: int = 0
    bias_list: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    us_k: float = 0.0
    us_x0: float = 0.0
    omp: object = None                 # parameters of the reference's OpenMP model (synthetic systems)

    @property
    def n_atoms(self) -> int:
        return int(self.pos.shape[0])

    @property
    def n_points(self) -> int:
        return self.n_atoms * int(self.n_mc)

    def vtot(self) -> np.ndarray:
        """Monte Carlo normalisation per IS-SPA type (isspa_class.cpp:41)."""
        r = self.rmax.astype(np.float64)
        return (4.0 / 3.0 * float(PI_F) * r * r * r * 0.0074 / float(np.float32(self.n_mc))).astype(np.float32)

    def bias_mass_fraction(self) -> np.ndarray:
        """m_i / M_group in float, as us::populate_mass (us_class.cpp:136-152)."""
        bl = self.bias_list.reshape(-1, 2)
        m = self.raw_mass[bl[:, 0]].astype(np.float32)
        tot = [np.float32(0), np.float32(0)]
        for mi, g in zip(m, bl[:, 1]):
            tot[g] = np.float32(tot[g] + mi)
        return np.array([np.float32(mi / tot[g]) for mi, g in zip(m, bl[:, 1])], np.float32)

    def copy(self) -> "System":
        kw = {}
        for k, v in self.__dict__.items():
            kw[k] = v.copy() if isinstance(v, np.ndarray) else v
        return System(**kw)

    # ------------------------------------------------------------------ ABI
    def to_desc(self):
        """ctypes description pointing at this object's arrays (keep `self` alive)."""
        keep = []

        def p(a, conv):
            a = conv(a)
            keep.append(a)
            return a.ctypes.data_as(C.c_void_p)

        d = abi.SystemDesc()
        d.n_atoms = self.n_atoms
        d.pos = p(self.pos, _f32)
        d.vel = p(self.vel, _f32)
        d.raw_mass = p(self.raw_mass, _f32)
        d.n_lj_types = int(self.n_lj_types)
        d.lj_type = p(self.lj_type, _i32)
        d.nb_parm_index = p(self.nb_parm_index, _i32)
        d.lj_ab = p(self.lj_ab, _f32)
        d.excl_len = int(len(self.excl_list))
        d.n_excl_cum = p(self.n_excl_cum, _i32)
        d.excl_list = p(self.excl_list if len(self.excl_list) else np.zeros(1, np.int32), _i32)
        d.n_bonds = int(len(self.bond_atoms))
        d.bond_atoms = p(self.bond_atoms if len(self.bond_atoms) else np.zeros((1, 3)), _i32)
        d.n_bond_types = int(len(self.bond_params))
        d.bond_params = p(self.bond_params if len(self.bond_params) else np.zeros((1, 2)), _f32)
        d.n_angles = int(len(self.angle_atoms))
        d.angle_atoms = p(self.angle_atoms if len(self.angle_atoms) else np.zeros((1, 4)), _i32)
        d.n_angle_types = int(len(self.angle_params))
        d.angle_params = p(self.angle_params if len(self.angle_params) else np.zeros((1, 2)), _f32)
        d.n_dihs = int(len(self.dih_atoms))
        d.dih_atoms = p(self.dih_atoms if len(self.dih_atoms) else np.zeros((1, 4)), _i32)
        d.dih_types = p(self.dih_types if len(self.dih_types) else np.zeros(1), _i32)
        d.n_dih_types = int(len(self.dih_params))
        d.dih_params = p(self.dih_params if len(self.dih_params) else np.zeros((1, 4)), _f32)
        d.scaled14 = p(self.scaled14 if len(self.scaled14) else np.ones((1, 2)), _f32)
        d.isspa_type = p(self.isspa_type, _i32)
        d.n_isspa_types = int(len(self.rmax))
        d.rmax = p(self.rmax, _f32)
        d.n_g, d.n_e, d.n_f = (int(self.g_table.shape[1]), int(self.e_table.shape[1]),
                               int(self.f_table.shape[1]))
        d.g_table = p(self.g_table, _f32)
        d.e_table = p(self.e_table, _f32)
        d.f_table = p(self.f_table, _f32)
        d.g_r0, d.g_dr, d.e_r0, d.e_dr, d.f_r0, d.f_dr = (self.g_r0, self.g_dr, self.e_r0, self.e_dr,
                                                          self.f_r0, self.f_dr)
        d.us_on = int(self.us_on)
        d.n_bias = int(len(self.bias_list)) if self.us_on else 0
        d.bias_list = p(self.bias_list if len(self.bias_list) else np.zeros((1, 2)), _i32)
        d.us_k, d.us_x0 = float(self.us_k), float(self.us_x0)
        d.n_mc = int(self.n_mc)
        d.box, d.kT, d.dt, d.pnu = float(self.box), float(self.kT), float(self.dt), float(self.pnu)
        d.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        return d, keep

    @staticmethod
    def from_desc(d: abi.SystemDesc) -> "System":
        n = d.n_atoms

        def arr(ptr, count, ctype, dtype, shape):
            if count <= 0 or not ptr:
                return np.zeros(shape if count > 0 else (0,) + tuple(shape[1:]), dtype)
            buf = (ctype * count).from_address(ptr)
            return np.ctypeslib.as_array(buf).astype(dtype).reshape(shape)

        F, I = C.c_float, C.c_int
        nt = d.n_lj_types
        nit = d.n_isspa_types
        return System(
            pos=arr(d.pos, 4 * n, F, np.float32, (n, 4)),
            vel=arr(d.vel, 4 * n, F, np.float32, (n, 4)),
            raw_mass=arr(d.raw_mass, n, F, np.float32, (n,)),
            n_lj_types=nt,
            lj_type=arr(d.lj_type, n, I, np.int32, (n,)),
            nb_parm_index=arr(d.nb_parm_index, nt * nt, I, np.int32, (nt * nt,)),
            lj_ab=arr(d.lj_ab, nt * (nt + 1), F, np.float32, (nt * (nt + 1) // 2, 2)),
            n_excl_cum=arr(d.n_excl_cum, n, I, np.int32, (n,)),
            excl_list=arr(d.excl_list, d.excl_len, I, np.int32, (d.excl_len,)),
            bond_atoms=arr(d.bond_atoms, 3 * d.n_bonds, I, np.int32, (d.n_bonds, 3)),
            bond_params=arr(d.bond_params, 2 * d.n_bond_types, F, np.float32, (d.n_bond_types, 2)),
            angle_atoms=arr(d.angle_atoms, 4 * d.n_angles, I, np.int32, (d.n_angles, 4)),
            angle_params=arr(d.angle_params, 2 * d.n_angle_types, F, np.float32, (d.n_angle_types, 2)),
            dih_atoms=arr(d.dih_atoms, 4 * d.n_dihs, I, np.int32, (d.n_dihs, 4)),
            dih_types=arr(d.dih_types, d.n_dihs, I, np.int32, (d.n_dihs,)),
            dih_params=arr(d.dih_params, 4 * d.n_dih_types, F, np.float32, (d.n_dih_types, 4)),
            scaled14=arr(d.scaled14, 2 * d.n_dih_types, F, np.float32, (d.n_dih_types, 2)),
            isspa_type=arr(d.isspa_type, n, I, np.int32, (n,)),
            rmax=arr(d.rmax, nit, F, np.float32, (nit,)),
            g_table=arr(d.g_table, nit * d.n_g, F, np.float32, (nit, d.n_g)),
            e_table=arr(d.e_table, nit * d.n_e, F, np.float32, (nit, d.n_e)),
            f_table=arr(d.f_table, nit * d.n_f, F, np.float32, (nit, d.n_f)),
            g_r0=d.g_r0, g_dr=d.g_dr, e_r0=d.e_r0, e_dr=d.e_dr, f_r0=d.f_r0, f_dr=d.f_dr,
            n_mc=d.n_mc, box=d.box, kT=d.kT, dt=d.dt, pnu=d.pnu, seed=d.seed,
            us_on=d.us_on,
            bias_list=arr(d.bias_list, 2 * d.n_bias, I, np.int32, (d.n_bias, 2)),
            us_k=d.us_k, us_x0=d.us_x0,
        )

    def write_isspatop(self, path: str, title: str = "") -> None:
        """Write this system's IS-SPA types, rmax and tables as an .isspatop file
        (the inverse of the reader used by from_config)."""
        d, keep = self.to_desc()
        abi.check(abi.lib().isspa_write_isspatop(C.byref(d), path.encode(), title.encode()), path)

    @staticmethod
    def from_config(path: str) -> "System":
        """Read a reference config file and everything it names (total_force_cuda.cpp:57-99)."""
        L = abi.lib()
        cfg = abi.RunConfig()
        abi.check(L.isspa_read_run_config(path.encode(), C.byref(cfg)), path)
        h = C.c_void_p()
        base = os.path.dirname(os.path.abspath(path)).encode()
        abi.check(L.isspa_system_load(C.byref(cfg), base, C.byref(h)), path)
        try:
            d = abi.SystemDesc()
            abi.check(L.isspa_system_describe(h, C.byref(d)))
            return System.from_desc(d)
        finally:
            L.isspa_system_free(h)


def read_run_config(path: str) -> abi.RunConfig:
    cfg = abi.RunConfig()
    abi.check(abi.lib().isspa_read_run_config(path.encode(), C.byref(cfg)), path)
    return cfg
