"""ctypes binding of libisspa_gb300.so (declarations mirror include/isspa_gb300.h).

The library must have been built (``build.py``); importing this module without
it raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libisspa_gb300.so")

OK = 0
ERR_ARG, ERR_IO, ERR_PARSE, ERR_CUDA, ERR_NOMEM = -1, -2, -3, -4, -5
ERR_BOUNDS, ERR_TIMEOUT, ERR_NONFINITE, ERR_UNSUPPORTED, ERR_STATE, ERR_OVERFLOW = -6, -7, -8, -9, -10, -11
ERR_LIST_FULL = -12


class IsspaError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().isspa_strerror(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


class SystemDesc(C.Structure):
    _fields_ = [
        ("n_atoms", C.c_int), ("pos", C.c_void_p), ("vel", C.c_void_p), ("raw_mass", C.c_void_p),
        ("n_lj_types", C.c_int), ("lj_type", C.c_void_p), ("nb_parm_index", C.c_void_p),
        ("lj_ab", C.c_void_p),
        ("excl_len", C.c_int), ("n_excl_cum", C.c_void_p), ("excl_list", C.c_void_p),
        ("n_bonds", C.c_int), ("bond_atoms", C.c_void_p), ("n_bond_types", C.c_int),
        ("bond_params", C.c_void_p),
        ("n_angles", C.c_int), ("angle_atoms", C.c_void_p), ("n_angle_types", C.c_int),
        ("angle_params", C.c_void_p),
        ("n_dihs", C.c_int), ("dih_atoms", C.c_void_p), ("dih_types", C.c_void_p),
        ("n_dih_types", C.c_int), ("dih_params", C.c_void_p), ("scaled14", C.c_void_p),
        ("isspa_type", C.c_void_p), ("n_isspa_types", C.c_int), ("rmax", C.c_void_p),
        ("n_g", C.c_int), ("n_e", C.c_int), ("n_f", C.c_int),
        ("g_table", C.c_void_p), ("e_table", C.c_void_p), ("f_table", C.c_void_p),
        ("g_r0", C.c_float), ("g_dr", C.c_float), ("e_r0", C.c_float), ("e_dr", C.c_float),
        ("f_r0", C.c_float), ("f_dr", C.c_float),
        ("us_on", C.c_int), ("n_bias", C.c_int), ("bias_list", C.c_void_p),
        ("us_k", C.c_float), ("us_x0", C.c_float),
        ("n_mc", C.c_int), ("box", C.c_float), ("kT", C.c_float), ("dt", C.c_float),
        ("pnu", C.c_float), ("seed", C.c_uint64),
    ]


class EngineOptions(C.Structure):
    _fields_ = [("isspa_terms", C.c_int), ("nonbond_terms", C.c_int), ("use_graph", C.c_int),
                ("field_split", C.c_int), ("force_chunk", C.c_int), ("mem_cap", C.c_size_t),
                ("force_atoms_per_thread", C.c_int), ("force_tail_chunk", C.c_int),
                ("field_vote", C.c_int), ("force_vote", C.c_int), ("integrator", C.c_int),
                ("nonbond_chunk", C.c_int), ("field_tma", C.c_int), ("nonbond_cutoff", C.c_float),
                ("nonbond_skin", C.c_float), ("nonbond_list_max", C.c_int), ("step_pdl", C.c_int),
                ("isspa_fused", C.c_int), ("force_overlap", C.c_int)]


class RunConfig(C.Structure):
    _fields_ = [(n, C.c_char * 512) for n in ("prmtop", "isspa_prmtop", "input_coord", "input_vel", "us_cfg",
                                                "for_out", "pos_out", "vel_out", "pos_rst_file",
                                                "vel_rst_file")] + \
               [(n, C.c_int) for n in ("n_mc", "n_steps", "delta_write", "seed", "us", "vel_rst",
                                       "pnu_set")] + \
               [(n, C.c_float) for n in ("temperature", "kT", "dt", "dt_ps", "pnu", "box", "eps",
                                         "cutoff")]


class NoallocInputs(C.Structure):
    """isspa_noalloc_inputs: device pointers owned by a caller that cannot allocate."""
    _fields_ = [("n_atoms", C.c_int), ("n_mc", C.c_int), ("n_isspa_types", C.c_int),
                ("pos", C.c_void_p), ("isspa_type", C.c_void_p), ("rmax", C.c_void_p),
                ("n_g", C.c_int), ("n_e", C.c_int), ("n_f", C.c_int),
                ("g_table", C.c_void_p), ("e_table", C.c_void_p), ("f_table", C.c_void_p),
                ("g_r0", C.c_float), ("g_dr", C.c_float), ("e_r0", C.c_float), ("e_dr", C.c_float),
                ("f_r0", C.c_float), ("f_dr", C.c_float), ("box", C.c_float),
                ("seed", C.c_uint64), ("step", C.c_uint32), ("terms", C.c_int), ("status_out", C.c_void_p)]


NOALLOC_SCRATCH_BYTES = 16 << 20
# ISSPA_NOALLOC_STATUS_* bits written to isspa_noalloc_inputs.status_out
NOALLOC_STATUS_OVERFLOW, NOALLOC_STATUS_NONFINITE, NOALLOC_STATUS_BOUNDS = 1, 2, 4
SHAPE_COUNT = 18  # ISSPA_SHAPE_COUNT
TERMS_NONE = -1  # ISSPA_TERMS_NONE: switches the IS-SPA or nonbond pass off

# isspa_energies components (the ISSPA_E_* enum), kcal/mol
ENERGY_NAMES = ("kin_before", "kin_after", "bond", "angle", "dihedral", "lj14", "coul14", "lj", "coul",
                "corr", "umbrella", "virial")

# (name, restype, argtypes); every exported entry point of include/isspa_gb300.h
_P = C.c_void_p
_FP = C.POINTER(C.c_float)
SIGNATURES = [
    ("isspa_strerror", C.c_char_p, [C.c_int]),
    ("isspa_default_options", None, [C.POINTER(EngineOptions)]),
    ("isspa_device_count", C.c_int, [C.POINTER(C.c_int)]),
    ("isspa_read_run_config", C.c_int, [C.c_char_p, C.POINTER(RunConfig)]),
    ("isspa_system_load", C.c_int, [C.POINTER(RunConfig), C.c_char_p, C.POINTER(_P)]),
    ("isspa_read_prmtop", C.c_int, [C.c_char_p, C.c_float, C.POINTER(_P)]),
    ("isspa_read_isspatop", C.c_int, [_P, C.c_char_p]),
    ("isspa_write_isspatop", C.c_int, [_P, C.c_char_p, C.c_char_p]),
    ("isspa_read_rst7", C.c_int, [_P, C.c_char_p, C.c_int]),
    ("isspa_read_us_config", C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_size_t]),
    ("isspa_system_describe", C.c_int, [_P, C.POINTER(SystemDesc)]),
    ("isspa_system_set_run", C.c_int, [_P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_uint64]),
    ("isspa_system_free", None, [_P]),
    ("isspa_engine_create", C.c_int, [C.POINTER(SystemDesc), C.c_int, C.POINTER(EngineOptions), C.POINTER(_P)]),
    ("isspa_engine_destroy", None, [_P]),
    ("isspa_engine_info", C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    ("isspa_engine_shapes", C.c_int, [_P, C.POINTER(C.c_int)]),
    ("isspa_autotune", C.c_int, [_P, C.c_int, C.POINTER(C.c_int)]),
    ("isspa_zero_forces", C.c_int, [_P]),
    ("bond_force_cuda", C.c_int, [_P, _FP]),
    ("angle_force_cuda", C.c_int, [_P, _FP]),
    ("dih_force_cuda", C.c_int, [_P, _FP]),
    ("isspa_force_cuda", C.c_int, [_P, _FP]),
    ("nonbond_force_cuda", C.c_int, [_P, _FP]),
    ("us_force_cuda", C.c_int, [_P, _FP]),
    ("leapfrog_cuda", C.c_int, [_P, _FP]),
    ("isspa_step", C.c_int, [_P, C.c_int]),
    ("isspa_time_steps", C.c_int, [_P, C.c_int, C.c_size_t, C.POINTER(C.c_double)]),
    ("isspa_time_steps_detailed", C.c_int, [_P, C.c_int, C.c_size_t, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    ("isspa_host_alloc", C.c_int, [C.c_size_t, C.POINTER(_P)]),
    ("isspa_host_free", None, [_P]),
    ("isspa_synchronize", C.c_int, [_P]),
    ("isspa_device_status", C.c_int, [_P, C.c_int]),
    ("isspa_nonbond_list_stats", C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("isspa_debug_stall_barrier", C.c_int, [_P]),
    ("isspa_set_positions", C.c_int, [_P, _P, C.c_int]),
    ("isspa_get_positions", C.c_int, [_P, _P, C.c_int]),
    ("isspa_set_velocities", C.c_int, [_P, _P, C.c_int]),
    ("isspa_get_velocities", C.c_int, [_P, _P, C.c_int]),
    ("isspa_get_forces", C.c_int, [_P, _P, C.c_int]),
    ("isspa_set_step", C.c_int, [_P, C.c_uint32]),
    ("isspa_get_step", C.c_int, [_P, C.POINTER(C.c_uint32)]),
    ("isspa_get_us_com", C.c_int, [_P, _P, _P]),
    ("isspa_step_host", C.c_int, [_P, _P, _P, _P, _P, _P]),
    ("isspa_set_mc_points", C.c_int, [_P, _P, C.c_longlong]),
    ("isspa_clear_mc_points", C.c_int, [_P]),
    ("isspa_get_point_fields", C.c_int, [_P, _P, _P, _P, _P, _P, C.c_longlong]),
    ("isspa_set_tables", C.c_int, [_P, _P, _P, _P, _P]),
    ("isspa_adjoint_mean_force", C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, _P, _P]),
    ("isspa_energies", C.c_int, [_P, _P]),
    ("isspa_neighbor_list", C.c_int, [_P, C.c_float, C.c_int, _P, _P]),
    ("isspa_cell_list", C.c_int, [_P, C.c_float, _P, _P]),
    ("isspa_measure_fp32_peak", C.c_int, [C.POINTER(C.c_double)]),
    ("isspa_force_noalloc", C.c_int, [C.POINTER(NoallocInputs), _P, _P]),
]

_lib = None


def lib():
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA engine first (build.py)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise IsspaError(status, what)


def device_count() -> int:
    n = C.c_int(0)
    lib().isspa_device_count(C.byref(n))
    return n.value
