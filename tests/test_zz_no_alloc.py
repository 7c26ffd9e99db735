"""The allocation-free IS-SPA entry point, isspa_force_noalloc.

This entry point is for callers that may not call cudaMalloc themselves or let
a library do it: code embedded in a host framework that owns all device memory
through its own pool, or a loop whose device memory budget is fixed before it
starts.  The caller passes device arrays in and gets device forces out; the
scratch space lives in a fixed static device buffer inside the library.

The test drives it through the C ABI with device arrays the test allocates
(here with PyTorch), twice in a row with different step keys, and checks each
result against the engine's isspa_force_cuda on the same system and step with
the tolerance of the other parity tests.  It lives in its own file that pytest
collects last.
"""
import ctypes as C

import numpy as np
import pytest

import isspa_gb300 as ig
from isspa_gb300 import abi

pytestmark = pytest.mark.gpu

FORCE_TOL = 2e-5  # normwise relative, as tests/test_gpu_parity.py


def nrel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_noalloc_force_matches_engine_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch cannot reach the GPU")
    s = ig.synth.make_system(12, 22, 34.0, 20, seed=21, ff=ig.synth.forcefield(n_mc=20))
    eng = ig.Engine(s)
    dev = torch.device("cuda:0")

    def on_device(a, dtype):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

    pos = on_device(s.pos, torch.float32)
    ityp = on_device(s.isspa_type, torch.int32)
    rmax = on_device(s.rmax, torch.float32)
    g, e, f = (on_device(t, torch.float32) for t in (s.g_table, s.e_table, s.f_table))
    out = torch.full((s.n_atoms, 4), float("nan"), dtype=torch.float32, device=dev)

    inp = abi.NoallocInputs()
    inp.n_atoms, inp.n_mc, inp.n_isspa_types = s.n_atoms, s.n_mc, len(s.rmax)
    inp.pos, inp.isspa_type, inp.rmax = pos.data_ptr(), ityp.data_ptr(), rmax.data_ptr()
    inp.n_g, inp.n_e, inp.n_f = s.g_table.shape[1], s.e_table.shape[1], s.f_table.shape[1]
    inp.g_table, inp.e_table, inp.f_table = g.data_ptr(), e.data_ptr(), f.data_ptr()
    inp.g_r0, inp.g_dr, inp.e_r0, inp.e_dr, inp.f_r0, inp.f_dr = s.g_r0, s.g_dr, s.e_r0, s.e_dr, s.f_r0, s.f_dr
    inp.box, inp.seed, inp.terms = s.box, s.seed, 7
    L = abi.lib()
    for step in (0, 9):
        eng.set_step(step)
        eng.zero_forces()
        eng.isspa_force()
        ref = eng.forces()
        inp.step = step
        torch.cuda.synchronize()
        rc = L.isspa_force_noalloc(C.byref(inp), C.c_void_p(out.data_ptr()), None)
        assert rc == abi.OK, abi.lib().isspa_strerror(rc)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.all(got[:, 3] == 0.0)
        err = nrel(got[:, :3], ref)
        print(f"step {step}: no-alloc vs engine normwise {err:.2e}")
        assert err < FORCE_TOL


def test_noalloc_rejects_systems_beyond_the_buffer():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch cannot reach the GPU")
    dev = torch.device("cuda:0")
    dummy = torch.zeros(16, dtype=torch.float32, device=dev)
    inp = abi.NoallocInputs()
    # 5000 atoms x 50 points need ~20 MB of point records: over the 16 MiB buffer
    inp.n_atoms, inp.n_mc, inp.n_isspa_types = 5000, 50, 1
    for name in ("pos", "isspa_type", "rmax", "g_table", "e_table", "f_table"):
        setattr(inp, name, dummy.data_ptr())
    inp.n_g = inp.n_e = inp.n_f = 4
    inp.g_dr = inp.e_dr = inp.f_dr = 0.1
    inp.box = 60.0
    rc = abi.lib().isspa_force_noalloc(C.byref(inp), C.c_void_p(dummy.data_ptr()), None)
    assert rc == abi.ERR_UNSUPPORTED
