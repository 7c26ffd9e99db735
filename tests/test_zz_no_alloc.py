"""The allocation-free IS-SPA entry point, isspa_force_noalloc.

This entry point is for callers that may not call cudaMalloc themselves or let
a library do it: code embedded in a host framework that owns all device memory
through its own pool, or a loop whose device memory budget is fixed before it
starts.  The caller passes device arrays in and gets device forces out; the
scratch space lives in a fixed static device buffer inside the library.

The tests drive it through the C ABI with device arrays the test allocates
(here with PyTorch) and check:
  * two calls in a row (different step keys) against the engine's
    isspa_force_cuda and against the FP64 oracle on the same MC points;
  * a field table on its own radial grid and single force terms against the
    oracle;
  * that repeated calls leave the device's free memory unchanged;
  * a system just under the buffer's limit against the engine, and the
    first size beyond it rejected before anything is enqueued;
  * the status word: a non-finite coordinate, an IS-SPA type outside the
    table and a charge large enough to push the forces beyond the fixed-point
    range are reported through status_out (made on the host, no GPU fault),
    and the next clean call reports 0;
  * argument checks (terms outside 0..7).
It lives in its own file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from isspa_gb300 import abi

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5  # normwise relative, as tests/test_gpu_parity.py


def nrel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="module")
def torch_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch cannot reach the GPU")
    return torch, torch.device("cuda:0")


class Call:
    """isspa_noalloc_inputs for one system, with device copies of its arrays."""

    def __init__(self, torch_dev, s, terms=7):
        torch, dev = torch_dev
        self.torch, self.s = torch, s

        def on_device(a, dtype):
            return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=dev)

        self.pos = on_device(s.pos, torch.float32)
        self.ityp = on_device(s.isspa_type, torch.int32)
        self.rmax = on_device(s.rmax, torch.float32)
        self.tabs = [on_device(t, torch.float32) for t in (s.g_table, s.e_table, s.f_table)]
        self.out = torch.full((s.n_atoms, 4), float("nan"), dtype=torch.float32, device=dev)
        self.status = torch.full((1,), -1, dtype=torch.int32, device=dev)
        inp = abi.NoallocInputs()
        inp.n_atoms, inp.n_mc, inp.n_isspa_types = s.n_atoms, s.n_mc, len(s.rmax)
        inp.pos, inp.isspa_type, inp.rmax = self.pos.data_ptr(), self.ityp.data_ptr(), self.rmax.data_ptr()
        inp.n_g, inp.n_e, inp.n_f = s.g_table.shape[1], s.e_table.shape[1], s.f_table.shape[1]
        inp.g_table, inp.e_table, inp.f_table = (t.data_ptr() for t in self.tabs)
        inp.g_r0, inp.g_dr, inp.e_r0, inp.e_dr, inp.f_r0, inp.f_dr = s.g_r0, s.g_dr, s.e_r0, s.e_dr, s.f_r0, s.f_dr
        inp.box, inp.seed, inp.terms = s.box, s.seed, terms
        inp.status_out = self.status.data_ptr()
        self.inp = inp

    def run(self, step, n_atoms=None):
        """Returns (rc, forces [n][3] or None, status bits or None)."""
        self.inp.step = step
        if n_atoms is not None:
            self.inp.n_atoms = n_atoms
        self.torch.cuda.synchronize()
        rc = abi.lib().isspa_force_noalloc(C.byref(self.inp), C.c_void_p(self.out.data_ptr()), None)
        if rc != abi.OK:
            return rc, None, None
        self.torch.cuda.synchronize()
        got = self.out.cpu().numpy()[:self.inp.n_atoms]
        assert np.all(got[:, 3] == 0.0)
        return rc, got[:, :3].astype(np.float64), int(self.status.cpu().numpy()[0])


def engine_force(s, step, terms=7):
    eng = ig.Engine(s, isspa_terms=terms)
    eng.set_step(step)
    eng.zero_forces()
    eng.isspa_force()
    f = eng.forces()
    eng.close()
    return f


@pytest.fixture(scope="module")
def medium():
    return ig.synth.make_system(12, 22, 34.0, 20, seed=21, ff=ig.synth.forcefield(n_mc=20))


def test_noalloc_force_matches_engine_and_oracle_two_calls(torch_dev, medium):
    s = medium
    call = Call(torch_dev, s)
    o = O.Oracle(s)
    for step in (0, 9):
        rc, got, status = call.run(step)
        assert rc == abi.OK, abi.lib().isspa_strerror(rc)
        assert status == 0
        e_eng = nrel(got, engine_force(s, step))
        e_orc = nrel(got, o.isspa_force(o.mc_points(seed=s.seed, step=step), terms=7))
        print(f"step {step}: no-alloc vs engine {e_eng:.2e}, vs FP64 oracle {e_orc:.2e}")
        assert e_eng < FORCE_TOL
        assert e_orc < FORCE_TOL


@pytest.mark.parametrize("terms", [1, 4])
def test_noalloc_separate_grids_and_terms_against_oracle(torch_dev, medium, terms):
    """A field table on its own radial grid (different r0, dr and length) and a
    single force term, against the oracle on the same Philox points."""
    s = medium.copy()
    s.e_r0 = float(np.float32(s.e_r0 + 0.03))
    s.e_dr = float(np.float32(s.e_dr * 1.1))
    s.e_table = np.ascontiguousarray(s.e_table[:, :-7])
    call = Call(torch_dev, s, terms=terms)
    rc, got, status = call.run(3)
    assert rc == abi.OK and status == 0
    o = O.Oracle(s)
    ref = o.isspa_force(o.mc_points(seed=s.seed, step=3), terms=terms)
    err = nrel(got, ref)
    print(f"terms={terms}, field table on its own grid: vs FP64 oracle {err:.2e}")
    assert err < FORCE_TOL


def test_noalloc_leaves_device_memory_unchanged(torch_dev, medium):
    torch, _ = torch_dev
    call = Call(torch_dev, medium)
    assert call.run(0)[0] == abi.OK  # first call on the device: module and symbol look-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for step in range(1, 6):
        assert call.run(step)[0] == abi.OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_just_under_the_buffer_limit(torch_dev):
    """The largest accepted size is found by descending from a system beyond
    the buffer: every larger size is rejected before anything is enqueued (so
    one atom more than the limit is rejected); a system within one chain of
    the limit then matches the engine."""
    ff = ig.synth.forcefield(n_mc=50)
    big = ig.synth.make_system(200, 22, 95.0, 50, seed=31, ff=ff)  # 4400 atoms: beyond the buffer
    call = Call(torch_dev, big)
    n_max = None
    for n in range(big.n_atoms, 0, -1):
        rc, _, _ = call.run(0, n_atoms=n)
        if rc == abi.OK:
            n_max = n
            break
        assert rc == abi.ERR_UNSUPPORTED
    assert n_max is not None and n_max < big.n_atoms
    print(f"largest system at nMC 50: {n_max} atoms ({n_max * 50} MC points)")
    s = ig.synth.make_system(n_max // 22, 22, 92.0, 50, seed=32, ff=ff)
    assert n_max - 22 < s.n_atoms <= n_max
    call = Call(torch_dev, s)
    for step in (0, 1):
        rc, got, status = call.run(step)
        assert rc == abi.OK and status == 0
        err = nrel(got, engine_force(s, step))
        print(f"{s.n_atoms} atoms, step {step}: no-alloc vs engine {err:.2e}")
        assert err < FORCE_TOL


def test_noalloc_status_word(torch_dev, medium):
    """Failures made on the host: a NaN coordinate (every field and force
    becomes non-finite; positions never become addresses) and an IS-SPA type
    outside the table (read as type 0).  Both come back through status_out;
    the next clean call reports 0."""
    s = medium.copy()
    s.pos = s.pos.copy()
    s.pos[7, 0] = np.nan
    rc, got, status = Call(torch_dev, s).run(0)
    assert rc == abi.OK
    assert status & abi.NOALLOC_STATUS_NONFINITE
    t = medium.copy()
    t.isspa_type = t.isspa_type.copy()
    t.isspa_type[3] = 99
    rc, got, status = Call(torch_dev, t).run(0)
    assert rc == abi.OK
    assert status == abi.NOALLOC_STATUS_BOUNDS
    assert np.all(np.isfinite(got))
    # a charge of 1e15 (the IS-SPA pass has no pair singularity to collapse:
    # MC points never coincide with atoms): forces far beyond the fixed-point
    # range are reported as overflow (or non-finite), and the call still
    # returns ISSPA_OK with the status word set
    u = medium.copy()
    u.pos = u.pos.copy()
    u.pos[5, 3] = 1.0e15
    rc, got, status = Call(torch_dev, u).run(0)
    assert rc == abi.OK
    assert status & (abi.NOALLOC_STATUS_OVERFLOW | abi.NOALLOC_STATUS_NONFINITE)
    rc, got, status = Call(torch_dev, medium).run(0)
    assert rc == abi.OK and status == 0


def test_noalloc_rejects_bad_arguments(torch_dev):
    torch, dev = torch_dev
    dummy = torch.zeros(16, dtype=torch.float32, device=dev)
    inp = abi.NoallocInputs()
    inp.n_atoms, inp.n_mc, inp.n_isspa_types = 10, 5, 1
    for name in ("pos", "isspa_type", "rmax", "g_table", "e_table", "f_table"):
        setattr(inp, name, dummy.data_ptr())
    inp.n_g = inp.n_e = inp.n_f = 4
    inp.g_dr = inp.e_dr = inp.f_dr = 0.1
    inp.box = 60.0
    for terms in (-1, 8):
        inp.terms = terms
        assert abi.lib().isspa_force_noalloc(C.byref(inp), C.c_void_p(dummy.data_ptr()), None) == abi.ERR_ARG
    # 5000 atoms x 50 points need ~20 MB of point records: over the 16 MiB buffer
    inp.terms = 7
    inp.n_atoms, inp.n_mc = 5000, 50
    rc = abi.lib().isspa_force_noalloc(C.byref(inp), C.c_void_p(dummy.data_ptr()), None)
    assert rc == abi.ERR_UNSUPPORTED
