"""The fused field + force launch (isspa_engine_options.isspa_fused = 1), through
the C ABI.

Each block of the fused launch computes one field tile's points (the field
kernel's code) and then those points' forces on every atom of the window (the
force kernel's per-pair code), so its forces equal the separate passes' up to
FP32 summation order (sums over a tile's points instead of a force work
item's).

* IS-SPA forces of every term mask that keeps the tabulated LJ term, against
  the FP64 oracle (tests/parity.py measures), at field splits 4, 8 and 16,
  with and without the voted atom loop: ADI2 at nMC 100 and a 264-atom
  window; three uneven batched windows against the separate passes (IS-SPA
  term) and the oracle (total force).
* The full step's forces against the oracle, and trajectories against the
  separate passes' (FP32 summation order only: within 1e-5 A after 12 steps).
* Determinism: graph replays, direct stream launches, programmatic launches
  and isspa_step_host give one trajectory bit for bit.
* The engine falls back to the separate passes where the fused launch does
  not apply (tabulated LJ term off, injected points, split 1 or 2), and
  rejects an out-of-range option.
"""
import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from parity import check_force, nrel

pytestmark = pytest.mark.gpu


def with_mc(s, n_mc):
    s = s.copy()
    s.n_mc = n_mc
    return s


@pytest.fixture(scope="module")
def medium():
    return ig.synth.make_system(12, 22, 34.0, 20, seed=21, ff=ig.synth.forcefield(n_mc=20))


def _fused_isspa(windows, **opts):
    opts.setdefault("field_split", 8)
    eng = ig.Engine(windows, isspa_fused=1, **opts)
    assert eng.shapes()["isspa_fused"] == 1
    eng.zero_forces()
    eng.isspa_force()
    f = eng.forces()
    assert eng.device_status() == 0
    eng.close()
    return f


@pytest.mark.parametrize("terms", [2, 3, 6, 7])
@pytest.mark.parametrize("which", ["adi2", "medium"])
def test_fused_isspa_terms_match_oracle(terms, which, adi2, medium):
    s = with_mc(adi2, 100) if which == "adi2" else medium
    f = _fused_isspa(s, isspa_terms=terms)
    o = O.Oracle(s)
    ref = o.isspa_force(o.mc_points(seed=s.seed, step=0), terms=terms)
    check_force(f, ref, f"fused isspa terms={terms} {which}")


@pytest.mark.parametrize("split", [4, 8, 16])
@pytest.mark.parametrize("vote", [0, 1])
def test_fused_splits_and_votes_match_oracle(split, vote, medium):
    f = _fused_isspa(medium, field_split=split, field_vote=vote)
    o = O.Oracle(medium)
    ref = o.isspa_force(o.mc_points(seed=medium.seed, step=0))
    check_force(f, ref, f"fused split {split} vote {vote}")


def test_fused_batched_windows_match_oracle():
    # The IS-SPA term alone of the 1078-atom window differs from the oracle by
    # 4.9e-5 per atom in the separate passes too (7e-6 normwise); the total
    # force, the quantity the step uses, is compared with the oracle as in
    # test_gpu_parity.py, and the IS-SPA term with the separate passes.
    wins = ig.synth.config_batched(n_windows=3, seed=9)
    f = _fused_isspa(wins, field_split=8)
    sep = ig.Engine(wins, isspa_fused=2, field_split=8)
    sep.zero_forces()
    sep.isspa_force()
    f_sep = sep.forces()
    sep.close()
    fused = ig.Engine(wins, isspa_fused=1, field_split=8)
    tot = fused.compute_forces()
    fused.close()
    off = 0
    for k, s in enumerate(wins):
        n = s.n_atoms
        d = nrel(f[off:off + n], f_sep[off:off + n])
        print(f"fused against separate passes, window {k} ({n} atoms): normwise {d:.2e}")
        assert d < 1e-6
        ref, _, _ = O.Oracle(s).total_force(seed=s.seed, step=0, window=k)
        check_force(tot[off:off + n], ref, f"fused batched window {k} ({n} atoms), total force")
        off += n


def test_fused_full_step_forces_and_trajectory():
    s = ig.synth.config_small(seed=3)
    eng = ig.Engine(s, isspa_fused=1, field_split=16)
    f = eng.compute_forces()
    ref, _, _ = O.Oracle(s).total_force(seed=s.seed, step=0)
    check_force(f, ref, "fused total force, 44 atoms")
    eng.close()
    out = {}
    for fused in (1, 2):
        e = ig.Engine(s, isspa_fused=fused, field_split=16)
        e.step(12)
        out[fused] = (e.positions(), e.velocities(), e.device_status())
        e.close()
    assert out[1][2] == 0 and out[2][2] == 0
    dx = np.abs(out[1][0][:, :3] - out[2][0][:, :3]).max()
    print(f"fused against separate passes, 44 atoms, 12 steps: max |dx| {dx:.2e} A")
    assert dx < 1e-5


@pytest.mark.parametrize("integ", [1, 2])
def test_fused_launch_paths_bit_identical(integ, adi2):
    s = with_mc(adi2, 100)
    runs = {}
    for pdl in (2, 1):
        for graph in (True, False):
            eng = ig.Engine(s, isspa_fused=1, field_split=16, integrator=integ, step_pdl=pdl, use_graph=graph)
            eng.step(10)
            runs[(pdl, graph)] = (eng.positions(), eng.velocities(), eng.get_step(), eng.device_status())
            eng.close()
    eng = ig.Engine(s, isspa_fused=1, field_split=16, integrator=integ, step_pdl=1)
    n = eng.n_atoms
    bufs = [ig.host_array((n, 4)) for _ in range(5)]
    bufs[0][:] = eng.positions()
    bufs[1][:] = eng.velocities()
    for k in range(10):
        src, dst = (0, 2) if k % 2 == 0 else (2, 0)
        eng.step_host(bufs[src], bufs[src + 1], bufs[dst], bufs[dst + 1], bufs[4])
    runs["host"] = (bufs[0].copy(), bufs[1].copy(), eng.get_step(), eng.device_status())
    eng.close()
    p0, v0, _, _ = runs[(2, True)]
    for key, (p, v, st, ds) in runs.items():
        assert ds == 0 and st == 10, key
        assert np.array_equal(p, p0), key
        assert np.array_equal(v, v0), key


def test_fused_falls_back_where_it_does_not_apply(medium):
    for opts in (dict(isspa_terms=5, field_split=8), dict(field_split=1), dict(field_split=2)):
        eng = ig.Engine(medium, isspa_fused=1, **opts)
        assert eng.shapes()["isspa_fused"] == 0, opts
        eng.close()
    eng = ig.Engine(medium, isspa_fused=1, field_split=8)
    assert eng.shapes()["isspa_fused"] == 1
    o = O.Oracle(medium)
    pts = o.mc_points(seed=medium.seed, step=0)
    eng.set_mc_points(pts)
    assert eng.shapes()["isspa_fused"] == 0  # injected points: the separate passes
    eng.zero_forces()
    eng.isspa_force()
    check_force(eng.forces(), o.isspa_force(pts), "injected points with isspa_fused set")
    eng.close()
    # asked for where it cannot apply (tabulated LJ term off): the autotuner
    # times the separate passes only
    eng = ig.Engine(medium, isspa_fused=1, isspa_terms=5)
    sh = eng.autotune()
    assert sh["isspa_fused"] == 0
    eng.step(3)
    assert eng.device_status() == 0
    eng.close()
    for bad in (-1, 3):
        with pytest.raises(RuntimeError):
            ig.Engine(medium, isspa_fused=bad)
