"""GPU parity at the benchmarked configurations, through the C ABI.

  * 1100 atoms (50 chains of 22, nMC 50, 60 A box) with the launch shapes the
    autotuner picks (as the benchmark runs it): each IS-SPA term, nonbond,
    bonded, the total force of a step and the integrator against the FP64
    oracle on the same Philox points;
  * 16 384 atoms (nMC 100, 1.64 M points), end to end: the oracle computes its
    own FP64 fields at all 1.64 M points, then the IS-SPA, nonbond and bonded
    forces on 64 sampled atoms are compared with the engine's total force;
  * 64 umbrella windows of 44-1100 atoms in one engine with autotuned shapes:
    the smallest, the largest and two other windows against the oracle;
  * the 1100-atom system over 20 steps against the FP64-state oracle stepped
    from the same state with the same Philox streams (positions within 1e-4 A,
    velocities within 1e-3 of the largest).
Measures and tolerances: tests/parity.py (normwise and per atom, 1e-5).
"""
import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from parity import check_force

pytestmark = pytest.mark.gpu

SHAPE_KEYS = ("field_split", "force_chunk", "force_tail_chunk", "force_atoms_per_thread", "field_vote", "force_vote")


def shape_options(shapes):
    return {k: int(shapes[k]) for k in SHAPE_KEYS}


@pytest.fixture(scope="module")
def plain():
    s = ig.synth.config_plain(seed=2)
    eng = ig.Engine(s)
    shapes = eng.autotune()
    eng.close()
    print("autotuned shapes:", shapes)
    o = O.Oracle(s)
    pts = o.mc_points(seed=s.seed, step=0)
    return s, shape_options(shapes), o, pts, o.field(pts)


@pytest.mark.parametrize("terms", [1, 2, 4, 7])
def test_plain_1100_isspa_terms_autotuned(plain, terms):
    s, opts, o, pts, field = plain
    eng = ig.Engine(s, isspa_terms=terms, **opts)
    eng.zero_forces()
    eng.isspa_force()
    check_force(eng.forces(), o.isspa_force(pts, field=field, terms=terms), f"1100 atoms, IS-SPA terms {terms}")
    assert eng.device_status() == 0


def test_plain_1100_nonbond_bonded_autotuned(plain):
    s, opts, o, _, _ = plain
    eng = ig.Engine(s, **opts)
    eng.zero_forces()
    eng.nonbond_force()
    check_force(eng.forces(), o.nonbond(7), "1100 atoms, nonbond")
    eng.zero_forces()
    eng.bond_force()
    eng.angle_force()
    eng.dih_force()
    check_force(eng.forces(), o.bonded(), "1100 atoms, bonded")


def test_plain_1100_full_step_autotuned(plain):
    """Total force of step 0 and the positions and velocities after it, as
    the benchmark's graph step computes them."""
    s, opts, o, pts, field = plain
    eng = ig.Engine(s, **opts)
    f = eng.compute_forces()
    ref = o.bonded() + o.isspa_force(pts, field=field) + o.nonbond(7)
    check_force(f, ref, "1100 atoms, total force of a step")
    eng2 = ig.Engine(s, **opts)
    eng2.step(1)
    po, vo, _ = o.leapfrog(ref, seed=s.seed, step=0)
    pos, vel = eng2.positions(), eng2.velocities()
    assert np.allclose(pos[:, :3], po, rtol=0, atol=2e-5 * s.box)
    check_force(vel[:, :3], vo, "1100 atoms, velocities after one graph step")
    assert eng2.get_step() == 1 and eng2.device_status() == 0


@pytest.mark.slow
def test_precision_16384_end_to_end():
    """The oracle's own FP64 fields at all 1.64 M points (2.7e10 pair terms on
    the host's cores), then the total force on 64 sampled atoms."""
    s = ig.synth.config_precision(seed=3)
    eng = ig.Engine(s)
    f = eng.compute_forces()
    assert eng.device_status() == 0
    o = O.Oracle(s)
    pts = o.mc_points(seed=s.seed, step=0)
    field = o.field(pts)
    atoms = np.sort(np.random.default_rng(0).choice(s.n_atoms, 64, replace=False))
    f_is = o.isspa_force_atoms(pts, field, atoms)
    ref = f_is + o.nonbond_atoms(atoms) + o.bonded()[atoms]
    check_force(f[atoms], ref, "16 384 atoms, total force on 64 sampled atoms (FP64 fields)")
    eng.zero_forces()
    eng.isspa_force()
    check_force(eng.forces()[atoms], f_is, "16 384 atoms, IS-SPA force on 64 sampled atoms (FP64 fields)")


def test_batched_64_windows_autotuned():
    wins = ig.synth.config_batched(n_windows=64, seed=4)
    eng = ig.Engine(wins)
    print("autotuned shapes:", eng.autotune())
    f = eng.compute_forces()
    assert eng.device_status() == 0
    com, _ = eng.us_com()
    sizes = np.array([w.n_atoms for w in wins])
    offs = np.concatenate([[0], np.cumsum(sizes)])
    rng = np.random.default_rng(1)
    pick = {int(np.argmin(sizes)), int(np.argmax(sizes))}
    while len(pick) < 4:
        pick.add(int(rng.integers(len(wins))))
    for w in sorted(pick):
        s = wins[w]
        ref, _, c = O.Oracle(s).total_force(seed=s.seed, step=0, window=w)
        check_force(f[offs[w]:offs[w + 1]], ref, f"64-window batch, window {w} ({s.n_atoms} atoms)")
        assert np.allclose(com[w], c, atol=1e-9)


def test_plain_1100_trajectory_tracks_fp64_oracle():
    """The benchmarked 1100-atom system with the autotuned shapes stepped 20
    times on the GPU and by the FP64-state oracle from the same state with the
    same Philox streams (MC points and Andersen draws): positions and
    velocities agree step by step up to the rounding of the state (each step's
    force error against FP64 is ~5e-7 normwise), so every kernel of the step
    and the update are pinned over a trajectory, not only at step 0."""
    s = ig.synth.config_plain(seed=2)
    eng = ig.Engine(s)
    eng.autotune()
    n = 20
    eng.step(n)
    assert eng.device_status() == 0
    t = s.copy()
    t.pos = np.ascontiguousarray(s.pos, np.float32).copy()
    t.vel = np.ascontiguousarray(s.vel, np.float32).copy()
    o = O.Oracle(t)  # reads o.pos / t.vel in place every call
    for k in range(n):
        f, _, _ = o.total_force(s.seed, k, 0)
        po, vo, _ = o.leapfrog(f, s.seed, k, 0)
        o.pos[:, :3] = po
        t.vel[:, :3] = vo
    L = float(s.box)
    dx = eng.positions()[:, :3].astype(np.float64) - o.pos[:, :3]
    dx -= L * np.round(dx / L)
    dv = eng.velocities()[:, :3].astype(np.float64) - t.vel[:, :3]
    vscale = float(np.abs(t.vel[:, :3]).max())
    print(f"1100 atoms, {n} steps: max |dx| {np.abs(dx).max():.2e} A, max |dv| {np.abs(dv).max():.2e} "
          f"(max |v| {vscale:.3e})")
    assert np.abs(dx).max() < 1e-4
    # (measured: 7.6e-6 A and 1.4e-4 of the largest velocity: a position
    # difference of that size over 20 steps of 0.041 time units comes with
    # velocity differences of this order, grown from the FP32 forces' rounding)
    assert np.abs(dv).max() < 1e-3 * vscale
