"""Bonded terms (FP32) and the fused integrator, through the C ABI.

* Near-planar torsions: chains laid out as planar zig-zags (bonds 1.4-1.6
  A, angles 100-120 deg, trans with some cis torsions) lifted out of the
  plane by noise of 1e-2 to 1e-4 A, so every torsion angle lies within ~1e-2
  to 1e-4 rad of 0 or pi, where the reference's acos / (1/sin phi) form
  loses its precision in FP32.  Each bonded term is compared per atom with
  the FP64 oracle (tests/parity.py measures, 1e-5).
* Bonds and angles at their minimum (stretch and bend forces that are small
  differences): absolute error within 1e-5 of the largest force.
* The fused integrator (bonded, umbrella and leapfrog in one cooperative
  kernel) gives the separate kernels' trajectory bit for bit: a plain
  system, a restrained batch of windows, and the reference's ADI2 inputs
  with its umbrella restraint.
* The single-kernel step (field, nonbond, bonded | force | update in one
  cooperative kernel) gives the separate kernels' trajectory bit for bit with
  the same launch shapes, on the same three systems.
* The step chain (field, force, leapfrog) launched as programmatic
  dependents gives the ordinary launches' trajectory bit for bit, with
  either integrator, through graph replays, direct stream launches and
  isspa_step_host with device-mapped buffers.
* The autotuner's integrator choice leaves the state where it was.
* The grid barrier's bounded wait: a barrier left mid-count runs out,
  the step reports ISSPA_ERR_TIMEOUT without a fault, and the same engine
  steps on cleanly after the status is reset.
"""
import math

import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from isspa_gb300 import abi
from parity import check_force

pytestmark = pytest.mark.gpu


def planar_chain(n, rng, origin):
    """A zig-zag of n atoms in the plane z = origin[2]: bonds 1.4-1.6 A and
    angles 100-120 deg (off the 1.5 A / 110 deg minimum, so stretch and bend
    forces are not vanishingly small); mostly alternating turns (trans), a
    same-direction turn (cis) now and then but never twice in a row."""
    x = np.zeros((n, 3))
    x[0] = origin
    ang = rng.uniform(0, 2 * math.pi)
    x[1] = x[0] + rng.uniform(1.4, 1.6) * np.array([math.cos(ang), math.sin(ang), 0.0])
    turn, last_cis = 1.0, True
    for i in range(2, n):
        cis = (not last_cis) and rng.random() < 0.2
        if not cis:
            turn = -turn
        last_cis = cis
        ang += turn * (math.pi - math.radians(rng.uniform(100.0, 120.0)))
        x[i] = x[i - 1] + rng.uniform(1.4, 1.6) * np.array([math.cos(ang), math.sin(ang), 0.0])
    return x


def equilibrium_chain(n, rng, origin, bond, theta):
    """A planar zig-zag exactly at the bond and angle minimum (stretch and
    bend forces that are differences of nearly equal numbers)."""
    x = np.zeros((n, 3))
    x[0] = origin
    ang = rng.uniform(0, 2 * math.pi)
    x[1] = x[0] + bond * np.array([math.cos(ang), math.sin(ang), 0.0])
    for i in range(2, n):
        ang += (-1) ** i * (math.pi - theta)
        x[i] = x[i - 1] + bond * np.array([math.cos(ang), math.sin(ang), 0.0])
    return x


@pytest.fixture(scope="module")
def flat_systems():
    out = {}
    base = ig.synth.make_system(2, 22, 60.0, 20, seed=12, ff=ig.synth.forcefield(n_mc=20))
    for noise in (1e-2, 1e-3, 1e-4):
        rng = np.random.default_rng(7)
        s = base.copy()
        pos = s.pos.copy()
        pos[:22, :3] = planar_chain(22, rng, np.array([20.0, 20.0, 15.0]))
        pos[22:, :3] = planar_chain(22, rng, np.array([20.0, 20.0, 40.0]))
        pos[:, 2] += rng.uniform(-noise, noise, len(pos))
        s.pos = pos.astype(np.float32)
        out[noise] = s
    return out


@pytest.mark.parametrize("noise", [1e-2, 1e-3, 1e-4])
def test_near_planar_torsions_match_fp64_oracle(flat_systems, noise):
    s = flat_systems[noise]
    o = O.Oracle(s)
    eng = ig.Engine(s)
    for name, call, ref in [("dihedrals + 1-4", eng.dih_force, o.bonded(bonds=False, angles=False)),
                            ("angles", eng.angle_force, o.bonded(bonds=False, dihedrals=False)),
                            ("bonds", eng.bond_force, o.bonded(angles=False, dihedrals=False))]:
        eng.zero_forces()
        call()
        check_force(eng.forces(), ref, f"near-planar chains (z noise {noise:g} A), {name}")
    eng.zero_forces()
    eng.bond_force()
    eng.angle_force()
    eng.dih_force()
    check_force(eng.forces(), o.bonded(), f"near-planar chains (z noise {noise:g} A), all bonded")
    assert eng.device_status() == 0


def test_near_minimum_stretch_and_bend_match_fp64_oracle():
    """Bonds within ~1e-6 A of r0 and angles within ~1e-6 rad of theta0: the
    stretch and bend forces are tiny differences, carried in double-float
    FP32; their absolute error against the FP64 oracle stays at FP32
    rounding of the forces' own size (normwise 1e-5 of the largest)."""
    s = ig.synth.make_system(2, 22, 60.0, 20, seed=12, ff=ig.synth.forcefield(n_mc=20))
    bp = np.asarray(s.bond_params).reshape(-1, 2)
    ap = np.asarray(s.angle_params).reshape(-1, 2)
    rng = np.random.default_rng(3)
    pos = s.pos.copy()
    pos[:22, :3] = equilibrium_chain(22, rng, np.array([20.0, 20.0, 15.0]), float(bp[0, 1]), float(ap[0, 1]))
    pos[22:, :3] = equilibrium_chain(22, rng, np.array([20.0, 20.0, 40.0]), float(bp[0, 1]), float(ap[0, 1]))
    pos[:, :2] += rng.uniform(-1e-6, 1e-6, (len(pos), 2))
    s.pos = pos.astype(np.float32)
    o = O.Oracle(s)
    eng = ig.Engine(s)
    for name, call, ref in [("angles", eng.angle_force, o.bonded(bonds=False, dihedrals=False)),
                            ("bonds", eng.bond_force, o.bonded(angles=False, dihedrals=False))]:
        eng.zero_forces()
        call()
        f = eng.forces()
        scale = float(np.abs(ref).max())
        err = float(np.abs(f - ref).max())
        print(f"chains at the minimum, {name}: max |F| {scale:.3e}, max |dF| {err:.3e}")
        assert err <= 1e-5 * max(scale, 1e-3)


def _trajectories(windows, steps, modes=(1, 2), **opts):
    out = []
    for integ in modes:
        eng = ig.Engine(windows, integrator=integ, **opts)
        assert eng.shapes()["integrator"] == integ
        eng.step(steps)
        out.append((eng.positions(), eng.velocities(), None, eng.us_com(), eng.get_step(), eng.device_status()))
        eng.close()
    return out


def _windows(which, adi2):
    if which == "medium":
        wins = ig.synth.make_system(12, 22, 34.0, 20, seed=21, ff=ig.synth.forcefield(n_mc=20))
        wins.pnu = 0.2
    elif which == "batched-umbrella":
        wins = ig.synth.config_batched(n_windows=3, seed=9)
    else:
        s = adi2.copy()
        s.n_mc = 20
        s.us_on = 1
        s.bias_list = np.array([(i, 0) for i in range(22)] + [(22 + i, 1) for i in range(22)], np.int32)
        s.us_k, s.us_x0 = 20.0, 10.0
        s.pnu = 0.05
        wins = s
    return wins


@pytest.mark.parametrize("which", ["medium", "batched-umbrella", "adi2-umbrella"])
def test_fused_integrator_bit_identical(which, adi2):
    (p1, v1, _, c1, st1, ds1), (p2, v2, _, c2, st2, ds2) = _trajectories(_windows(which, adi2), 12)
    assert ds1 == 0 and ds2 == 0
    assert st1 == st2 == 12
    assert np.array_equal(p1, p2)
    assert np.array_equal(v1, v2)
    assert np.array_equal(c1[0], c2[0]) and np.array_equal(c1[1], c2[1])


@pytest.mark.parametrize("which", ["medium", "batched-umbrella", "adi2-umbrella"])
def test_single_kernel_step_bit_identical(which, adi2):
    """The whole step as one cooperative kernel against the separate kernels,
    both with split-4 field tiles and the same work lists."""
    (p1, v1, _, c1, st1, ds1), (p3, v3, _, c3, st3, ds3) = _trajectories(_windows(which, adi2), 12, modes=(1, 3),
                                                                         field_split=4)
    assert ds1 == 0 and ds3 == 0
    assert st1 == st3 == 12
    assert np.array_equal(p1, p3)
    assert np.array_equal(v1, v3)
    assert np.array_equal(c1[0], c3[0]) and np.array_equal(c1[1], c3[1])


@pytest.mark.parametrize("integ", [1, 2])
@pytest.mark.parametrize("which", ["medium", "batched-umbrella", "adi2-umbrella"])
def test_programmatic_launches_bit_identical(which, integ, adi2):
    wins = _windows(which, adi2)
    runs = {}
    for pdl in (2, 1):
        for graph in (True, False):
            eng = ig.Engine(wins, integrator=integ, step_pdl=pdl, use_graph=graph)
            sh = eng.shapes()
            assert sh["integrator"] == integ and sh["step_pdl"] == (1 if pdl == 1 else 0)
            eng.step(12)
            runs[(pdl, graph)] = (eng.positions(), eng.velocities(), eng.get_step(), eng.device_status())
            eng.close()
    # isspa_step_host, device-mapped buffers read and written by the kernels
    eng = ig.Engine(wins, integrator=integ, step_pdl=1)
    n = eng.n_atoms
    bufs = [ig.host_array((n, 4)) for _ in range(5)]
    bufs[0][:] = eng.positions()
    bufs[1][:] = eng.velocities()
    for k in range(12):
        src, dst = (0, 2) if k % 2 == 0 else (2, 0)
        eng.step_host(bufs[src], bufs[src + 1], bufs[dst], bufs[dst + 1], bufs[4])
    runs["host"] = (bufs[0].copy(), bufs[1].copy(), eng.get_step(), eng.device_status())
    eng.close()
    p0, v0, st0, ds0 = runs[(2, True)]
    assert ds0 == 0 and st0 == 12
    for key, (p, v, st, ds) in runs.items():
        assert ds == 0 and st == 12, key
        assert np.array_equal(p, p0), key
        assert np.array_equal(v, v0), key


def test_step_pdl_option_checked():
    s = ig.synth.config_small(seed=1)
    for bad in (-1, 3):
        with pytest.raises(RuntimeError):
            ig.Engine(s, step_pdl=bad)
    eng = ig.Engine(s, integrator=3, step_pdl=1)
    assert eng.shapes()["integrator"] == 3  # the single-kernel step has no chain to launch
    eng.step(2)
    assert eng.device_status() == 0


def test_autotune_restores_state():
    s = ig.synth.config_small(seed=1)
    a = ig.Engine(s)
    b = ig.Engine(s)
    a.step(3)
    b.step(3)
    sh = a.autotune()
    assert sh["integrator"] in (1, 2, 3) and sh["step_pdl"] in (0, 1)
    assert a.get_step() == 3
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())
    a.step(5)
    b.step(5)
    # the tuned shapes move results at FP32 rounding level only
    assert np.allclose(a.positions(), b.positions(), rtol=0, atol=1e-4)


@pytest.mark.parametrize("mode", [2, 3], ids=["fused-integrator", "single-kernel-step"])
def test_grid_barrier_timeout_is_reported(mode):
    """A grid barrier left mid-count (as after a lost block) never completes:
    every block's bounded wait runs out, the step reports ISSPA_ERR_TIMEOUT,
    nothing faults, and after the status reset the engine steps on cleanly
    from a valid state."""
    s = ig.synth.config_small(seed=1)
    eng = ig.Engine(s, integrator=mode)
    ref = ig.Engine(s, integrator=mode)
    assert eng.shapes()["integrator"] == mode
    L = abi.lib()
    abi.check(L.isspa_debug_stall_barrier(eng._h), "stall barrier")
    eng.step(1)
    assert eng.device_status() == abi.ERR_TIMEOUT
    assert eng.device_status(reset=True) == abi.ERR_TIMEOUT
    assert eng.device_status() == 0
    eng.set_positions(s.pos)
    eng.set_velocities(s.vel)
    eng.set_step(0)
    eng.zero_forces()
    eng.step(10)
    ref.step(10)
    assert eng.device_status() == 0
    assert np.array_equal(eng.positions(), ref.positions())
