"""Force work items starting on stamped field tiles (isspa_engine_options.
force_overlap = 1), through the C ABI.

In isspa_step the field blocks stamp their tiles once their point records are
written, and each force item waits (bounded) only for the tiles its chunk lies
in; under programmatic launches the force pass then starts in the field
pass's last wave.  The work lists and the per-item arithmetic are unchanged,
and forces accumulate in fixed point, so:

* trajectories with and without the overlap are bit-identical: the 1100-atom
  system, three uneven batched windows and the ADI2 dimer, with either
  integrator, programmatic or ordinary launches, graph replays or direct
  stream launches, and through isspa_step_host;
* the stamps survive changes of the launch shapes between steps (a new field
  split, a switch of integrator) and the per-call functions in between;
* the option is reported in the shapes and checked.
"""
import numpy as np
import pytest

import isspa_gb300 as ig

pytestmark = pytest.mark.gpu


def _windows(which, adi2):
    if which == "plain":
        return ig.synth.config_plain(seed=2)
    if which == "batched":
        return ig.synth.config_batched(n_windows=3, seed=9)
    s = adi2.copy()
    s.n_mc = 100
    s.us_on = 1
    s.bias_list = np.array([(i, 0) for i in range(22)] + [(22 + i, 1) for i in range(22)], np.int32)
    s.us_k, s.us_x0 = 20.0, 10.0
    s.pnu = 0.05
    return s


def _run(wins, steps, **opts):
    eng = ig.Engine(wins, **opts)
    eng.step(steps)
    out = (eng.positions(), eng.velocities(), eng.get_step(), eng.device_status(), eng.shapes())
    eng.close()
    return out


@pytest.mark.parametrize("which", ["plain", "batched", "adi2"])
@pytest.mark.parametrize("integ", [1, 2])
def test_overlap_trajectories_bit_identical(which, integ, adi2):
    wins = _windows(which, adi2)
    steps = 6 if which == "plain" else 10
    ref = _run(wins, steps, integrator=integ, step_pdl=2, force_overlap=2, isspa_fused=2)
    assert ref[3] == 0 and ref[4]["force_overlap"] == 0
    for pdl in (1, 2):
        for graph in (True, False):
            got = _run(wins, steps, integrator=integ, step_pdl=pdl, force_overlap=1, isspa_fused=2,
                       use_graph=graph)
            assert got[4]["force_overlap"] == 1
            assert got[3] == 0 and got[2] == steps
            assert np.array_equal(got[0], ref[0]), (pdl, graph)
            assert np.array_equal(got[1], ref[1]), (pdl, graph)


def test_overlap_through_step_host(adi2):
    wins = _windows("adi2", adi2)
    ref = _run(wins, 8, force_overlap=2, isspa_fused=2, step_pdl=1)
    eng = ig.Engine(wins, force_overlap=1, isspa_fused=2, step_pdl=1)
    n = eng.n_atoms
    bufs = [ig.host_array((n, 4)) for _ in range(5)]
    bufs[0][:] = eng.positions()
    bufs[1][:] = eng.velocities()
    for k in range(8):
        src, dst = (0, 2) if k % 2 == 0 else (2, 0)
        eng.step_host(bufs[src], bufs[src + 1], bufs[dst], bufs[dst + 1], bufs[4])
    assert eng.device_status() == 0
    assert np.array_equal(bufs[0], ref[0]) and np.array_equal(bufs[1], ref[1])
    eng.close()


def test_overlap_across_shape_changes_and_calls():
    """Steps with the overlap, interleaved with per-call force evaluations, an
    autotune (new field split, step mode, stamps left from its trial steps)
    and steps again: the same trajectory as without the overlap."""
    s = ig.synth.make_system(12, 22, 34.0, 20, seed=21, ff=ig.synth.forcefield(n_mc=20))
    traj = {}
    for ov in (2, 1):
        eng = ig.Engine(s, force_overlap=ov, isspa_fused=2, step_pdl=1, field_split=8)
        eng.step(3)
        eng.compute_forces()
        eng.zero_forces()
        eng.step(2)
        eng.autotune()
        eng.step(4)
        traj[ov] = (eng.positions(), eng.velocities(), eng.device_status())
        eng.close()
    assert traj[1][2] == 0 and traj[2][2] == 0
    # the autotuner may pick different shapes in the two engines: FP32
    # summation order of the force items only
    assert np.allclose(traj[1][0], traj[2][0], rtol=0, atol=1e-4)
    for ov in (2, 1):
        eng = ig.Engine(s, force_overlap=ov, isspa_fused=2, step_pdl=1, field_split=8)
        eng.step(3)
        eng.compute_forces()
        eng.zero_forces()
        eng.step(2)
        traj[ov] = (eng.positions(), eng.velocities(), eng.device_status())
        eng.close()
    assert np.array_equal(traj[1][0], traj[2][0]) and np.array_equal(traj[1][1], traj[2][1])


def test_overlap_option_checked_and_inapplicable_modes():
    s = ig.synth.config_small(seed=1)
    for bad in (-1, 3):
        with pytest.raises(RuntimeError):
            ig.Engine(s, force_overlap=bad)
    eng = ig.Engine(s, force_overlap=1, isspa_fused=1, field_split=16)
    assert eng.shapes()["isspa_fused"] == 1 and eng.shapes()["force_overlap"] == 0  # no separate force pass
    eng.step(3)
    assert eng.device_status() == 0
    eng.close()
    eng = ig.Engine(s, force_overlap=1, integrator=3)
    assert eng.shapes()["integrator"] == 3 and eng.shapes()["force_overlap"] == 0
    eng.step(3)
    assert eng.device_status() == 0
    eng.close()
