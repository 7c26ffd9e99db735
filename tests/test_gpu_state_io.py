"""Host-buffer state transfer through the C ABI.

* isspa_step_host (upload positions and velocities, one step, download
  positions, velocities and the step's forces) chained over 10 steps gives
  the trajectory of 10 graph-replayed isspa_step calls bit for bit;
* the forces it returns are those of the per-call sequence on the same state;
* set/get of positions, velocities and the step counter round-trip exactly,
  and a restored state continues the same trajectory;
* with isspa_host_alloc buffers (read and written by kernels over the host
  link) the chain is bit for bit the chain through ordinary host memory
  (copies), also with inputs or outputs left out.
"""
import numpy as np
import pytest

import isspa_gb300 as ig

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return ig.synth.make_system(6, 22, 36.0, 20, seed=8, ff=ig.synth.forcefield(n_mc=20))


def test_step_host_chain_equals_graph_steps(system):
    a, b = ig.Engine(system), ig.Engine(system)
    n = a.n_atoms
    pos, vel = a.positions(), a.velocities()
    out_p, out_v, out_f = (np.zeros((n, 4), np.float32) for _ in range(3))
    forces = []
    for _ in range(10):
        a.step_host(pos, vel, out_p, out_v, out_f)
        forces.append(out_f[:, :3].copy())
        pos, vel = out_p.copy(), out_v.copy()
    b_forces = []
    for _ in range(10):
        f = b.compute_forces()  # the step's forces on b's current state
        b.zero_forces()
        b_forces.append(f)
        b.step(1)
    assert np.array_equal(pos, b.positions())
    assert np.array_equal(vel, b.velocities())
    assert a.get_step() == b.get_step() == 10
    for fa, fb in zip(forces, b_forces):
        assert np.array_equal(fa, fb)
    assert a.device_status() == 0


def test_state_round_trip_and_restore(system):
    eng = ig.Engine(system)
    eng.step(7)
    p, v, st = eng.positions(), eng.velocities(), eng.get_step()
    eng.step(5)
    ahead = eng.positions()
    eng.set_positions(p)
    eng.set_velocities(v)
    eng.set_step(st)
    assert np.array_equal(eng.positions(), p) and np.array_equal(eng.velocities(), v)
    assert eng.get_step() == st
    eng.step(5)
    assert np.array_equal(eng.positions(), ahead)


def test_step_host_direct_buffers_equal_copies(system):
    a, b = ig.Engine(system), ig.Engine(system)
    n = a.n_atoms
    bufs = [ig.host_array((n, 4)) for _ in range(5)]
    bufs[0][:] = a.positions()
    bufs[1][:] = a.velocities()
    pos, vel = b.positions(), b.velocities()
    outs = [np.zeros((n, 4), np.float32) for _ in range(3)]
    for k in range(10):
        src, dst = (0, 2) if k % 2 == 0 else (2, 0)
        a.step_host(bufs[src], bufs[src + 1], bufs[dst], bufs[dst + 1], bufs[4])
        b.step_host(pos, vel, *outs)
        pos, vel = outs[0].copy(), outs[1].copy()
        assert np.array_equal(bufs[4], outs[2])
        assert np.array_equal(bufs[dst], pos) and np.array_equal(bufs[dst + 1], vel)
    # inputs left out: the step continues from the device state
    a.step_host(None, None, bufs[0], None, bufs[4])
    b.step_host(None, None, outs[0], None, outs[2])
    assert np.array_equal(bufs[0], outs[0]) and np.array_equal(bufs[4], outs[2])
    # a mapped input with an ordinary output buffer falls back to copies
    f_plain = np.zeros((n, 4), np.float32)
    a.step_host(bufs[0], None, None, None, f_plain)
    b.step_host(outs[0], None, None, None, outs[2])
    assert np.array_equal(f_plain, outs[2])
    assert a.device_status() == 0
