"""Failure detection without a GPU fault.

A numerical failure is made on the host side: two atoms of different chains
(a pair the nonbond pass never excludes) are placed on one another, or 0.05 A
apart.  The kernels' own checks flag the resulting force (non-finite, or
beyond the fixed-point accumulator's range) in the engine's sticky status
word; the host reads it through isspa_device_status, clears it, restores a
valid state and steps on in the same context.

Non-finite or huge positions never become memory addresses in a step kernel:
the only position-derived indices are the table bins of the field and force
passes, and both are range-checked before the table is read.
"""
import numpy as np
import pytest

import isspa_gb300 as ig
from isspa_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sep, code", [(0.0, abi.ERR_NONFINITE), (0.05, abi.ERR_OVERFLOW)],
                         ids=["coincident", "0.05A"])
def test_collapsed_pair_trips_device_status(sep, code):
    s = ig.synth.make_system(2, 22, 36.0, 20, seed=4, ff=ig.synth.forcefield(n_mc=20))
    bad = s.copy()
    bad.pos = s.pos.copy()
    bad.pos[5, :3] = s.pos[30, :3] + np.array([sep, 0.0, 0.0], np.float32)  # chain 0 onto chain 1
    eng = ig.Engine(bad)
    assert eng.device_status() == 0
    eng.step(1)
    assert eng.device_status() == code
    assert eng.device_status(reset=True) == code  # read and clear
    assert eng.device_status() == 0
    # same context, valid state again: clean steps
    eng.set_positions(s.pos)
    eng.set_velocities(s.vel)
    eng.step(10)
    assert eng.device_status() == 0
    assert np.all(np.isfinite(eng.positions()))
