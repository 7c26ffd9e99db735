"""Edge cases of the step on the GPU, against the FP64 oracle.

* a single atom (no bonded terms, its own MC points only, zero charge);
* an ion pair (two one-atom chains, no bonds);
* nMC = 1 (one MC point per atom);
* one engine batching windows of 1, 2 and 44 atoms with different boxes
  (work lists with ragged and nearly empty windows);
* 100 graph steps of each without a tripped device status.
"""
import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from parity import check_force

pytestmark = pytest.mark.gpu


def _sys(n_chains, length, n_mc, box=30.0, seed=3):
    return ig.synth.make_system(n_chains, length, box, n_mc, seed=seed, ff=ig.synth.forcefield(n_mc=n_mc))


@pytest.mark.parametrize("shape", [(1, 1, 20), (2, 1, 20), (1, 22, 1), (2, 22, 1)],
                         ids=["single-atom", "ion-pair", "chain-nmc1", "two-chains-nmc1"])
def test_small_systems_match_oracle(shape):
    s = _sys(*shape)
    eng = ig.Engine(s)
    f = eng.compute_forces()
    ref, _, _ = O.Oracle(s).total_force(seed=s.seed, step=0)
    check_force(f, ref, f"{shape}")
    eng.zero_forces()
    eng.step(100)
    assert eng.device_status() == 0
    assert np.all(np.isfinite(eng.positions()))


def test_ragged_batch_matches_oracle():
    wins = [_sys(1, 1, 20, box=30.0, seed=5), _sys(2, 1, 20, box=35.0, seed=6), _sys(2, 22, 20, box=40.0, seed=7)]
    eng = ig.Engine(wins)
    f = eng.compute_forces()
    off = 0
    for w, s in enumerate(wins):
        ref, _, _ = O.Oracle(s).total_force(seed=s.seed, step=0, window=w)
        check_force(f[off:off + s.n_atoms], ref, f"ragged batch window {w}")
        off += s.n_atoms
    eng.zero_forces()
    eng.step(100)
    assert eng.device_status() == 0
