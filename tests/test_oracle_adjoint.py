"""The FP64 adjoint of the oracle (the naive reference gradient) against FP64
central finite differences in the 25 force-field parameters (CPU only)."""
import numpy as np
import pytest

import isspa_gb300.synth as synth
import oracle as O
from adjoint_harness import central_differences, chain_to_theta, oracle_J, tables_np, theta0


def test_oracle_adjoint_matches_fp64_finite_differences():
    pytest.importorskip("torch")
    ff = synth.forcefield(n_mc=10)
    s = synth.make_system(2, 22, 40.0, 10, seed=3, ff=ff, us=(10.0, 6.0))
    th = theta0(ff)
    steps = [5]
    t = tables_np(th, ff)
    o = O.Oracle(s, tables={"g": t["g"], "f": t["f"], "lj_ab": t["lj_ab"]})
    pts = o.mc_points(seed=s.seed, step=steps[0], window=0)
    J, df, dg, dA, dB = o.adjoint(pts)
    grad = chain_to_theta(th, ff, df, dg, dA, dB)
    fd = central_differences(lambda x: oracle_J(x, ff, [[s.pos]], [s], steps), th, rel=1e-4)
    err = np.abs(grad - fd).max() / np.abs(fd).max()
    # central differences at h = 1e-4 relative carry an O(h^2) truncation
    # error of ~2e-6 here (the LJ terms go as sigma^12)
    assert err < 1e-5, (err, grad, fd)
    # every parameter family carries gradient
    for i in range(5):
        assert np.abs(fd[5 * i:5 * i + 5]).max() > 0
