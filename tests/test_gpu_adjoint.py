"""GPU adjoint of the mean COM-axis force (differentiation workload: 25 chains,
550 atoms, 50 A box, umbrella windows; reduced here to 2 windows, nMC 20 and
2 frames to keep the FP64 finite differences quick).

Checks, through the C ABI and a torch.autograd.Function wrapper:
  * J per window against the FP64 oracle (1e-5 relative);
  * dJ/dtables against the oracle's naive FP64 adjoint (1e-5 normwise);
  * dJ/dtheta for theta = (epsilon, sigma, x0, w, g0) per type against FP64
    central finite differences with h = 1e-4 relative (target 1e-4).
"""
import numpy as np
import pytest

import isspa_gb300 as ig
import isspa_gb300.synth as synth
import oracle as O
from adjoint_harness import central_differences, make_mean_force_function, oracle_J, params_of, tables_np, theta0

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    ff = synth.forcefield(n_mc=20)
    base = synth.make_system(25, 22, 50.0, 20, seed=5, ff=ff, us=(10.0, 5.0))
    wins = []
    for x0 in (5.0, 9.0):
        s = base.copy()
        s.us_x0 = x0
        wins.append(s)
    th = theta0(ff)
    t = tables_np(th, ff)
    for s in wins:  # the engine starts from the generator's tables at theta0
        s.g_table, s.f_table, s.lj_ab = (t["g"].astype(np.float32), t["f"].astype(np.float32),
                                         t["lj_ab"].astype(np.float32))
    eng = ig.Engine(wins)
    eng.step(10)
    pos1 = eng.positions()
    eng.step(10)
    pos2 = eng.positions()
    frames = np.stack([pos1, pos2])
    steps = [101, 202]
    n = base.n_atoms
    per_window = [[frames[f][w * n:(w + 1) * n] for f in range(2)] for w in range(2)]
    return ff, wins, eng, frames, steps, per_window, th


def test_adjoint_value_and_table_gradient_match_fp64_oracle(setup):
    ff, wins, eng, frames, steps, per_window, th = setup
    J, df, dg, dA, dB = eng.adjoint_mean_force(steps, frames)
    t = tables_np(th, ff)
    for w, s in enumerate(wins):
        Jo = 0.0
        acc = [np.zeros_like(df[w]), np.zeros_like(dg[w]), np.zeros_like(dA[w]), np.zeros_like(dB[w])]
        for f, st in enumerate(steps):
            sf = s.copy()
            sf.pos = per_window[w][f]
            o = O.Oracle(sf, tables={"g": t["g"], "f": t["f"], "lj_ab": t["lj_ab"]})
            pts = o.mc_points(seed=s.seed, step=st, window=w)
            Jo += o.mean_force(pts)
            _, a, b, c, d = o.adjoint(pts)
            for k, v in enumerate((a, b, c, d)):
                acc[k] += v
        Jo /= len(steps)
        acc = [a / len(steps) for a in acc]
        print(f"window {w}: J gpu {J[w]:.6f} oracle {Jo:.6f}")
        assert abs(J[w] - Jo) <= 1e-5 * max(abs(Jo), 1.0)
        for got, ref in zip((df[w], dg[w], dA[w], dB[w]), acc):
            if np.abs(ref).max() == 0:
                assert np.abs(got).max() == 0
                continue
            assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_adjoint_theta_gradient_matches_central_differences(setup):
    torch = pytest.importorskip("torch")
    ff, wins, eng, frames, steps, per_window, th = setup
    MeanForce = make_mean_force_function()
    theta = torch.tensor(th, requires_grad=True)
    T = synth.tables_from_params(params_of(theta, ff), xp=torch)
    J = MeanForce.apply(T["g"], T["f"], T["lj_ab"], eng, np.asarray(steps), frames, wins[0].e_table)
    J.sum().backward()
    grad = theta.grad.numpy()
    fd = central_differences(lambda x: oracle_J(x, ff, per_window, wins, steps), th, rel=1e-4)
    err = np.abs(grad - fd).max() / np.abs(fd).max()
    print("dJ/dtheta gpu", np.round(grad, 6))
    print("dJ/dtheta fd ", np.round(fd, 6))
    print("normwise relative error", err)
    assert err < 1e-4


def test_adjoint_repeat_calls_agree(setup):
    """Consecutive multi-frame calls give the same J and gradients (FP64
    atomics only reorder sums); each frame's uploads are ordered after the
    previous frame's adjoint kernels."""
    ff, wins, eng, frames, steps, per_window, th = setup
    a = eng.adjoint_mean_force(steps, frames)
    eng.step(3)
    b = eng.adjoint_mean_force(steps, frames)
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= 1e-12 * max(np.abs(x).max(), 1e-300)


@pytest.mark.slow
def test_adjoint_full_differentiation_workload():
    """The differentiation workload at full size (16 windows of 550 atoms,
    nMC 50, r0 5..12 A): J and dJ/dtables of the first and last windows against
    the oracle's naive FP64 adjoint for one frame (1e-5 relative)."""
    wins = synth.config_adjoint()
    eng = ig.Engine(wins)
    eng.step(20)
    pos = eng.positions()
    J, df, dg, dA, dB = eng.adjoint_mean_force([20])
    n = wins[0].n_atoms
    for w in (0, len(wins) - 1):
        s = wins[w].copy()
        s.pos = pos[w * n:(w + 1) * n]
        o = O.Oracle(s)
        pts = o.mc_points(seed=s.seed, step=20, window=w)
        _, a, b, c, d = o.adjoint(pts)
        Jo = o.mean_force(pts)  # J also carries the bonded forces
        print(f"window {w}: J gpu {J[w]:.6f} oracle {Jo:.6f}")
        assert abs(J[w] - Jo) <= 1e-5 * max(abs(Jo), 1.0)
        for got, ref in zip((df[w], dg[w], dA[w], dB[w]), (a, b, c, d)):
            assert np.abs(got - ref).max() <= 1e-5 * max(np.abs(ref).max(), 1e-300)
    assert eng.device_status() == 0
