"""Test-harness pieces for the mean-force gradient (not part of the library).

* `theta_params`: the 25 force-field parameters theta = (epsilon, sigma, x0, w,
  g0) per type, as a torch tensor, mapped to table parameters.
* `MeanForce`: torch.autograd.Function around the engine's
  isspa_adjoint_mean_force (forward = J per window, backward = dJ/dtables).
* `oracle_J`: J from the FP64 oracle with FP64 tables, for central differences.
"""
from __future__ import annotations

import numpy as np

import isspa_gb300.synth as synth
import oracle as O

NAMES = ("epsilon", "sigma", "x0", "w", "g0")


def theta0(ff):
    p = ff["params"]
    return np.concatenate([p[k] for k in NAMES]).astype(np.float64)


def params_of(theta, ff):
    """Table parameters with theta (numpy or torch) in place of the five per-type sets."""
    p = dict(ff["params"])
    nt = len(p["sigma"])
    for i, k in enumerate(NAMES):
        p[k] = theta[i * nt:(i + 1) * nt]
    return p


def chain_to_theta(theta, ff, df, dg, dA, dB):
    """dJ/dtheta from dJ/dtables through the differentiable table generator."""
    import torch

    th = torch.tensor(np.asarray(theta, np.float64), requires_grad=True)
    T = synth.tables_from_params(params_of(th, ff), xp=torch)
    lin = ((torch.from_numpy(np.asarray(dg)) * T["g"]).sum() + (torch.from_numpy(np.asarray(df)) * T["f"]).sum()
           + (torch.from_numpy(np.asarray(dA)) * T["lj_ab"][:, 0]).sum()
           + (torch.from_numpy(np.asarray(dB)) * T["lj_ab"][:, 1]).sum())
    lin.backward()
    return th.grad.numpy()


def central_differences(fun, theta, rel=1e-4):
    theta = np.asarray(theta, np.float64)
    out = np.zeros_like(theta)
    for k in range(len(theta)):
        h = rel * abs(theta[k])
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        out[k] = (fun(tp) - fun(tm)) / (2 * h)
    return out


def tables_np(theta, ff):
    return synth.tables_from_params(params_of(np.asarray(theta, np.float64), ff))


def oracle_J(theta, ff, frames, window_systems, steps):
    """sum over windows of the frame-mean COM-axis force, all in FP64."""
    t = tables_np(theta, ff)
    tot = 0.0
    for w, s in enumerate(window_systems):
        Jw = 0.0
        for f, st in enumerate(steps):
            sf = s.copy()
            sf.pos = frames[w][f]
            o = O.Oracle(sf, tables={"g": t["g"], "f": t["f"], "lj_ab": t["lj_ab"]})
            pts = o.mc_points(seed=s.seed, step=int(st), window=w)
            Jw += o.mean_force(pts)
        tot += Jw / len(steps)
    return tot


def make_mean_force_function():
    import torch

    class MeanForce(torch.autograd.Function):
        """J_w(tables) through the GPU engine; backward = the engine's adjoint."""

        @staticmethod
        def forward(ctx, g, f, lj_ab, engine, steps, frames, e_table):
            engine.set_tables(g.detach().cpu().numpy(), e_table, f.detach().cpu().numpy(),
                              lj_ab.detach().cpu().numpy())
            J, df, dg, dA, dB = engine.adjoint_mean_force(steps, frames)
            ctx.save_for_backward(torch.from_numpy(dg), torch.from_numpy(df),
                                  torch.from_numpy(np.stack([dA, dB], -1)))
            return torch.from_numpy(J)

        @staticmethod
        def backward(ctx, gJ):
            dg, df, dlj = ctx.saved_tensors
            gw = gJ.to(dg.dtype)
            return ((gw[:, None, None] * dg).sum(0), (gw[:, None, None] * df).sum(0),
                    (gw[:, None, None] * dlj).sum(0), None, None, None, None)

    return MeanForce
