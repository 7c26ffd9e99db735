"""Test-harness pieces for umbrella-window statistics (not part of the library).

* `window_system`: the 44-atom two-chain system with a COM-distance restraint
  between the chains, unwrapped along the bonds and centred in an 80 A box.
  The reference's restraint takes each group's centre of mass from the
  wrapped coordinates (us_force_cuda.cu:29-34), which is meaningless for a
  group straddling the box edge; in a box twice the system's size no group
  reaches an edge during the runs used here.
* `oracle_cv_series`: the CV |COM0 - COM1| of every `every`-th step of an
  oracle MD run (IS-SPA, nonbond, bonded, restraint, leapfrog + Andersen),
  with the engine's Philox keys.
* `replica_stats`, `umbrella_integration`: the mean restraint force
  -k(<d> - x0) of a window from independent replicas (each replica its own
  Philox window index, so its own thermostat and MC-point streams); the
  standard error comes from the spread of the replica means, which unlike
  blocks of one run are uncorrelated (the CV relaxes over tens of ps).  Then
  the free-energy profile from integrating the mean forces between window
  means (trapezoids), with propagated errors.
"""
from __future__ import annotations

import numpy as np

import isspa_gb300.synth as synth
import oracle as O

K_US = 10.0
X0S = (6.0, 8.0, 10.0, 12.0)
REPLICAS = 8
EQUIL_STEPS = 10_000
PROD_STEPS = 50_000
EVERY = 10


def window_index(replica: int, window: int) -> int:
    """Position of (replica, window) in the batched engine: replica-major."""
    return replica * len(X0S) + window


def window_system(x0: float, box: float = 80.0, seed: int = 1):
    s = synth.make_system(2, 22, 40.0, 20, seed=seed, us=(K_US, x0))
    L0 = float(s.box)
    xyz = s.pos[:, :3].astype(np.float64)
    for c in range(2):
        for i in range(22 * c + 1, 22 * (c + 1)):
            xyz[i] -= L0 * np.round((xyz[i] - xyz[i - 1]) / L0)
    com0, com1 = xyz[:22].mean(0), xyz[22:].mean(0)
    xyz[22:] -= L0 * np.round((com1 - com0) / L0)
    xyz += 0.5 * box - xyz.mean(0)
    pos = s.pos.copy()
    pos[:, :3] = xyz
    s.pos = np.ascontiguousarray(pos, np.float32)
    s.box = np.float32(box)
    return s


def _cv(com, box):
    d = com[0] - com[1]
    d = d - box * np.where(d > 0.5 * box, 1.0, np.where(d < -0.5 * box, -1.0, 0.0))
    return float(np.linalg.norm(d))


def oracle_cv_series(s, n_steps: int, every: int, window: int = 0, threads: int = 1):
    t = s.copy()
    t.pos = np.ascontiguousarray(s.pos, np.float32).copy()
    t.vel = np.ascontiguousarray(s.vel, np.float32).copy()
    o = O.Oracle(t, threads=threads)  # reads o.pos / t.vel in place every call
    cv = []
    for k in range(n_steps):
        f, _, com = o.total_force(s.seed, k, window)
        po, vo, _ = o.leapfrog(f, s.seed, k, window)
        if (k + 1) % every == 0:
            cv.append(_cv(com, float(s.box)))
        if not np.all(np.isfinite(po)):
            raise FloatingPointError(f"oracle run diverged at step {k}")
        o.pos[:, :3] = po
        t.vel[:, :3] = vo
    return np.asarray(cv)


def replica_stats(replica_means, x0: float, k: float = K_US):
    r = np.asarray(replica_means, np.float64)
    m, se = float(r.mean()), float(r.std(ddof=1) / np.sqrt(len(r)))
    return {"mean_cv": m, "se_cv": se, "mean_force": -k * (m - x0), "se_force": k * se,
            "replica_means": r.tolist()}


def umbrella_integration(mean_cv, mean_force, se_force):
    """A(xi) at the window means (A = 0 at the first), with standard errors:
    dA/dxi = -<F_restraint> = k(<xi> - x0), integrated by trapezoids."""
    order = np.argsort(mean_cv)
    xi = np.asarray(mean_cv)[order]
    g = -np.asarray(mean_force)[order]
    se = np.asarray(se_force)[order]
    A, var = [0.0], [0.0]
    for i in range(1, len(xi)):
        h = xi[i] - xi[i - 1]
        A.append(A[-1] + 0.5 * h * (g[i] + g[i - 1]))
        var.append(var[-1] + (0.5 * h) ** 2 * (se[i] ** 2 + se[i - 1] ** 2))
    return xi, np.asarray(A), np.sqrt(np.asarray(var))
