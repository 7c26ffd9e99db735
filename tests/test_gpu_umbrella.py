"""Umbrella-window mean forces on the GPU against the FP64 oracle's runs.

Four 44-atom windows (COM-distance restraint between the two chains, k = 10,
x0 = 6, 8, 10, 12 A; full IS-SPA model, Andersen thermostat at 298 K), 8
independent replicas each, run as one batched engine of 32 windows for
10 000 + 50 000 steps.  The mean restraint force -k(<d> - x0) of every window
(standard error from the spread of the replica means) agrees with the
oracle's own runs of the same replicas (tests/golden/us_windows_44.json, made
by tests/golden/make_us_windows.py) within 2 combined standard errors, and so
does the free-energy profile obtained by integrating the mean forces
(umbrella integration) across the windows.  The runs start from the same
states with the same Philox keys and separate chaotically, so the comparison
is statistical.

The same comparison step by step: one restrained window run on the GPU and by
the FP64-state oracle from the same state with the same Philox streams (MC
points and thermostat draws) follows one trajectory up to the rounding of the
state, so the CV agrees within 1e-3 A over the first 200 steps (two oracle
runs started 1e-6 A apart differ by 2e-5 A there), where a bias of 1 % in the
restraint force would already move it by ~0.1 A.
"""
import json
import os

import numpy as np
import pytest

import isspa_gb300 as ig
import us_harness as U

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "us_windows_44.json")


def test_window_mean_forces_agree_with_oracle_within_two_sigma():
    with open(GOLDEN) as f:
        ref = json.load(f)
    assert ref["k"] == U.K_US and ref["every"] == U.EVERY and ref["prod_steps"] == U.PROD_STEPS
    assert ref["replicas"] == U.REPLICAS
    wins = [U.window_system(x0) for _ in range(U.REPLICAS) for x0 in U.X0S]
    eng = ig.Engine(wins)
    n = (U.EQUIL_STEPS + U.PROD_STEPS) // U.EVERY
    cv = np.zeros((n, len(wins)))
    for k in range(n):
        eng.step(U.EVERY)
        cv[k] = eng.us_com()[1]
    assert eng.device_status() == 0
    means = cv[U.EQUIL_STEPS // U.EVERY:].mean(0)
    gpu = [U.replica_stats([means[U.window_index(r, w)] for r in range(U.REPLICAS)], x0)
           for w, x0 in enumerate(U.X0S)]
    orc = ref["windows"]
    z = []
    for g, o in zip(gpu, orc):
        se = np.hypot(g["se_force"], o["se_force"])
        z.append((g["mean_force"] - o["mean_force"]) / se)
        print(f"x0 {o['x0']:5.1f}: mean force GPU {g['mean_force']:+.3f} +- {g['se_force']:.3f}, "
              f"oracle {o['mean_force']:+.3f} +- {o['se_force']:.3f}, z {z[-1]:+.2f}")
    xg, Ag, sg = U.umbrella_integration([g["mean_cv"] for g in gpu], [g["mean_force"] for g in gpu],
                                        [g["se_force"] for g in gpu])
    xo, Ao, so = U.umbrella_integration([o["mean_cv"] for o in orc], [o["mean_force"] for o in orc],
                                        [o["se_force"] for o in orc])
    zA = (Ag[-1] - Ao[-1]) / np.hypot(sg[-1], so[-1])
    print(f"PMF from {xg[0]:.2f} to {xg[-1]:.2f} A: GPU {Ag[-1]:+.3f} +- {sg[-1]:.3f} kcal/mol, "
          f"oracle ({xo[0]:.2f} to {xo[-1]:.2f} A) {Ao[-1]:+.3f} +- {so[-1]:.3f}, z {zA:+.2f}")
    assert np.all(np.abs(z) <= 2.0)
    assert abs(zA) <= 2.0


def test_window_tracks_fp64_oracle_step_by_step():
    """One 44-atom window (x0 = 10 A, full model: IS-SPA, nonbond, bonded,
    restraint, leapfrog + Andersen) on the GPU and in the FP64-state oracle,
    same state and Philox streams: the restraint CV of every step agrees."""
    s = U.window_system(10.0)
    n = 200
    cv_o = U.oracle_cv_series(s, n, 1)
    eng = ig.Engine(s)
    cv_g = np.zeros(n)
    for k in range(n):
        eng.step(1)
        cv_g[k] = eng.us_com()[1][0]
    assert eng.device_status() == 0
    d = np.abs(cv_g - cv_o)
    print(f"CV {cv_o[0]:.4f} -> {cv_o[-1]:.4f} A over {n} steps; |GPU - oracle| max over the first 20 / 100 / "
          f"{n} steps: {d[:20].max():.2e} / {d[:100].max():.2e} / {d.max():.2e} A")
    assert d[:20].max() < 1e-4
    assert d.max() < 1e-3
