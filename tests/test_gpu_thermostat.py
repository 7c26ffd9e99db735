"""Andersen thermostat: sampled velocities against the Maxwell-Boltzmann
distribution at the set temperature, at the collision probabilities of the
reference's velocity-histogram check (timing_tests/LJ/pnu/vel_dist.py:
pnu = 0.01, 0.05, 0.10 per step).

220 atoms (10 chains), full IS-SPA model; after 5 000 steps of equilibration,
velocities every 100 steps for 20 000 steps.  With z = v sqrt(m/kT) per
component:
  * shape: kurtosis <z^4>/<z^2>^2 = 3 within 2 %, and the Kolmogorov-Smirnov
    distance of z/sqrt(<z^2>) to the unit normal below 0.006;
  * scale: <z^2> = 1 within 4 %.  The stored velocities are the leapfrog's
    half-step ones, whose variance exceeds kT/m by O((w dt)^2) for a mode of
    frequency w; the k = 300 bonds (period ~30 fs) give about 2 % at 2 fs, and
    the second test shows the excess falling when the step is halved.
"""
from math import erf, sqrt

import numpy as np
import pytest

import isspa_gb300 as ig
import isspa_gb300.synth as synth

pytestmark = pytest.mark.gpu


def _sample(pnu, dt_scale=1.0, n_samples=200, every=100):
    s = synth.make_system(10, 22, 40.0, 20, seed=17, pnu=pnu)
    s.dt = s.dt * dt_scale
    eng = ig.Engine(s)
    eng.step(int(5000 / dt_scale))
    m = s.vel[:, 3].astype(np.float64)
    z = []
    for _ in range(n_samples):
        eng.step(int(every / dt_scale))
        v = eng.velocities()[:, :3].astype(np.float64)
        z.append(v * np.sqrt(m / float(s.kT))[:, None])
    assert eng.device_status() == 0
    return np.concatenate(z).ravel()


def _ks_normal(z):
    zs = np.sort(z)
    cdf = 0.5 * (1.0 + np.vectorize(erf)(zs / sqrt(2.0)))
    n = len(zs)
    return float(max(np.max(np.arange(1, n + 1) / n - cdf), np.max(cdf - np.arange(n) / n)))


@pytest.mark.parametrize("pnu", [0.01, 0.05, 0.10])
def test_velocities_are_maxwell_boltzmann(pnu):
    z = _sample(pnu)
    m2, m4 = float(np.mean(z * z)), float(np.mean(z ** 4))
    kurt = m4 / (m2 * m2)
    ks = _ks_normal(z / sqrt(m2))
    print(f"pnu {pnu}: <z^2> {m2:.4f}, kurtosis {kurt:.4f}, KS distance (standardised) {ks:.4f} "
          f"over {len(z)} samples")
    assert abs(kurt - 3.0) < 0.06
    assert ks < 0.006
    assert abs(m2 - 1.0) < 0.04


def test_half_step_velocity_excess_shrinks_with_the_time_step():
    e2 = float(np.mean(_sample(0.05) ** 2)) - 1.0
    e1 = float(np.mean(_sample(0.05, dt_scale=0.5) ** 2)) - 1.0
    print(f"<z^2> - 1: {e2:+.4f} at 2 fs, {e1:+.4f} at 1 fs")
    assert e1 < 0.5 * e2
