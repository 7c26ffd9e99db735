"""Regenerate tests/golden/us_windows_44.json: oracle umbrella-window statistics.

Runs the FP64 oracle MD of the four 44-atom umbrella windows of
tests/us_harness.py (IS-SPA, nonbond, bonded, COM restraint k = 10 at
x0 = 6, 8, 10, 12 A; leapfrog + Andersen at 298 K), REPLICAS independent
replicas each (Philox window index = the replica's position in a batched
engine), for EQUIL_STEPS + PROD_STEPS steps, and stores every replica's mean
CV over its production part and the window's mean restraint force with its
standard error over replicas.  The GPU test compares its own run of the same
replicas against these numbers (mean forces within 2 standard errors).
Takes ~10 minutes on 8 cores:

    python tests/golden/make_us_windows.py
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "isspa-force-cuda_gb300"), os.path.join(ROOT, "oracle"),
                os.path.dirname(HERE)]


def _run(job):
    import us_harness as U

    r, w = job
    s = U.window_system(U.X0S[w])
    cv = U.oracle_cv_series(s, U.EQUIL_STEPS + U.PROD_STEPS, U.EVERY, window=U.window_index(r, w))
    return float(cv[U.EQUIL_STEPS // U.EVERY:].mean())


def main():
    import us_harness as U

    jobs = [(r, w) for r in range(U.REPLICAS) for w in range(len(U.X0S))]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        means = dict(zip(jobs, pool.map(_run, jobs)))
    wins = []
    for w, x0 in enumerate(U.X0S):
        st = U.replica_stats([means[(r, w)] for r in range(U.REPLICAS)], x0)
        st.update(window=w, x0=x0)
        wins.append(st)
    doc = {"k": U.K_US, "replicas": U.REPLICAS, "equil_steps": U.EQUIL_STEPS, "prod_steps": U.PROD_STEPS,
           "every": U.EVERY, "windows": wins}
    with open(os.path.join(HERE, "us_windows_44.json"), "w") as f:
        json.dump(doc, f, indent=1)
    for w in wins:
        print(f"x0 {w['x0']:5.1f}: <d> {w['mean_cv']:.3f} +- {w['se_cv']:.3f}, "
              f"mean force {w['mean_force']:+.3f} +- {w['se_force']:.3f}")


if __name__ == "__main__":
    main()
