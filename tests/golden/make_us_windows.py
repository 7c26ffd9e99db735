"""Regenerate tests/golden/us_windows_44.json: oracle umbrella-window statistics.

Runs the FP64 oracle MD of the four 44-atom umbrella windows of
tests/us_harness.py (IS-SPA, nonbond, bonded, COM restraint k = 10 at
x0 = 6, 8, 10, 12 A; leapfrog + Andersen at 298 K; Philox window index =
window number, as in a batched engine) for EQUIL_STEPS + PROD_STEPS steps and
stores the block-averaged CV and mean restraint force of the production part.
The GPU test compares its own run of the same windows against these numbers
(mean forces within 2 standard errors).  Takes ~10 minutes on 4 cores:

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


def _run(w):
    import us_harness as U

    s = U.window_system(U.X0S[w])
    cv = U.oracle_cv_series(s, U.EQUIL_STEPS + U.PROD_STEPS, U.EVERY, window=w)
    prod = cv[U.EQUIL_STEPS // U.EVERY:]
    out = U.mean_force_stats(prod, U.X0S[w])
    out.update(window=w, x0=U.X0S[w], n_samples=len(prod))
    return out


def main():
    import us_harness as U

    with mp.get_context("spawn").Pool(len(U.X0S)) as pool:
        wins = pool.map(_run, range(len(U.X0S)))
    doc = {"k": U.K_US, "equil_steps": U.EQUIL_STEPS, "prod_steps": U.PROD_STEPS, "every": U.EVERY,
           "n_blocks": U.N_BLOCKS, "windows": wins}
    with open(os.path.join(HERE, "us_windows_44.json"), "w") as f:
        json.dump(doc, f, indent=1)
    for w in wins:
        print(f"x0 {w['x0']:5.1f}: <d> {w['mean_cv']:.3f} +- {w['se_cv']:.3f}, "
              f"mean force {w['mean_force']:+.3f} +- {w['se_force']:.3f}")


if __name__ == "__main__":
    main()
