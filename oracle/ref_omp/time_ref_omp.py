"""Time the reference's OpenMP CPU path (cpu_ispa_force, isspa_force.omp.c:11-105)
on a synthetic workload's sizes and parabola parameters.

Caveats printed with the number: the OpenMP path is a simplified IS-SPA model
(LJ only, parabolic g(r), no electrostatics, no periodic box) and draws its
random numbers from glibc rand(), which serialises the threads.
"""
import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "isspa-force-cuda_gb300"))
sys.path.insert(0, HERE)


def run(threads=None, budget_s=10.0):
    import build_ref
    import isspa_gb300.synth as synth

    L = C.CDLL(build_ref.build())
    s = synth.config_plain(seed=2)
    om = s.omp
    N, M = s.n_atoms, s.n_mc
    xyz = np.ascontiguousarray(s.pos[:, :3], np.float32)
    f = np.zeros_like(xyz)
    ityp = np.ascontiguousarray(s.lj_type, np.int32)
    arrs = [np.ascontiguousarray(om[k], np.float32) for k in ("w", "x0", "g0", "gr2", "alpha", "lj_A", "lj_B")]
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    threads = threads or len(os.sched_getaffinity(0))
    n, t0 = 0, time.perf_counter()
    while True:
        f[:] = 0
        L.cpu_ispa_force(p(xyz), p(f), *[p(a) for a in arrs], p(ityp), N, M, threads)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": N * n / dt, "unit": "atom-steps/s (one force call per step)", "threads": threads,
            "calls": n, "seconds": dt, "n_atoms": N, "n_mc": M,
            "caveat": "simplified LJ-only IS-SPA model, no PBC/electrostatics, glibc rand() serialised"}


if __name__ == "__main__":
    print(json.dumps(run(int(sys.argv[1]) if len(sys.argv) > 1 else None)))
