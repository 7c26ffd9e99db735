"""Time the reference's OpenMP CPU path (cpu_ispa_force, isspa_force.omp.c:11-105)
at a synthetic workload's sizes and parabola parameters.

Benchmark infrastructure only.  Caveats printed with every number: the OpenMP
path is a simplified IS-SPA model (LJ only, parabolic g(r), no electrostatics,
no periodic box) and draws its random numbers from glibc rand(), which
serialises the threads.  One call is one IS-SPA force evaluation of every atom
(nMC points each), counted as one step.
"""
import ctypes as C
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "isspa-force-cuda_gb300"), HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

CAVEAT = ("reference src/isspa_force.omp.c (unmodified): simplified IS-SPA model, LJ only, parabolic g(r), "
          "no electrostatics, no periodic box, glibc rand() serialises the threads; one call = one force "
          "evaluation of every atom = one step")


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "Model name", "cpu model"):
            for line in txt.splitlines():
                if line.startswith(key):
                    return line.split(":", 1)[1].strip()
        import subprocess

        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine()


class RefOmp:
    """cpu_ispa_force bound to one synthetic system (its OpenMP-model parameters)."""

    def __init__(self, system):
        import build_ref

        self.lib = C.CDLL(build_ref.build())
        self.lib.cpu_ispa_force.restype = None
        self.source_sha256 = open(build_ref.STAGED + ".sha256").read().strip() \
            if os.path.exists(build_ref.STAGED + ".sha256") else None
        s = system
        om = s.omp
        self.n, self.m = int(s.n_atoms), int(s.n_mc)
        self.xyz = np.ascontiguousarray(s.pos[:, :3], np.float32)
        self.f = np.zeros_like(self.xyz)
        self.ityp = np.ascontiguousarray(s.lj_type, np.int32)
        self.arrs = [np.ascontiguousarray(om[k], np.float32) for k in ("w", "x0", "g0", "gr2", "alpha", "lj_A", "lj_B")]

    def call(self, threads: int):
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        self.f[:] = 0
        self.lib.cpu_ispa_force(p(self.xyz), p(self.f), *[p(a) for a in self.arrs], p(self.ityp),
                                C.c_int(self.n), C.c_int(self.m), C.c_int(threads))
        return self.f

    def rate(self, threads: int, budget_s: float, min_calls: int = 1, max_calls: int = 1 << 30):
        """Atom-steps/s over repeated calls (one call per step) for about budget_s."""
        n, t0 = 0, time.perf_counter()
        while n < max_calls:
            self.call(threads)
            n += 1
            if n >= min_calls and time.perf_counter() - t0 >= budget_s:
                break
        dt = time.perf_counter() - t0
        return self.n * n / dt, n, dt


def run(threads=None, budget_s=10.0):
    import isspa_gb300.synth as synth

    r = RefOmp(synth.config_plain(seed=2))
    threads = threads or len(os.sched_getaffinity(0))
    v, n, dt = r.rate(threads, budget_s)
    return {"value": v, "unit": "atom-steps/s (one force call per step)", "threads": threads, "calls": n,
            "seconds": dt, "n_atoms": r.n, "n_mc": r.m, "cpu": cpu_model(), "caveat": CAVEAT,
            "source_sha256": r.source_sha256}


if __name__ == "__main__":
    print(json.dumps(run(int(sys.argv[1]) if len(sys.argv) > 1 else None)))
