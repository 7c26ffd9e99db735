"""Runs the reference's own IS-SPA field and force CUDA kernels on given MC
points (oracle/ref_cuda/ref_isspa_harness.cu, built by
oracle/ref_omp/build_ref.build_cuda from the staged, unmodified reference
source).  Test infrastructure only; needs a GPU."""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "ref_omp"))


def harness(fast_math: bool = True) -> str:
    import build_ref

    return build_ref.build_cuda(fast_math)


def forces(system, pts, runs: int = 5, fast_math: bool = True) -> np.ndarray:
    """IS-SPA force of every atom ([runs][N][3]) from the reference kernels on
    the points `pts` ([N*nMC][3]); each run starts from zeroed accumulators
    (the reference's float atomics make runs differ at rounding level).
    fast_math=False uses the build without -use_fast_math."""
    s = system
    n, m = int(s.n_atoms), int(s.n_mc)
    nt = len(s.rmax)
    g = np.ascontiguousarray(s.g_table, np.float32)
    e = np.ascontiguousarray(s.e_table, np.float32)
    f = np.ascontiguousarray(s.f_table, np.float32)
    hdr = np.array([n, m, nt, f.shape[1], g.shape[1], e.shape[1], runs, 0], np.int32)
    prm = np.array([s.box, s.f_r0, s.f_dr, s.g_r0, s.g_dr, s.e_r0, s.e_dr], np.float32)
    with tempfile.TemporaryDirectory() as d:
        fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        with open(fin, "wb") as fh:
            for a in (hdr, prm, np.ascontiguousarray(s.pos, np.float32).reshape(n, 4),
                      np.ascontiguousarray(s.isspa_type, np.int32), np.ascontiguousarray(s.rmax, np.float32),
                      np.ascontiguousarray(s.vtot(), np.float32), g, e, f,
                      np.ascontiguousarray(pts, np.float32).reshape(n * m, 3)):
                fh.write(a.tobytes())
        r = subprocess.run([harness(fast_math), fin, fout], capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness exited {r.returncode}: {r.stderr.strip()}")
        out = np.fromfile(fout, np.float32).reshape(runs, n, 4)
    return out[:, :, :3].astype(np.float64)
