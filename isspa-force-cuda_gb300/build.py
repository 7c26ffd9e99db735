"""Build recipe of libisspa_gb300.so (sm_103a) and the drop-in executable.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library next to this file; nothing is installed.  Host code carries no
architecture-specific flags so the same sources build on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libisspa_gb300.so")
EXE = os.path.join(HERE, "total_force_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "k_isspa.cu", "k_md.cu", "k_adjoint.cu", "k_energy.cu", "k_noalloc.cu", "io.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")
    return cand


def _flags():
    # -ftz=true: no denormal operands occur on any decision path (distances,
    # bins, table weights are all far from 1e-38), and flushing lets the
    # compiler drop the denormal fix-ups of rsqrt/sqrt/division.
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC", "-I", INCLUDE,
                   "-I", CSRC, "--expt-relaxed-constexpr"]


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    cmd = [nvcc()] + _flags() + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu"] + cmd[1:]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "isspa_gb300.h"))
    srcs = [os.path.join(CSRC, s) for s in SOURCES] + [os.path.join(CSRC, "main_total_force.cpp")]
    if not force and not _stale(LIB, srcs + headers) and not _stale(EXE, srcs + headers):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        futs = [ex.submit(_compile, s, verbose) for s in SOURCES + ["main_total_force.cpp"]]
        objs = [f.result() for f in futs]
    lib_objs, main_obj = objs[:-1], objs[-1]
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + lib_objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    r = subprocess.run([nvcc()] + ARCH + ["-o", EXE, main_obj, "-L", HERE, "-lisspa_gb300",
                        "-Xlinker", "-rpath,$ORIGIN"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of the drop-in executable failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
