"""Build recipe of libisspa_gb300.so (sm_103a) and the drop-in executable.

Each translation unit is compiled by nvcc in parallel and linked into one
shared library next to this file; nothing is installed.  Host code carries no
architecture-specific flags so the same sources build on x86-64 and aarch64.
Objects are kept per host architecture (_build/<machine>/) and recompiled only
when their source or a header changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build", platform.machine() or "host")
STAMP = os.path.join(BUILD, "linked")  # the library beside this file was linked from these objects
LIB = os.path.join(HERE, "libisspa_gb300.so")
EXE = os.path.join(HERE, "total_force_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["engine.cu", "k_isspa.cu", "k_md.cu", "k_nblist.cu", "k_adjoint.cu", "k_energy.cu", "k_noalloc.cu",
           "io.cpp"]


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


def _obj(src: str) -> str:
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".o")


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "isspa_gb300.h"))
    units = SOURCES + ["main_total_force.cpp"]
    srcs = [os.path.join(CSRC, s) for s in units]
    fresh = os.path.exists(STAMP) and not _stale(STAMP, srcs + headers)
    if not force and fresh and not _stale(LIB, [STAMP]) and not _stale(EXE, [STAMP]):
        return LIB
    todo = [s for s in units if force or _stale(_obj(s), [os.path.join(CSRC, s)] + headers)]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        for f in [ex.submit(_compile, s, verbose) for s in todo]:
            f.result()
    objs = [_obj(s) for s in units]
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
    with open(STAMP, "w") as f:
        f.write(platform.machine() + "\n")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
