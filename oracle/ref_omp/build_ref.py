"""Build the reference's own CPU and CUDA code paths as checkers / CPU baseline.

Test and benchmark infrastructure only: the engine never links any of it.

Where a reference checkout is present (the ISSPA_REFERENCE environment
variable, else a checkout named `reference` beside this repository) the files
below are staged, byte for byte, into oracle/_ref/src/ with their SHA-256.
oracle/_ref/ is git-ignored (nothing of it is committed) but travels with the
working tree, so a machine without the checkout - the GPU host - compiles the
same unmodified sources there.  Every output goes to oracle/_ref/ only.

  * CPU: src/isspa_force.omp.c, compiled unmodified with its `main` renamed so
    that `cpu_ispa_force` (isspa_force.omp.c:11-105) can be called through
    ctypes:  gcc -O3 -fopenmp -fPIC -shared -Dmain=ref_omp_main ... -lm
  * CUDA: src/isspa_force_cuda.cu and the headers it includes, compiled into
    oracle/ref_cuda/ref_isspa_harness.cu (which #includes the file unmodified
    and runs its field and force kernels on given MC points) with the
    reference's own nvcc flags (-use_fast_math -lineinfo, src/Makefile:1) for
    sm_103a; needs nvcc, and runs only on a GPU.
"""
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
REPO = os.path.dirname(ORACLE)
OUT_DIR = os.path.join(ORACLE, "_ref")
SRC_DIR = os.path.join(OUT_DIR, "src")
STAGED = os.path.join(SRC_DIR, "isspa_force.omp.c")
LIB = os.path.join(OUT_DIR, "libref_omp.so")
HARNESS_SRC = os.path.join(ORACLE, "ref_cuda", "ref_isspa_harness.cu")
HARNESS = os.path.join(OUT_DIR, "ref_isspa_harness")
OMP_FILES = ["isspa_force.omp.c"]
CUDA_FILES = ["isspa_force_cuda.cu", "isspa_force_cuda.h", "isspa_class.h", "constants.h",
              "cuda_vector_routines.h", "init_rand.cuh"]


def checkout():
    """Path of a reference checkout holding src/isspa_force.omp.c, or None."""
    cands = [os.environ.get("ISSPA_REFERENCE", ""), os.path.join(os.path.dirname(REPO), "reference")]
    for c in cands:
        if c and os.path.exists(os.path.join(c, "src", OMP_FILES[0])):
            return c
    return None


def sha256(path: str) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def stage() -> str:
    """Copies the unmodified sources into oracle/_ref/src/ when a checkout is
    present; returns the staged OpenMP file (which may predate this call)."""
    ref = checkout()
    if ref is not None:
        os.makedirs(SRC_DIR, exist_ok=True)
        for name in OMP_FILES + CUDA_FILES:
            src = os.path.join(ref, "src", name)
            dst = os.path.join(SRC_DIR, name)
            if not os.path.exists(src):
                continue
            if not os.path.exists(dst) or sha256(dst) != sha256(src):
                shutil.copyfile(src, dst)
                with open(dst + ".sha256", "w") as f:
                    f.write(sha256(src) + "\n")
    if not os.path.exists(STAGED):
        raise FileNotFoundError("no reference checkout and no staged copy of src/isspa_force.omp.c")
    return STAGED


def build() -> str:
    src = stage()
    os.makedirs(OUT_DIR, exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        tmp = LIB + ".tmp"
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-Dmain=ref_omp_main",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def build_cuda(fast_math: bool = True) -> str:
    """The reference CUDA harness, with the reference's -use_fast_math (as its
    Makefile builds) or without it (IEEE division, square root and tanh: a
    diagnostic of what the flag contributes); raises when the staged sources
    or nvcc are missing."""
    stage()
    for name in CUDA_FILES:
        if not os.path.exists(os.path.join(SRC_DIR, name)):
            raise FileNotFoundError("reference CUDA source not staged: src/" + name)
    out = HARNESS if fast_math else HARNESS + "_ieee"
    deps = [HARNESS_SRC] + [os.path.join(SRC_DIR, n) for n in CUDA_FILES]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = out + ".tmp"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
                           "-Wno-deprecated-gpu-targets", "-Wno-deprecated-declarations", "-I", SRC_DIR]
                          + (["-use_fast_math"] if fast_math else []) + ["-o", tmp, HARNESS_SRC])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build())
    print(build_cuda())
    print(build_cuda(fast_math=False))
