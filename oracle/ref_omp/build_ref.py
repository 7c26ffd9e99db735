"""Build the reference's OpenMP CPU path (cpu_ispa_force) as a CPU baseline.

Test and benchmark infrastructure only: the engine never links it.

The reference file src/isspa_force.omp.c is compiled unmodified, with its
`main` renamed so that `cpu_ispa_force` (isspa_force.omp.c:11-105) can be
called through ctypes:
    gcc -O3 -fopenmp -fPIC -shared -Dmain=ref_omp_main isspa_force.omp.c -lm
Where a reference checkout is present (the ISSPA_REFERENCE environment
variable, else a checkout named `reference` beside this repository) the file
is first staged, byte for byte, into oracle/_ref/src/ with its SHA-256.
oracle/_ref/ is git-ignored (nothing of it is committed) but travels with the
working tree, so a machine without the checkout - the GPU host - compiles the
same unmodified source there.  Every output goes to oracle/_ref/ only.
"""
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT_DIR = os.path.join(os.path.dirname(HERE), "_ref")
STAGED = os.path.join(OUT_DIR, "src", "isspa_force.omp.c")
LIB = os.path.join(OUT_DIR, "libref_omp.so")
REL_SRC = os.path.join("src", "isspa_force.omp.c")


def checkout():
    """Path of a reference checkout holding src/isspa_force.omp.c, or None."""
    cands = [os.environ.get("ISSPA_REFERENCE", ""), os.path.join(os.path.dirname(REPO), "reference")]
    for c in cands:
        if c and os.path.exists(os.path.join(c, REL_SRC)):
            return c
    return None


def sha256(path: str) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def stage() -> str:
    """Copies the unmodified source into oracle/_ref/src/ when a checkout is
    present; returns the staged path (which may predate this call)."""
    ref = checkout()
    if ref is not None:
        src = os.path.join(ref, REL_SRC)
        if not os.path.exists(STAGED) or sha256(STAGED) != sha256(src):
            os.makedirs(os.path.dirname(STAGED), exist_ok=True)
            shutil.copyfile(src, STAGED)
            with open(STAGED + ".sha256", "w") as f:
                f.write(sha256(src) + "\n")
    if not os.path.exists(STAGED):
        raise FileNotFoundError("no reference checkout and no staged copy of " + REL_SRC)
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


if __name__ == "__main__":
    print(build())
