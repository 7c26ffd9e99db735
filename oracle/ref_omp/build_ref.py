"""Build the reference's OpenMP CPU path as a checker / CPU baseline.

Compiles src/isspa_force.omp.c of the reference checkout, unmodified, with its
`main` renamed so that `cpu_ispa_force` can be called from Python:
    gcc -O3 -fopenmp -fPIC -shared -Dmain=ref_omp_main isspa_force.omp.c
Output goes to oracle/_ref/ only (git-ignored).  The reference tree exists only
where the reference is checked out, so this builds nowhere else.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(os.path.dirname(HERE), "_ref")
LIB = os.path.join(OUT_DIR, "libref_omp.so")
REF = os.environ.get("ISSPA_REFERENCE", "/root/reference")


def build() -> str:
    src = os.path.join(REF, "src", "isspa_force.omp.c")
    if not os.path.exists(src):
        raise FileNotFoundError(src)
    os.makedirs(OUT_DIR, exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-Dmain=ref_omp_main",
                               "-o", LIB, src, "-lm"])
    return LIB


if __name__ == "__main__":
    print(build())
