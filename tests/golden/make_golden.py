"""Regenerate the golden fixtures of tests/golden from the reference checkout.

Run from the repository root with the reference tree available:
    python tests/golden/make_golden.py /path/to/ISSPA-Force-Cuda

It copies the reference's ADI2 inputs and its FP64 golden force files, and
condenses the reference's 1000-seed per-term frame files into per-atom means
and standard errors (the criterion of timing_tests/ADI2/10000MC/compare/
compare.py:27-48 is the frame average).  Nothing here runs at test time.
"""
from __future__ import annotations

import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TERMS = ["LJsolu", "LJsolv", "Csolu", "Csolv", "Csolv_pair", "Csolv_CDD"]


def frames(path):
    """Per-atom force frames of an ISSPA_force*.xyz file (7 columns per row)."""
    rows = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) == 7:
                rows.append([float(x) for x in t[1:7]])
    a = np.array(rows)
    return a.reshape(-1, 44, 6)


def main(ref):
    adi = os.path.join(ref, "timing_tests", "ADI2")
    cmp_dir = os.path.join(adi, "10000MC", "compare")
    for f in ["ADI2.prmtop", "ADI2.isspatop", "ADI2.rst7"]:
        shutil.copy(os.path.join(adi, f), os.path.join(HERE, f))
    for t in TERMS:
        shutil.copy(os.path.join(cmp_dir, f"ADI2.multi.frc.{t}.dat"), os.path.join(HERE, f"ADI2.multi.frc.{t}.dat"))
        a = frames(os.path.join(cmp_dir, f"ISSPA_force_{t}_10000.xyz"))
        mean = a[:, :, 3:].mean(0)
        sem = a[:, :, 3:].std(0, ddof=1) / np.sqrt(len(a)) if len(a) > 1 else np.zeros_like(mean)
        np.savez(os.path.join(HERE, f"ref_frames_{t}.npz"), mean=mean, sem=sem, n_frames=len(a),
                 pos=a[0, :, :3])
    # the umbrella-sampling inputs of one ADI2 window (ADI2_US)
    us = os.path.join(ref, "timing_tests", "ADI2_US")
    shutil.copy(os.path.join(us, "ADI2.us"), os.path.join(HERE, "ADI2.us"))
    # step-0 total forces of the 10000MC run (nMC=1000, seed 8622; curand stream)
    shutil.copy(os.path.join(adi, "10000MC", "ADI.2.forces.xyz"), os.path.join(HERE, "ADI.2.forces.xyz"))
    # the same run's IS-SPA output file: the tabulated-LJ term alone (the last
    # frame of the LJsolv study, ISSPA_force_LJsolv_10000.xyz), same MC sample
    shutil.copy(os.path.join(adi, "10000MC", "ISSPA_force.xyz"), os.path.join(HERE, "ADI2.ISSPA_force.step0.xyz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
