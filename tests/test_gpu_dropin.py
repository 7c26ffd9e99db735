"""The drop-in executable (total_force_gb300) on the reference's own inputs.

Runs the ADI2 dimer with umbrella sampling through the same config / prmtop /
isspatop / rst7 / US files total_force_cuda.x reads, and checks the output
files' formats (atom_class.cpp:248-328, us_class.cpp:132) and contents
against the engine driven through the C ABI.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import isspa_gb300 as ig

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
EXE = os.path.join(ROOT, "isspa-force-cuda_gb300", "total_force_gb300")


def read_xyz_frames(path, ncol):
    frames, cur = [], []
    with open(path) as f:
        lines = f.read().splitlines()
    k = 0
    while k < len(lines):
        n = int(lines[k])
        assert int(lines[k + 1]) == n
        rows = [ln.split() for ln in lines[k + 2:k + 2 + n]]
        assert all(r[0] == "C" and len(r) == ncol + 1 for r in rows)
        frames.append(np.array([[float(x) for x in r[1:]] for r in rows]))
        k += 2 + n
    return frames


@pytest.fixture()
def rundir(tmp_path):
    for f in ["ADI2.prmtop", "ADI2.isspatop", "ADI2.rst7"]:
        shutil.copy(os.path.join(GOLDEN, f), tmp_path / f)
    (tmp_path / "us.cfg").write_text(open(os.path.join(GOLDEN, "ADI2.us")).read().replace("XXX", "10.0"))
    cfg = open(os.path.join(GOLDEN, "adi2_config.txt")).read()
    cfg = cfg.replace("nMC = 1000", "nMC = 50").replace("nSteps = 1", "nSteps = 25") \
             .replace("deltaWrite = 100", "deltaWrite = 10").replace("US = 0", "US = 1\nusCfgFile = us.cfg\npnu = 0.02")
    (tmp_path / "config.txt").write_text(cfg)
    return tmp_path


def test_dropin_outputs(rundir):
    r = subprocess.run([EXE, "config.txt"], cwd=rundir, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Average ns/day" in r.stdout
    forces = read_xyz_frames(rundir / "ADI2.forces.xyz", 3)
    pos = read_xyz_frames(rundir / "ADI2.positions.xyz", 3)
    vel = read_xyz_frames(rundir / "ADI2.velocities.xyz", 3)
    isf = read_xyz_frames(rundir / "ISSPA_force.xyz", 6)
    assert len(forces) == len(pos) == len(vel) == len(isf) == 3  # steps 0, 10, 20
    # CV file "%8d  %8.3f" at the output steps
    cv = [ln for ln in open(rundir / "ADI2.equil.window.10.0.dat").read().splitlines()]
    assert [int(c.split()[0]) for c in cv] == [0, 10, 20]
    assert all(len(c) == 18 for c in cv)
    # restart files: title, atom count, 6F12.7 rows, box line
    rst = open(rundir / "ADI2.positions.rst").read().splitlines()
    assert rst[0] == "Restart Positions from ISSPA CUDA Code" and int(rst[1]) == 44
    assert len(rst) == 2 + 22 + 1 and len(rst[2]) == 72
    assert rst[-1].split() == ["200.0000000"] * 3 + ["90.0000000"] * 3 and len(rst[-1]) == 72
    # frame 0 equals the engine's step-0 forces on the same inputs
    s = ig.System.from_config(str(rundir / "config.txt"))
    eng = ig.Engine(s)
    f0 = eng.compute_forces()
    assert np.allclose(forces[0], f0, atol=2e-6 * np.abs(f0).max() + 1.5e-6)
    assert np.allclose(pos[0], s.pos[:, :3], atol=1.5e-6)
    com, cvv = eng.us_com()
    assert abs(float(cv[0].split()[1]) - cvv[0]) < 1e-3


def test_dropin_long_run_autotunes(rundir):
    """A run of 1000 steps or more times the launch-shape candidates first and
    reports the choice; the run completes with its CV file intact."""
    cfg = (rundir / "config.txt").read_text()
    (rundir / "config.txt").write_text(cfg.replace("nSteps = 25", "nSteps = 2000").replace("deltaWrite = 10",
                                                                                              "deltaWrite = 500"))
    r = subprocess.run([EXE, "config.txt"], cwd=rundir, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "launch shapes: field split" in r.stdout
    cv = [ln for ln in (rundir / "ADI2.equil.window.10.0.dat").read_text().splitlines() if ln.strip()]
    assert [int(c.split()[0]) for c in cv] == [0, 500, 1000, 1500]
    pos = read_xyz_frames(rundir / "ADI2.positions.xyz", 3)
    assert len(pos) == 4
    assert all(np.all(np.isfinite(p)) for p in pos)
