"""Precision workload: 256 chains of 64 atoms (16 384 atoms), 120 A box,
nMC = 100 (1.64 M MC points), charges +-0.8 e.

A full FP64 oracle pass at this size is too slow for a test, so each stage is
checked on samples against the FP64 oracle:
  * the MC points of the whole system: bit-identical;
  * the field pass at 512 sampled points (all 16 384 atoms each);
  * the IS-SPA force on 64 sampled atoms from all 1.64 M points, given the
    engine's own fields (isolates the force pass);
  * the nonbond force on the same atoms against all partners.
"""
import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from parity import check_force

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

FIELD_TOL = 2e-5  # per-point fields; forces: tests/parity.py


def nrel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="module")
def big():
    s = ig.synth.config_precision(seed=3)
    assert s.n_atoms == 16384 and s.n_mc == 100
    return s


def test_precision_workload_against_fp64_oracle_samples(big):
    s = big
    eng = ig.Engine(s)
    rng = np.random.default_rng(0)
    o = O.Oracle(s)
    xyz, w, n, E, E0 = eng.point_fields()
    pts = o.mc_points(seed=s.seed, step=0)
    assert np.array_equal(xyz, pts)
    idx = np.sort(rng.choice(len(pts), 512, replace=False))
    wo, no, Eo, E0o = o.field_at(pts, idx)
    assert np.array_equal(n[idx], no)
    errs = {"w": nrel(w[idx], wo), "E": nrel(E[idx], Eo), "E0": nrel(E0[idx], E0o)}
    atoms = np.sort(rng.choice(s.n_atoms, 64, replace=False))
    eng.zero_forces()
    eng.isspa_force()
    f_is = eng.forces()
    ref = o.isspa_force_atoms(pts, (w.astype(np.float64), n, E.astype(np.float64), E0.astype(np.float64)), atoms)
    check_force(f_is[atoms], ref, "16 384 atoms, IS-SPA force on 64 atoms (engine's fields)")
    eng.zero_forces()
    eng.nonbond_force()
    check_force(eng.forces()[atoms], o.nonbond_atoms(atoms), "16 384 atoms, nonbond on 64 atoms")
    print("normwise relative field errors vs FP64 oracle:", errs)
    for k, v in errs.items():
        assert v < FIELD_TOL, (k, v)
    assert eng.device_status() == 0


def test_precision_workload_voted_loops_bit_identical(big):
    """At this size almost every group of four atoms (field pass) or points
    (force pass) is out of range for all lanes, the case the warp-voted loops
    speed up; with the same split and chunks they reproduce the per-pair loops'
    IS-SPA force of all 16 384 atoms bit for bit."""
    out = []
    for vote in (0, 1):
        eng = ig.Engine(big, field_split=1, force_chunk=512, force_tail_chunk=64, field_vote=vote, force_vote=vote)
        sh = eng.shapes()
        assert sh["field_vote"] == vote and sh["force_vote"] == vote
        eng.zero_forces()
        eng.isspa_force()
        out.append(eng.forces())
        assert eng.device_status() == 0
        eng.close()
    assert np.array_equal(out[0], out[1])
