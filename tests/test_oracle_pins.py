"""The oracle against the reference's own golden vectors (CPU only).

* Philox4x32-10 against the Random123 known-answer vectors.
* Nonbond sub-terms against the reference's FP64 golden force files for the
  ADI2 dimer (timing_tests/ADI2/10000MC/compare/ADI2.multi.frc.*.dat).
* IS-SPA force branches against the reference's 1000-seed per-term frame
  averages at nMC = 1000 (ISSPA_force_{Csolv,LJsolv,Csolv_CDD}_10000.xyz),
  as a z-test of the means.
* The reference's step-0 total force of one run (timing_tests/ADI2/10000MC/
  ADI.2.forces.xyz: bonded + IS-SPA + nonbond, total_force_cuda.cpp:109-121)
  against the oracle's bonded and nonbond terms plus its IS-SPA distribution.
"""
import math
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def nrel(a, b):
    return float(np.abs(np.asarray(a) - b).max() / np.abs(b).max())


def test_philox_known_answers():
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, out in kat:
        assert tuple(O.philox(ctr, key)) == out


@pytest.mark.parametrize("x", [1e-6, 1e-3, 0.1, 0.2499, 0.25, 0.5, 1.0, 3.0, 7.0, 30.0])
def test_langevin_against_closed_form_high_precision(x):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 50  # the reference's closed forms, evaluated without cancellation error
    X = mp.mpf(x)
    c = mp.coth(X)
    c1 = c - 1 / X
    c2 = 1 - 2 * c1 / X
    c3 = c - 3 * c2 / X
    ref = [float(c1), float(1.5 * c2 - 0.5), float(2.5 * c3 - 1.5 * c1)]
    got = O.langevin(x)
    for g, r in zip(got, ref):
        assert abs(g - r) <= 1e-12 * abs(r) + 1e-300


def test_langevin_small_field_limits():
    p1, p2, p3 = O.langevin(1e-4)
    assert math.isclose(p1, 1e-4 / 3, rel_tol=1e-8)
    assert math.isclose(p2, 1e-8 / 15, rel_tol=1e-8)
    assert math.isclose(p3, 1e-12 / 105, rel_tol=1e-8)
    assert O.langevin(0.0) == [0.0, 0.0, 0.0]


@pytest.mark.parametrize("term,mask,tol", [("LJsolu", O.NB_LJ, 2e-5), ("Csolu", O.NB_COUL, 5e-6),
                                           ("Csolv_pair", O.NB_CORR, 5e-6)])
def test_nonbond_terms_match_fp64_golden(adi2, term, mask, tol):
    f = O.Oracle(adi2).nonbond(mask)
    gold = np.loadtxt(os.path.join(GOLDEN, f"ADI2.multi.frc.{term}.dat"))
    # the golden files were written at the rst7 coordinates
    assert np.allclose(gold[:, :3], adi2.pos[:, :3], atol=1e-5)
    assert nrel(f, gold[:, 3:]) < tol


def test_nonbond_single_frame_reference_output(adi2):
    """The reference's own single-frame per-term outputs (Csolu, LJsolu, Csolv_pair)."""
    o = O.Oracle(adi2)
    for term, mask in [("LJsolu", O.NB_LJ), ("Csolu", O.NB_COUL), ("Csolv_pair", O.NB_CORR)]:
        r = np.load(os.path.join(GOLDEN, f"ref_frames_{term}.npz"))
        assert nrel(o.nonbond(mask), r["mean"]) < 2e-5


@pytest.mark.slow
def test_isspa_terms_match_reference_frame_averages(adi2):
    o = O.Oracle(adi2)
    nf = 150
    acc = {1: [], 2: [], 4: []}
    for k in range(nf):
        pts = o.mc_points(seed=5000 + k, step=0)
        fld = o.field(pts)
        for m in acc:
            acc[m].append(o.isspa_force(pts, fld, m))
    for m, name in [(O.MULTIPOLE, "Csolv"), (O.LJ_TAB, "LJsolv"), (O.CDD, "Csolv_CDD")]:
        a = np.array(acc[m])
        mean, sem = a.mean(0), a.std(0, ddof=1) / np.sqrt(nf)
        r = np.load(os.path.join(GOLDEN, f"ref_frames_{name}.npz"))
        assert int(r["n_frames"]) == 1000
        z = (mean - r["mean"]) / np.sqrt(sem ** 2 + r["sem"] ** 2)
        # components of a frame share one point set: bound rms and max of z
        assert np.sqrt(np.mean(z ** 2)) < 1.6, name
        assert np.abs(z).max() < 5.0, name


def test_oracle_field_invariants(adi2):
    s = adi2.copy()
    s.n_mc = 50
    o = O.Oracle(s)
    pts = o.mc_points(seed=1, step=0)
    # points lie in the ball r^2 < 0.99 rmax^2 around their owner
    owner = np.repeat(np.arange(s.n_atoms), s.n_mc)
    d = np.linalg.norm(pts - s.pos[owner, :3], axis=1)
    assert np.all(d < np.sqrt(0.99) * s.rmax[s.isspa_type[owner]] + 1e-4)
    w, n, E, E0 = o.field(pts)
    assert np.all(n >= 1)  # the owner is always in range
    assert np.all(w >= 0)
    # a point's counts depend only on geometry: same points, same counts
    assert np.array_equal(n, o.field(pts)[1])


def test_oracle_determinism_and_step_keying(adi2):
    s = adi2.copy()
    s.n_mc = 20
    o = O.Oracle(s)
    a = o.mc_points(seed=7, step=3)
    assert np.array_equal(a, o.mc_points(seed=7, step=3))
    assert not np.array_equal(a, o.mc_points(seed=7, step=4))
    assert not np.array_equal(a, o.mc_points(seed=8, step=3))
    assert not np.array_equal(a, o.mc_points(seed=7, step=3, window=1))


def _xyz_rows(path, n=44):
    with open(path) as f:
        lines = f.read().split("\n")[2:2 + n]
    return np.array([[float(v) for v in line.split()[1:]] for line in lines])


def test_step0_total_force_against_reference_output(adi2):
    """One run of the reference (nMC 1000, 200 A box, its curand point stream)
    wrote the step-0 total force (bonded, IS-SPA and nonbond) and, in its
    IS-SPA output file, the tabulated mean-LJ term of the same MC sample
    (that build's study of the LJsolv branch).  The total minus the oracle's
    bonded and nonbond forces minus that recorded term is the run's multipole
    + CDD sample: compared per component with the oracle's mean and spread
    over 40 Philox samples at the same nMC (z-scores; the spread is ~0.3 % of
    the total force, so a 1 % error in the bonded terms gives rms z ~ 25).
    The recorded tabulated-LJ term is checked the same way."""
    tot = _xyz_rows(os.path.join(GOLDEN, "ADI.2.forces.xyz"))
    rec = _xyz_rows(os.path.join(GOLDEN, "ADI2.ISSPA_force.step0.xyz"))
    assert np.allclose(rec[:, :3], adi2.pos[:, :3], atol=1e-5)
    assert adi2.n_mc == 1000 and adi2.box == 200.0
    o = O.Oracle(adi2)
    det = o.bonded() + o.nonbond(O.NB_LJ | O.NB_COUL | O.NB_CORR)
    mp, lj = [], []
    for k in range(40):
        pts = o.mc_points(seed=9000 + k, step=0)
        fld = o.field(pts)
        mp.append(o.isspa_force(pts, fld, O.MULTIPOLE | O.CDD))
        lj.append(o.isspa_force(pts, fld, O.LJ_TAB))
    for label, sample, dist in [("multipole + CDD", tot - det - rec[:, 3:], np.array(mp)),
                                ("tabulated LJ", rec[:, 3:], np.array(lj))]:
        sd = dist.std(0, ddof=1) * np.sqrt(1.0 + 1.0 / len(dist))
        z = (sample - dist.mean(0)) / sd
        rms, mx = float(np.sqrt(np.mean(z ** 2))), float(np.abs(z).max())
        print(f"{label}: rms z {rms:.2f}, max |z| {mx:.2f} over {z.size} components")
        assert rms < 1.5, label
        assert mx < 4.5, label
