"""GPU parity: every kernel of the step against the CPU oracle, through the C ABI.

Tolerances (FP32 kernels vs the FP64-valued oracle, identical geometric
decisions by construction, except that the field pass may pick a density-table
bin one off at a bin edge, where its interpolation is continuous, when the
density and field tables share one radial grid):
  * MC points, in-range counts: bit-identical;
  * per-point density product, mean field: normwise relative 2e-5;
  * forces of each term: 1e-5 relative, normwise (max |dF| / max |F|) and per
    atom (|dF_i| / |F_i| above a floor), as tests/parity.py states;
  * integrator: 1e-5 relative on positions and velocities.
"""
import os

import numpy as np
import pytest

import isspa_gb300 as ig
import oracle as O
from parity import check_force

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELD_TOL = 2e-5  # per-point fields, normwise


def nrel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def with_mc(s, n_mc):
    s = s.copy()
    s.n_mc = n_mc
    return s


@pytest.fixture(scope="module")
def adi2_100(adi2):
    return with_mc(adi2, 100)


@pytest.fixture(scope="module")
def synth_small():
    return ig.synth.config_small(seed=3)


@pytest.fixture(scope="module")
def synth_medium():
    # 12 chains = 264 atoms in a 34 A box, nMC 20: dense enough for min-image and all branches
    ff = ig.synth.forcefield(n_mc=20)
    return ig.synth.make_system(12, 22, 34.0, 20, seed=21, ff=ff)


def test_mc_points_bit_identical(adi2_100):
    eng = ig.Engine(adi2_100)
    xyz, w, n, E, E0 = eng.point_fields()
    o = O.Oracle(adi2_100)
    ref = o.mc_points(seed=adi2_100.seed, step=0)
    assert np.array_equal(xyz, ref)
    eng.set_step(17)
    xyz17 = eng.point_fields()[0]
    assert np.array_equal(xyz17, o.mc_points(seed=adi2_100.seed, step=17))
    assert not np.array_equal(xyz17, xyz)


@pytest.mark.parametrize("split", [1, 2, 4, 8, 16])
def test_field_vote_loop_bit_identical(synth_medium, split):
    """The warp-voted atom loop of the field pass, and atom rounds staged by
    bulk copies (TMA) instead of thread loads, give the per-pair loop's forces
    and trajectory bit for bit, at every atom-loop split."""
    out = []
    for vote, tma in ((0, 0), (1, 0), (0, 1), (1, 1)):
        eng = ig.Engine(synth_medium, field_split=split, field_vote=vote, field_tma=tma)
        sh = eng.shapes()
        assert sh["field_vote"] == vote and sh["field_split"] == split and sh["field_tma"] == tma
        eng.zero_forces()
        eng.isspa_force()
        f = eng.forces()
        eng.step(5)
        out.append((f, eng.positions()))
        assert eng.device_status() == 0
    for f, p in out[1:]:
        assert np.array_equal(f, out[0][0])
        assert np.array_equal(p, out[0][1])


def test_field_tma_batched_windows_bit_identical():
    """Bulk-copied atom rounds over windows of odd sizes and odd first atoms
    (1, 2, 44, 23 and 1100 atoms) give the plain staging's forces bit for bit."""
    ff = ig.synth.forcefield(n_mc=20)
    wins = [ig.synth.make_system(c, ln, 40.0, 20, seed=40 + k, ff=ff)
            for k, (c, ln) in enumerate([(1, 1), (2, 1), (2, 22), (1, 23), (50, 22)])]
    out = []
    for tma in (0, 1):
        eng = ig.Engine(wins, field_tma=tma)
        eng.zero_forces()
        eng.isspa_force()
        out.append(eng.forces())
        assert eng.device_status() == 0
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("which", ["adi2", "medium", "medium-two-grids"])
def test_field_matches_oracle(which, adi2_100, synth_medium):
    s = adi2_100 if which == "adi2" else synth_medium
    if which == "medium-two-grids":
        # field table on its own radial grid: its interpolation jumps at the
        # density bin's edges, so the bin must be the oracle's exactly
        s = s.copy()
        s.e_r0 = float(np.float32(s.e_r0 + 0.03))
        s.e_dr = float(np.float32(s.e_dr * 1.1))
    eng = ig.Engine(s)
    xyz, w, n, E, E0 = eng.point_fields()
    o = O.Oracle(s)
    w_o, n_o, E_o, E0_o = o.field(xyz)
    assert np.array_equal(n, n_o)
    assert nrel(w, w_o) < FIELD_TOL
    assert nrel(E, E_o) < FIELD_TOL
    assert nrel(E0, E0_o) < FIELD_TOL


@pytest.mark.parametrize("terms", [1, 2, 4, 7])
@pytest.mark.parametrize("which", ["adi2", "medium"])
def test_isspa_force_terms_match_oracle(terms, which, adi2_100, synth_medium):
    s = adi2_100 if which == "adi2" else synth_medium
    eng = ig.Engine(s, isspa_terms=terms)
    eng.zero_forces()
    eng.isspa_force()
    f = eng.forces()
    o = O.Oracle(s)
    pts = o.mc_points(seed=s.seed, step=0)
    ref = o.isspa_force(pts, terms=terms)
    check_force(f, ref, f"isspa terms={terms} {which}")


@pytest.mark.parametrize("terms", [1, 2, 4, 7])
def test_nonbond_matches_oracle_and_golden(terms, adi2):
    eng = ig.Engine(with_mc(adi2, 10), nonbond_terms=terms)
    eng.zero_forces()
    eng.nonbond_force()
    f = eng.forces()
    ref = O.Oracle(adi2).nonbond(terms)
    check_force(f, ref, f"nonbond terms={terms} adi2")
    names = {1: "LJsolu", 2: "Csolu", 4: "Csolv_pair"}
    if terms in names:
        gold = np.loadtxt(os.path.join(GOLDEN, f"ADI2.multi.frc.{names[terms]}.dat"))[:, 3:]
        assert nrel(f, gold) < 2e-5  # reference CUDA's own agreement: 9e-6, 2e-6, 3e-6


def test_nonbond_medium(synth_medium):
    eng = ig.Engine(synth_medium)
    eng.zero_forces()
    eng.nonbond_force()
    check_force(eng.forces(), O.Oracle(synth_medium).nonbond(7), "nonbond medium")


def test_nonbond_partner_chunks_bit_identical(synth_medium):
    """Partners per nonbond work item (128..all, ragged last items) move no
    bit of the force: the per-stage sums start at the same partners."""
    out = []
    for chunk in (128, 256, 384, 1024):
        eng = ig.Engine(synth_medium, nonbond_chunk=chunk)
        assert eng.shapes()["nonbond_partners_per_item"] == chunk
        eng.zero_forces()
        eng.nonbond_force()
        out.append(eng.forces())
        eng.close()
    for f in out[1:]:
        assert np.array_equal(f, out[0])
    check_force(out[0], O.Oracle(synth_medium).nonbond(7), "nonbond medium, 128-partner items")


@pytest.mark.parametrize("which", ["adi2", "medium"])
def test_bonded_matches_oracle(which, adi2, synth_medium):
    s = with_mc(adi2, 10) if which == "adi2" else synth_medium
    eng = ig.Engine(s)
    eng.zero_forces()
    eng.bond_force()
    eng.angle_force()
    eng.dih_force()
    check_force(eng.forces(), O.Oracle(s).bonded(), f"bonded {which}")


def test_umbrella_matches_oracle(adi2):
    s = with_mc(adi2, 10)
    s.us_on = 1
    s.bias_list = np.array([(i, 0) for i in range(22)] + [(22 + i, 1) for i in range(22)], np.int32)
    s.us_k, s.us_x0 = 20.0, 10.0
    eng = ig.Engine(s)
    eng.zero_forces()
    eng.us_force()
    f = eng.forces()
    ref, com = O.Oracle(s).us()
    assert nrel(f, ref) < 1e-6
    gcom, cv = eng.us_com()
    assert np.allclose(gcom[0], com, rtol=1e-12, atol=1e-9)
    d = com[0] - com[1]
    assert abs(cv[0] - np.linalg.norm(d)) < 1e-9


def test_leapfrog_matches_oracle(synth_medium):
    s = synth_medium.copy()
    s.pnu = 0.3  # exercise both branches
    eng = ig.Engine(s)
    f = eng.compute_forces().astype(np.float64)
    eng.leapfrog()
    pos, vel = eng.positions(), eng.velocities()
    po, vo, res = O.Oracle(s).leapfrog(f, seed=s.seed, step=0)
    assert 0 < res.sum() < len(res)
    assert np.allclose(pos[:, :3], po, rtol=0, atol=2e-5 * s.box)
    assert nrel(vel[:, :3], vo) < 1e-5
    assert eng.get_step() == 1


def test_full_step_forces_match_oracle(synth_small):
    eng = ig.Engine(synth_small)
    f = eng.compute_forces()
    ref, _, _ = O.Oracle(synth_small).total_force(seed=synth_small.seed, step=0)
    check_force(f, ref, "total force, 44 atoms")


def test_graph_step_equals_call_sequence(synth_medium):
    a = ig.Engine(synth_medium)
    b = ig.Engine(synth_medium, use_graph=False)
    c = ig.Engine(synth_medium)
    a.step(10)
    b.step(10)
    for _ in range(10):
        c.compute_forces()
        c.leapfrog()
    pa, pb, pc = a.positions(), b.positions(), c.positions()
    assert np.array_equal(pa, pb)  # deterministic: fixed-point accumulation
    assert np.array_equal(pa, pc)
    assert a.get_step() == 10


@pytest.mark.parametrize("chunk, tail", [(128, 0), (37, 0), (256, 32)])
def test_force_kernel_atoms_per_thread_bit_identical(synth_medium, chunk, tail):
    """With the same point chunks, the 2-atoms-per-thread force kernel gives the
    1-atom kernel's forces bit for bit (each atom sees the same arithmetic in
    the same order), also with a ragged chunk, partial atom tiles and short
    chunks listed last."""
    out = []
    for apt in (1, 2):
        eng = ig.Engine(synth_medium, force_atoms_per_thread=apt, force_chunk=chunk, force_tail_chunk=tail)
        assert eng.shapes()["force_atoms_per_thread"] == apt
        eng.zero_forces()
        eng.isspa_force()
        out.append(eng.forces())
        eng.step(3)
        out.append(eng.positions())
    assert np.array_equal(out[0], out[2])
    assert np.array_equal(out[1], out[3])


@pytest.mark.parametrize("chunk, tail", [(128, 0), (37, 0), (256, 32)])
def test_force_vote_loop_bit_identical(synth_medium, chunk, tail):
    """The warp-voted point loop of the force pass gives the per-pair loop's
    forces and trajectory bit for bit (ragged chunks, partial tiles, short
    chunks listed last)."""
    out = []
    for vote in (0, 1):
        eng = ig.Engine(synth_medium, force_chunk=chunk, force_tail_chunk=tail, force_vote=vote)
        assert eng.shapes()["force_vote"] == vote
        eng.zero_forces()
        eng.isspa_force()
        out.append(eng.forces())
        eng.step(5)
        out.append(eng.positions())
    assert np.array_equal(out[0], out[2])
    assert np.array_equal(out[1], out[3])


@pytest.mark.parametrize("chunk, tail", [(512, 32), (128, 16), (64, 0)])
def test_force_work_list_with_short_items_last(synth_medium, chunk, tail):
    """Long chunks followed by short ones cover every (atom, point) pair once:
    the IS-SPA force matches the oracle, and the item count is that of the two
    chunk lengths."""
    s = synth_medium
    eng = ig.Engine(s, force_chunk=chunk, force_tail_chunk=tail)
    sh = eng.shapes()
    assert sh["force_chunk"] == chunk and sh["force_tail_chunk"] == tail
    tiles = -(-s.n_atoms // 128)
    P = s.n_atoms * s.n_mc
    if tail == 0:
        assert sh["force_items"] == tiles * -(-P // chunk)
    else:
        n_long = (sh["force_items"] // tiles)  # chunks of both lengths
        assert sh["force_items"] % tiles == 0 and n_long > -(-P // chunk)
    eng.zero_forces()
    eng.isspa_force()
    o = O.Oracle(s)
    ref = o.isspa_force(o.mc_points(seed=s.seed, step=0), terms=7)
    check_force(eng.forces(), ref, f"isspa chunk {chunk} tail {tail}")


def test_point_injection(adi2_100):
    s = adi2_100
    o = O.Oracle(s)
    pts = o.mc_points(seed=999, step=5)
    eng = ig.Engine(s)
    eng.set_mc_points(pts)
    eng.zero_forces()
    eng.isspa_force()
    check_force(eng.forces(), o.isspa_force(pts), "injected points")
    eng.clear_mc_points()
    eng.zero_forces()
    eng.isspa_force()
    check_force(eng.forces(), o.isspa_force(o.mc_points(seed=s.seed, step=0)), "Philox points again")


@pytest.mark.parametrize("shapes", [{}, {"force_chunk": 96, "force_tail_chunk": 32, "field_split": 4,
                                         "field_vote": 1, "force_vote": 1}, "autotuned"],
                         ids=["default", "tail-vote", "autotuned"])
def test_batched_windows_match_oracle(shapes):
    """Windows of different sizes in one engine against the oracle window by
    window: with the default shapes, with short force chunks listed last
    (per-window tail stretches) and both warp-voted loops, and with whatever
    the autotuner picks."""
    wins = ig.synth.config_batched(n_windows=3, seed=9)
    if shapes == "autotuned":
        eng = ig.Engine(wins)
        print(eng.autotune())
    else:
        eng = ig.Engine(wins, **shapes)
    f = eng.compute_forces()
    off = 0
    com, cv = eng.us_com()
    for w, s in enumerate(wins):
        o = O.Oracle(s)
        ref, _, c = o.total_force(seed=s.seed, step=0, window=w)
        n = s.n_atoms
        check_force(f[off:off + n], ref, f"batched window {w} ({n} atoms)")
        assert np.allclose(com[w], c, atol=1e-9)
        off += n


def test_neighbor_and_cell_lists_bit_exact(synth_medium):
    eng = ig.Engine(synth_medium)
    rows, counts = eng.neighbor_list(10.0, 256)
    r_o, c_o = O.Oracle(synth_medium).neighbor_list(10.0, 256)
    assert np.array_equal(counts, c_o)
    assert np.array_equal(rows, r_o)
    nc = [3, 3, 3]
    assert np.array_equal(eng.cell_list(34.0 / 3, nc), O.Oracle(synth_medium).cell_index(34.0 / 3, nc))


def test_statistical_pin_to_reference_frames(adi2):
    """Per-term means over 4000 seeds at nMC=1000 vs the reference's 1000-seed
    frame averages (timing_tests/ADI2/10000MC/compare).  All 132 components of
    a frame come from one point set, so their noise is correlated: the test
    bounds the rms and the maximum of the z-scores rather than their median."""
    for terms, name in [(1, "Csolv"), (2, "LJsolv"), (4, "Csolv_CDD")]:
        eng = ig.Engine(adi2, isspa_terms=terms)
        acc = []
        for k in range(4000):
            eng.set_step(k)
            eng.zero_forces()
            eng.isspa_force()
            acc.append(eng.forces())
        a = np.array(acc, np.float64)
        mean, sem = a.mean(0), a.std(0, ddof=1) / np.sqrt(len(a))
        r = np.load(os.path.join(GOLDEN, f"ref_frames_{name}.npz"))
        z = (mean - r["mean"]) / np.sqrt(sem ** 2 + r["sem"] ** 2)
        rms = float(np.sqrt(np.mean(z ** 2)))
        print(name, "rms z", rms, "median |z|", np.median(np.abs(z)), "max |z|", np.abs(z).max())
        assert rms < 1.6
        assert np.abs(z).max() < 5.0
        eng.close()
