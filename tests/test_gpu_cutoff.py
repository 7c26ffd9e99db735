"""The optional cutoff mode of the nonbond pass (isspa_engine_options.
nonbond_cutoff > 0), through the C ABI.

The reference evaluates every nonbond pair (nonbond_force_cuda.cu:31-174; the
`rCut2` it is handed is unused) and never calls its neighbour-list and
cell-list kernels (neighborlist_cuda.cu, cell_list_cuda.cu).  The engine's
cutoff mode truncates LJ, Coulomb and the IS-SPA correction at rc (a pair
counts iff its FP32 squared distance is below rc^2) and finds the pairs
through a Verlet list over per-window cell lists rebuilt on the device.

* Forces against the FP64 oracle's truncated sums (tests/parity.py measures):
  every term mask on the 1100-atom system (4^3 cells per window), a 44-atom
  window (3^3 cells), a 264-atom window whose box holds fewer than three list
  radii (one cell: the whole window), and three batched windows of different
  sizes; the cutoff visibly changes the force (against all pairs).
* A cutoff beyond every minimum-image distance gives the all-pairs forces.
* The list's independence: trajectories with skins of 0.3, 2 and 4 A (many or
  few rebuilds) are bit-identical, with either integrator; the number of
  builds falls as the skin grows.
* Energies of the truncated potential against the oracle's.
* A row capacity too small for the system is reported as
  ISSPA_ERR_LIST_FULL, without a fault, and the status resets.
* Options: negative or non-finite cutoff rejected; the single-kernel step
  falls back to the separate kernels; the adjoint refuses the cutoff mode;
  the shapes report the rows and cells.
"""
import ctypes as C
import math

import numpy as np
import pytest

import isspa_gb300 as ig
import isspa_gb300.synth as synth
from isspa_gb300 import abi
import oracle as O
from parity import check_force, nrel

pytestmark = pytest.mark.gpu

RC = 10.0


def nonbond(s, terms=7, **opts):
    eng = ig.Engine(s, nonbond_terms=terms, **opts)
    eng.zero_forces()
    eng.nonbond_force()
    f = eng.forces()
    st = eng.device_status()
    shapes = eng.shapes()
    eng.close()
    assert st == 0
    return f, shapes


@pytest.fixture(scope="module")
def plain():
    return synth.config_plain(seed=2)


@pytest.mark.parametrize("terms", [1, 2, 4, 7])
def test_cutoff_matches_oracle_1100(plain, terms):
    f, sh = nonbond(plain, terms, nonbond_cutoff=RC)
    assert sh["nonbond_list_cells"] == 4 ** 3  # 60 A box, list radius 12 A
    ref = O.Oracle(plain, nonbond_cutoff=RC).nonbond(terms)
    check_force(f, ref, f"1100 atoms, cutoff {RC} A, nonbond terms {terms}")
    full = O.Oracle(plain).nonbond(terms)
    assert nrel(ref, full) > 1e-4  # the truncation is visible (LJ alone: 8.5e-4 at 10 A)


@pytest.mark.parametrize("which", ["44 atoms (27 cells)", "264 atoms in a 34 A box (one cell)"])
def test_cutoff_matches_oracle_small_boxes(which):
    if which.startswith("44"):
        s = synth.config_small(seed=1)
        cells = 27
    else:
        s = synth.make_system(12, 22, 34.0, 20, seed=21, ff=synth.forcefield(n_mc=20))
        cells = 1
    f, sh = nonbond(s, nonbond_cutoff=RC)
    assert sh["nonbond_list_cells"] == cells
    check_force(f, O.Oracle(s, nonbond_cutoff=RC).nonbond(), f"{which}, cutoff {RC} A")


def test_cutoff_batched_windows_match_oracle():
    # two umbrella windows of the 60 A batch and one window whose 34 A box holds
    # fewer than three list radii (one cell)
    wins = synth.config_batched(n_windows=2, seed=9)
    wins.append(synth.make_system(12, 22, 34.0, 50, seed=77, ff=synth.forcefield(n_mc=50)))
    eng = ig.Engine(wins, nonbond_cutoff=RC)
    eng.zero_forces()
    eng.nonbond_force()
    f = eng.forces()
    assert eng.device_status() == 0
    off = 0
    for w, s in enumerate(wins):
        n = s.n_atoms
        check_force(f[off:off + n], O.Oracle(s, nonbond_cutoff=RC).nonbond(),
                    f"batched window {w} ({n} atoms, {s.box:g} A box), cutoff {RC} A")
        off += n


def test_cutoff_beyond_the_box_is_all_pairs(plain):
    rc = 60.0 * math.sqrt(3.0)  # beyond every minimum-image distance in the 60 A box
    f, sh = nonbond(plain, nonbond_cutoff=rc)
    assert sh["nonbond_list_cells"] == 1
    full, _ = nonbond(plain)
    ref = O.Oracle(plain).nonbond()
    check_force(f, ref, "cutoff beyond the box, against all pairs (oracle)")
    assert nrel(f, full) < 2e-6  # the all-pairs kernel, up to FP32 summation order


@pytest.mark.parametrize("integrator", [1, 2])
def test_cutoff_trajectory_independent_of_skin(plain, integrator):
    s = plain.copy()
    s.pnu = 0.05
    runs = {}
    for skin in (0.3, 2.0, 4.0):
        eng = ig.Engine(s, nonbond_cutoff=RC, nonbond_skin=skin, integrator=integrator)
        eng.step(40)
        runs[skin] = (eng.positions(), eng.velocities(), eng.nonbond_list_stats(), eng.device_status())
        eng.close()
    print({k: v[2] for k, v in runs.items()})
    for skin in (2.0, 4.0):
        assert runs[skin][3] == 0
        assert np.array_equal(runs[skin][0], runs[0.3][0])
        assert np.array_equal(runs[skin][1], runs[0.3][1])
    b = [runs[k][2]["builds"] for k in (0.3, 2.0, 4.0)]
    assert b[0] > b[1] >= b[2] >= 1


def test_cutoff_energies_match_oracle(plain):
    s = plain.copy()
    eng = ig.Engine(s, nonbond_cutoff=RC)
    eng.step(5)
    f = eng.compute_forces()
    eng.zero_forces()
    e = eng.energies()[0]
    t = s.copy()
    t.pos, t.vel = eng.positions(), eng.velocities()
    ref = O.Oracle(t, nonbond_cutoff=RC).energies(f)
    full = O.Oracle(t).energies(f)
    names = list(abi.ENERGY_NAMES)
    for name in ("lj", "coul", "corr"):
        k = names.index(name)
        rel = abs(e[k] - ref[k]) / max(abs(ref[k]), 1e-300)
        print(f"cutoff {RC} A, {name}: GPU {e[k]:.6f}, oracle {ref[k]:.6f} (all pairs {full[k]:.6f}), rel {rel:.1e}")
        assert rel < 2e-6
    d = np.abs(e[:11] - ref[:11])
    assert d.max() <= 2e-6 * np.abs(ref[:11]).max()


def test_cutoff_row_overflow_reported(plain):
    eng = ig.Engine(plain, nonbond_cutoff=RC, nonbond_list_max=4)
    assert eng.shapes()["nonbond_list_rows"] == 4
    eng.step(2)
    assert eng.device_status() == abi.ERR_LIST_FULL
    assert eng.device_status(reset=True) == abi.ERR_LIST_FULL
    assert eng.device_status() == 0
    assert eng.nonbond_list_stats()["fullest_row"] > 4


def test_cutoff_options(plain):
    L = abi.lib()
    for bad in (-1.0, float("nan"), float("inf")):
        with pytest.raises(RuntimeError):
            ig.Engine(plain, nonbond_cutoff=bad)
    eng = ig.Engine(plain, nonbond_cutoff=RC, integrator=3)
    sh = eng.shapes()
    assert sh["integrator"] == 1
    assert sh["nonbond_list_rows"] >= 32 and sh["nonbond_list_cells"] == 64
    st = eng.nonbond_list_stats()
    assert st["builds"] == 0
    eng.step(1)
    assert eng.nonbond_list_stats()["builds"] == 1
    J = (C.c_double * 1)()
    steps = (C.c_uint32 * 1)(0)
    assert L.isspa_adjoint_mean_force(eng._h, 1, None, steps, J, None, None, None, None) == abi.ERR_UNSUPPORTED
    eng.close()
    plain_eng = ig.Engine(plain)
    assert plain_eng.shapes()["nonbond_list_rows"] == 0
    b, m = C.c_int(), C.c_int()
    assert L.isspa_nonbond_list_stats(plain_eng._h, C.byref(b), C.byref(m)) == abi.ERR_STATE
