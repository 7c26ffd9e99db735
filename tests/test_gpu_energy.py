"""Energies, virial and NVE drift on the GPU, against the FP64 oracle.

* isspa_energies per component against the oracle's FP64 energies of the same
  state (44- and 1100-atom systems with an umbrella restraint; two windows
  batched); pair energies are FP32 per pair with FP64 sums, so the bound is
  normwise over the components: max |dE| <= 2e-6 max |E|.  The virial sums
  pair terms r . F of both signs that are each far larger than the total near
  contacts; its bound is 1e-5 of its magnitude.
* isspa_energies leaves the trajectory untouched (bit-identical positions).
* NVE (no thermostat, no IS-SPA mean-field force), 44 atoms, 2 fs: the GPU
  run tracks the FP64-state oracle run over its first 200 steps and its
  energy drift over 100 000 steps (200 ps) is reported beside the oracle
  run's (same length).
* NVE of the 16 384-atom precision workload over 50 000 steps (slow): drift
  rate reported; energies at the last frame checked against the oracle; the
  first 25 ps repeated at 1 fs show the drift coming from the 2 fs time step
  (it shrinks with dt, where FP32 rounding would grow with the step count).
"""
import time

import numpy as np
import pytest

import isspa_gb300 as ig
import isspa_gb300.synth as synth
from isspa_gb300 import abi
import nve_harness as H
import oracle as O

pytestmark = pytest.mark.gpu

NAMES = abi.ENERGY_NAMES
TOL = 2e-6


def _check(e_gpu, e_orc, label):
    d = np.abs(e_gpu - e_orc)
    scale = np.abs(e_orc[:11]).max()
    rel = {n: float(d[k] / max(abs(e_orc[k]), 1e-300)) for k, n in enumerate(NAMES)}
    print(f"{label}: normwise {d[:11].max() / scale:.2e}; virial {rel['virial']:.2e}; per component",
          {n: f"{v:.1e}" for n, v in rel.items()})
    assert d[:11].max() <= TOL * scale
    assert d[11] <= 1e-5 * abs(e_orc[11])


@pytest.mark.parametrize("which", ["small", "plain"])
def test_energies_match_fp64_oracle(which):
    if which == "small":
        s = synth.make_system(2, 22, 40.0, 20, seed=11, us=(10.0, 6.0))
    else:
        s = synth.make_system(50, 22, 60.0, 50, seed=2, ff=synth.forcefield(n_mc=50), us=(10.0, 8.0))
    eng = ig.Engine(s)
    eng.step(5)
    f = eng.compute_forces()
    eng.zero_forces()
    e = eng.energies()[0]
    t = s.copy()
    t.pos, t.vel = eng.positions(), eng.velocities()
    ref = O.Oracle(t).energies(f)
    _check(e, ref, which)
    assert e[0] > 0 and e[1] > 0 and e[10] > 0
    assert eng.device_status() == 0


def test_batched_windows_energies():
    base = synth.make_system(3, 22, 40.0, 20, seed=12, us=(10.0, 5.0))
    other = synth.make_system(5, 22, 45.0, 20, seed=13, us=(10.0, 9.0))
    # IS-SPA off: its MC points (and so the kick in the after-kick kinetic
    # energy) carry the window index in their Philox counters
    eng = ig.Engine([base, other], isspa_terms=abi.TERMS_NONE)
    e = eng.energies()
    for w, s in enumerate((base, other)):
        single = ig.Engine(s, isspa_terms=abi.TERMS_NONE).energies()[0]
        d = np.abs(e[w] - single).max() / np.abs(single).max()
        print(f"window {w}: batched vs single {d:.1e}")
        # the batch tiles the pair work differently, so the FP32 per-stage
        # partial sums round differently
        assert d <= 1e-9


def test_energies_leave_the_trajectory_unchanged():
    s = synth.make_system(2, 22, 40.0, 20, seed=11)
    a, b = ig.Engine(s), ig.Engine(s)
    for _ in range(3):
        a.step(4)
        b.step(4)
        b.energies()
    assert np.array_equal(a.positions(), b.positions())
    assert np.array_equal(a.velocities(), b.velocities())
    assert a.get_step() == b.get_step()


def test_nve_small_against_fp64_oracle_run():
    s = synth.make_system(2, 22, 40.0, 20, seed=1, pnu=0.0)
    eng = ig.Engine(s, isspa_terms=abi.TERMS_NONE)
    # early steps: the two runs start from the same state and track each other
    st_o, e_o = H.oracle_nve(s, 200, 10)
    e_g = []
    for k in range(0, 201, 10):
        e_g.append(eng.energies()[0])
        if k < 200:
            eng.step(10)
    E_g, E_o = H.total_energy(np.asarray(e_g)), H.total_energy(e_o)
    ke = 0.5 * (e_o[0, 0] + e_o[0, 1])
    _check(np.asarray(e_g)[0], e_o[0], "nve step 0")
    early = np.abs(E_g - E_o).max()
    print(f"first 200 steps: max |E_gpu - E_oracle| = {early:.2e} kcal/mol (kinetic {ke:.1f})")
    assert early <= 1e-3 * ke
    # long run: drift rate of each
    n, every = 100_000, 500
    t0 = time.time()
    st_o, e_o = H.oracle_nve(s, n, every)
    t_orc = time.time() - t0
    eng = ig.Engine(s, isspa_terms=abi.TERMS_NONE)
    e_g = []
    t0 = time.time()
    for k in range(0, n + 1, every):
        e_g.append(eng.energies()[0])
        if k < n:
            eng.step(every)
    t_gpu = time.time() - t0
    dg = H.drift(st_o, H.total_energy(np.asarray(e_g)), s.n_atoms)
    do = H.drift(st_o, H.total_energy(e_o), s.n_atoms)
    print(f"NVE 44 atoms, {n} steps of 2 fs: GPU FP32 drift {dg['kcal_per_mol_ns']:+.2f} kcal/mol/ns "
          f"({dg['kcal_per_mol_ns_dof']:+.4f} per dof), rms fluct {dg['rms_fluct']:.3f}; "
          f"FP64-state oracle {do['kcal_per_mol_ns']:+.2f} ({do['kcal_per_mol_ns_dof']:+.4f}), "
          f"rms fluct {do['rms_fluct']:.3f}; wall {t_gpu:.1f} s GPU, {t_orc:.1f} s oracle")
    # the FP32 run conserves energy as well as the FP64-state run, within the
    # chaotic spread of two trajectories that separated after a few hundred steps
    bound = abs(do["kcal_per_mol_ns"]) + 4.0 * (dg["rms_fluct"] + do["rms_fluct"]) / dg["span_ns"]
    assert abs(dg["kcal_per_mol_ns"]) <= bound
    assert eng.device_status() == 0


@pytest.mark.slow
def test_nve_precision_workload_drift_report():
    s = synth.config_precision(seed=3)
    s.pnu = 0.0

    def run(system, n, every):
        eng = ig.Engine(system, isspa_terms=abi.TERMS_NONE)
        e, st = [], []
        for k in range(0, n + 1, every):
            e.append(eng.energies()[0])
            st.append(k)
            if k < n:
                eng.step(every)
        return eng, np.asarray(st), np.asarray(e)

    n, every = 50_000, 1000
    t0 = time.time()
    eng, steps, e_g = run(s, n, every)
    wall = time.time() - t0
    d = H.drift(steps, H.total_energy(e_g), s.n_atoms)
    # the first 25 ps at 2 fs and again at 1 fs
    early = steps <= 12_500
    d2 = H.drift(steps[early], H.total_energy(e_g[early]), s.n_atoms)
    s1 = s.copy()
    s1.dt = s.dt / 2
    _, st1, e1 = run(s1, 25_000, 1000)
    d1 = H.drift(st1, H.total_energy(e1), s.n_atoms, fs_per_step=1.0)
    print(f"first 25 ps: drift {d2['kcal_per_mol_ns']:+.1f} kcal/mol/ns at 2 fs, "
          f"{d1['kcal_per_mol_ns']:+.1f} at 1 fs (ratio {d2['kcal_per_mol_ns'] / d1['kcal_per_mol_ns']:.1f})")
    assert abs(d1["kcal_per_mol_ns"]) < abs(d2["kcal_per_mol_ns"])
    ke = 0.5 * (e_g[:, 0] + e_g[:, 1])
    print(f"NVE 16384 atoms, {n} steps of 2 fs (100 ps): drift {d['kcal_per_mol_ns']:+.2f} kcal/mol/ns "
          f"= {d['kcal_per_mol_ns_dof']:+.5f} per dof, rms fluct {d['rms_fluct']:.3f} kcal/mol, "
          f"mean kinetic {ke.mean():.1f} kcal/mol, E0 {H.total_energy(e_g[0]):.3f}, "
          f"E_end {H.total_energy(e_g[-1]):.3f}; {wall:.1f} s")
    # the last frame's energies against the FP64 oracle
    t = s.copy()
    t.pos, t.vel = eng.positions(), eng.velocities()
    f = eng.compute_forces()
    eng.zero_forces()
    _check(eng.energies()[0], O.Oracle(t).energies(f), "precision workload, last frame")
    assert abs(d["kcal_per_mol_ns_dof"]) < 1.0
    assert eng.device_status() == 0
