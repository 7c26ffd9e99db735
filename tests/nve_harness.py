"""Test-harness pieces for energy-conservation (NVE) runs (not part of the library).

* `oracle_nve`: a reference NVE trajectory with the FP64 oracle forces and an
  FP64 integrator state (positions and velocities kept in double; only the
  force evaluation sees the float-rounded coordinates, as the oracle takes
  float positions).  Conservative terms only: bonded with 1-4, nonbond LJ +
  Coulomb + IS-SPA correction, umbrella; no IS-SPA mean-field force and no
  thermostat.  The update is the reference's thermostat-free leapfrog with
  its wrap (leapfrog_cuda.cu:57-64).
* `total_energy`, `drift`: E(t) = potential + (K(t-dt/2) + K(t+dt/2))/2 and
  the least-squares drift rate with the residual fluctuation.
"""
from __future__ import annotations

import numpy as np

import oracle as O

FS_PER_STEP = 2.0  # dt = 0.002 ps (internal 0.002 * 20.455)


def total_energy(e: np.ndarray) -> np.ndarray:
    """e[..., 12] energy components (ISSPA_E_* order) -> total energy."""
    e = np.asarray(e)
    return e[..., 2:11].sum(-1) + 0.5 * (e[..., 0] + e[..., 1])


def drift(steps, E, n_atoms: int, fs_per_step: float = FS_PER_STEP) -> dict:
    """Linear drift of E (kcal/mol) against time: per ns, per ns and degree
    of freedom, and the RMS residual about the fit."""
    t_ns = np.asarray(steps, np.float64) * fs_per_step * 1e-6
    E = np.asarray(E, np.float64)
    slope, icpt = np.polyfit(t_ns, E, 1)
    res = E - (slope * t_ns + icpt)
    return {"kcal_per_mol_ns": float(slope), "kcal_per_mol_ns_dof": float(slope / (3 * n_atoms)),
            "rms_fluct": float(np.sqrt(np.mean(res ** 2))), "span_ns": float(t_ns[-1] - t_ns[0])}


def oracle_nve(s, n_steps: int, every: int, threads: int = 0):
    """Returns (steps, energies[n_samples][12]) of an FP64-state NVE run."""
    pos = s.pos[:, :3].astype(np.float64).copy()
    vel = s.vel[:, :3].astype(np.float64).copy()
    q = np.asarray(s.pos[:, 3], np.float32)
    m = np.asarray(s.vel[:, 3], np.float64)
    dt, box = float(s.dt), float(s.box)
    steps, out = [], []
    for k in range(n_steps + 1):
        t = s.copy()
        t.pos = np.ascontiguousarray(np.c_[pos.astype(np.float32), q], np.float32)
        t.vel = np.ascontiguousarray(np.c_[vel, m].astype(np.float32))
        o = O.Oracle(t, threads=threads)
        f = o.bonded(with_14=True) + o.nonbond(7)
        if t.us_on:
            f += o.us()[0]
        vnew = vel + f * dt / m[:, None]
        if k % every == 0:
            e = o.energies(f)
            e[0] = 0.5 * np.sum(m[:, None] * vel * vel)
            e[1] = 0.5 * np.sum(m[:, None] * vnew * vnew)
            steps.append(k)
            out.append(e)
        if k == n_steps:
            break
        vel = vnew
        pos = pos + vel * dt
        pos = np.where(pos > box, pos - box, np.where(pos < 0.0, pos + box, pos))
    return np.asarray(steps), np.asarray(out)
