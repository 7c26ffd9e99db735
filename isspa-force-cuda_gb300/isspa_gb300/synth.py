"""Seeded synthetic IS-SPA systems (stand-ins for the reference's run fixtures).

There is no public benchmark dataset for this engine; these generators build
systems with the shapes and value distributions of the benchmark workloads:

* linear chains with bonds (k=300 kcal/mol/A^2, r0=1.5 A), angles (k=50,
  110 deg) and dihedrals (n=3, V=1.4) along the backbone; 1-2, 1-3 and 1-4
  exclusions as Amber writes them;
* 5 LJ types with sigma in [2.5, 3.5] A and epsilon in [0.05, 0.2] kcal/mol,
  Lorentz-Berthelot A/B coefficients in Amber's packed-triangle layout;
* charges uniform in +-qmax e, shifted to net zero per chain, in Amber units;
* chain conformations as self-avoiding random walks placed without overlap;
* IS-SPA tables on the fixtures' grid r = 0.05 + 0.1 k, k < 120: a parabolic
  g(r) (0 inside the excluded radius, g0 - alpha (r - x0)^2, then 1; the
  parametrisation of the reference's OpenMP model), a damped oscillating mean
  field, and the LJ force against one solvent site as the mean-force table.
"""
from __future__ import annotations

import math
from typing import List, Optional, Tuple

import numpy as np

from .system import System

AMBER_CHARGE = 18.2223
N_TYPES = 5
MASSES = np.array([12.01, 14.01, 16.00, 12.01, 32.06], np.float32)
GRID_R0, GRID_DR, GRID_N = 0.05, 0.1, 120
KT_PER_K = 0.00198717          # config_class.cpp:125
DT = np.float32(0.002) * np.float32(20.455)  # config_class.cpp:123-124


def forcefield(seed: int = 7, rmax: float = 12.0, n_mc: int = 50):
    """Shared force field: LJ types, IS-SPA tables and OpenMP-model parameters."""
    rng = np.random.default_rng(seed)
    sig = rng.uniform(2.5, 3.5, N_TYPES)
    eps = rng.uniform(0.05, 0.2, N_TYPES)
    nt = N_TYPES
    lj_ab = np.zeros((nt * (nt + 1) // 2, 2), np.float32)
    nbp = np.zeros(nt * nt, np.int32)
    for i in range(nt):
        for j in range(i + 1):
            k = i * (i + 1) // 2 + j
            s = 0.5 * (sig[i] + sig[j])
            e = math.sqrt(eps[i] * eps[j])
            lj_ab[k] = (4 * e * s ** 12, 4 * e * s ** 6)
            nbp[i * nt + j] = k
            nbp[j * nt + i] = k
    r = (GRID_R0 + GRID_DR * np.arange(GRID_N)).astype(np.float64)
    x0 = rng.uniform(3.8, 4.6, nt)
    w = rng.uniform(0.7, 0.9, nt)
    g0 = rng.uniform(1.5, 1.9, nt)
    alpha = g0 / w ** 2
    r_ex = x0 - w
    r_end = x0 + np.sqrt((g0 - 1.0) / alpha)
    amp = rng.uniform(0.5, 2.5, nt)
    sig_s, eps_s = 3.15, 0.152
    g = np.zeros((nt, GRID_N)); e = np.zeros((nt, GRID_N)); f = np.zeros((nt, GRID_N))
    for t in range(nt):
        inside = (r >= r_ex[t]) & (r <= r_end[t])
        g[t] = np.where(r < r_ex[t], 0.0, np.where(inside, g0[t] - alpha[t] * (r - x0[t]) ** 2, 1.0))
        d = np.maximum(r - r_ex[t], 0.0)
        e[t] = np.where(r >= r_ex[t], amp[t] * np.sin(2 * np.pi * d / 3.0) * np.exp(-d / 2.5), 0.0)
        s = 0.5 * (sig[t] + sig_s)
        ee = math.sqrt(eps[t] * eps_s)
        sr = s / r
        f[t] = np.where(r >= r_ex[t], 24 * ee / r * (2 * sr ** 12 - sr ** 6), 0.0)
    omp = dict(x0=x0.astype(np.float32), g0=g0.astype(np.float32), w=w.astype(np.float32),
               alpha=alpha.astype(np.float32),
               gr2=np.stack([r_ex ** 2, r_end ** 2], 1).astype(np.float32).ravel(),
               lj_A=np.array([lj_ab[t * (t + 1) // 2 + t, 0] for t in range(nt)], np.float32),
               lj_B=np.array([lj_ab[t * (t + 1) // 2 + t, 1] for t in range(nt)], np.float32))
    params = dict(sigma=sig, epsilon=eps, x0=x0, w=w, g0=g0, e_amp=amp, sigma_s=sig_s, epsilon_s=eps_s,
                  r_cut=r_ex.copy())
    return dict(lj_ab=lj_ab, nbp=nbp, rmax=np.full(nt, rmax, np.float32),
                g=g.astype(np.float32), e=e.astype(np.float32), f=f.astype(np.float32), omp=omp,
                n_mc=n_mc, params=params)


def grid_r() -> np.ndarray:
    """Radii of the tabulated grid (the fixtures' r = 0.05 + 0.1 k)."""
    return GRID_R0 + GRID_DR * np.arange(GRID_N)


def tables_from_params(p: dict, xp=np):
    """Force-field tables as functions of the per-type parameters, in FP64.

    sigma, epsilon (LJ, Lorentz-Berthelot) give the packed A/B coefficients and
    the tabulated mean LJ force against one solvent site (zero below the fixed
    radius r_cut, so that the table is smooth in every parameter); x0, w, g0
    give the parabolic g(r): 0 below x0 - w, g0 - (g0/w^2)(r - x0)^2 up to where
    it reaches 1, then 1.  `xp` may be numpy or torch (for automatic
    differentiation in the tests)."""
    sig, eps = p["sigma"], p["epsilon"]
    nt = sig.shape[0]
    r = xp.asarray(grid_r()) if xp is np else xp.tensor(grid_r(), dtype=sig.dtype)
    A, B = [], []
    for i in range(nt):
        for j in range(i + 1):
            s = 0.5 * (sig[i] + sig[j])
            e = xp.sqrt(eps[i] * eps[j])
            A.append(4 * e * s ** 12)
            B.append(4 * e * s ** 6)
    lj_ab = xp.stack([xp.stack(A), xp.stack(B)], 1)
    g_rows, f_rows = [], []
    for t in range(nt):
        x0, w, g0 = p["x0"][t], p["w"][t], p["g0"][t]
        alpha = g0 / w ** 2
        r_ex = x0 - w
        r_end = x0 + xp.sqrt((g0 - 1.0) / alpha)
        par = g0 - alpha * (r - x0) ** 2
        g_rows.append(xp.where(r < r_ex, xp.zeros_like(r), xp.where(r <= r_end, par, xp.ones_like(r))))
        s = 0.5 * (sig[t] + p["sigma_s"])
        e = xp.sqrt(eps[t] * p["epsilon_s"])
        sr = s / r
        lj = 24 * e / r * (2 * sr ** 12 - sr ** 6)
        f_rows.append(xp.where(r >= float(p["r_cut"][t]), lj, xp.zeros_like(r)))
    return dict(lj_ab=lj_ab, g=xp.stack(g_rows), f=xp.stack(f_rows))


def _grow_chain(rng, length: int, start: np.ndarray, max_tries: int = 200) -> Optional[np.ndarray]:
    bond, theta = 1.5, math.radians(110.0)
    for _ in range(max_tries):
        x = np.zeros((length, 3))
        x[0] = start
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if length > 1:
            x[1] = x[0] + bond * d
        ok = True
        for i in range(2, length):
            placed = False
            for _ in range(30):
                b1 = x[i - 1] - x[i - 2]
                b1 /= np.linalg.norm(b1)
                a = rng.normal(size=3)
                a -= a.dot(b1) * b1
                a /= np.linalg.norm(a)
                nd = -math.cos(theta) * b1 + math.sin(theta) * a
                cand = x[i - 1] + bond * nd
                if i >= 3:
                    dd = np.linalg.norm(x[: i - 2] - cand, axis=1)
                    lim = np.full(i - 2, 3.0)
                    lim[-1] = 2.5  # the 1-4 partner
                    if np.any(dd < lim):
                        continue
                x[i] = cand
                placed = True
                break
            if not placed:
                ok = False
                break
        if ok:
            return x
    return None


def make_chains(n_chains: int, length: int, box: float, rng) -> np.ndarray:
    """Self-avoiding chains placed without overlap (min image distance >= 3 A),
    checked against already placed atoms through a 3 A cell grid."""
    m = max(1, int(box // 3.0))
    cell = box / m
    grid = {}
    out = []

    def clash(xw):
        for p in xw:
            c = np.floor(p / cell).astype(int) % m
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        lst = grid.get(((c[0] + dx) % m, (c[1] + dy) % m, (c[2] + dz) % m))
                        if not lst:
                            continue
                        d = np.asarray(lst) - p
                        d -= box * np.round(d / box)
                        if np.min(np.einsum("ij,ij->i", d, d)) < 9.0:
                            return True
        return False

    for c in range(n_chains):
        for _ in range(2000):
            x = _grow_chain(rng, length, rng.uniform(0, box, 3))
            if x is None:
                continue
            xw = np.mod(x, box)
            if clash(xw):
                continue
            for p in xw:
                k = tuple(np.floor(p / cell).astype(int) % m)
                grid.setdefault(k, []).append(p)
            out.append(xw)
            break
        else:
            raise RuntimeError("could not place chain %d" % c)
    return np.concatenate(out).astype(np.float32)


def make_system(n_chains: int, length: int, box: float, n_mc: int, seed: int, qmax: float = 0.6,
                ff: Optional[dict] = None, temperature: float = 298.0, pnu: float = 0.02,
                us: Optional[Tuple[float, float]] = None, run_seed: int = 12345) -> System:
    """One window: `n_chains` chains of `length` atoms in a cubic box."""
    ff = ff if ff is not None else forcefield(n_mc=n_mc)
    rng = np.random.default_rng(seed)
    N = n_chains * length
    xyz = make_chains(n_chains, length, box, rng)
    types = rng.integers(0, N_TYPES, N).astype(np.int32)
    q = rng.uniform(-qmax, qmax, (n_chains, length))
    q -= q.mean(axis=1, keepdims=True)
    q = (q.ravel() * AMBER_CHARGE).astype(np.float32)
    pos = np.zeros((N, 4), np.float32)
    pos[:, :3] = xyz
    pos[:, 3] = q
    mass = MASSES[types]
    kT = np.float32(temperature) * np.float32(KT_PER_K)
    vel = np.zeros((N, 4), np.float32)
    vel[:, :3] = rng.normal(size=(N, 3)) * np.sqrt(kT / mass)[:, None]
    vel[:, 3] = np.where(mass < 2.0, 12.0, mass)
    bonds, angles, dihs = [], [], []
    excl_cnt, excl = [], []
    for c in range(n_chains):
        o = c * length
        for i in range(length):
            if i + 1 < length:
                bonds.append((o + i, o + i + 1, 0))
            if i + 2 < length:
                angles.append((o + i, o + i + 1, o + i + 2, 0))
            if i + 3 < length:
                dihs.append((o + i, o + i + 1, o + i + 2, o + i + 3))
            partners = [o + j for j in range(i + 1, min(i + 4, length))]
            if not partners:
                partners = [-1]  # Amber writes one 0 for "no exclusions"
            excl_cnt.append(len(partners))
            excl.extend(partners)
    sys = System(
        pos=pos, vel=vel, raw_mass=mass.astype(np.float32), n_lj_types=N_TYPES, lj_type=types,
        nb_parm_index=ff["nbp"], lj_ab=ff["lj_ab"],
        n_excl_cum=np.cumsum(excl_cnt).astype(np.int32), excl_list=np.array(excl, np.int32),
        bond_atoms=np.array(bonds, np.int32).reshape(-1, 3),
        bond_params=np.array([[600.0, 1.5]], np.float32),
        angle_atoms=np.array(angles, np.int32).reshape(-1, 4),
        angle_params=np.array([[100.0, math.radians(110.0)]], np.float32),
        dih_atoms=np.array(dihs, np.int32).reshape(-1, 4),
        dih_types=np.zeros(len(dihs), np.int32),
        dih_params=np.array([[3.0, 1.4, 0.0, 0.0]], np.float32),
        scaled14=np.array([[1.2, 2.0]], np.float32),
        isspa_type=types.copy(), rmax=ff["rmax"], g_table=ff["g"], e_table=ff["e"], f_table=ff["f"],
        g_r0=GRID_R0, g_dr=np.float32(GRID_R0 + GRID_DR) - np.float32(GRID_R0),
        e_r0=GRID_R0, e_dr=np.float32(GRID_R0 + GRID_DR) - np.float32(GRID_R0),
        f_r0=GRID_R0, f_dr=np.float32(GRID_R0 + GRID_DR) - np.float32(GRID_R0),
        n_mc=n_mc, box=box, kT=float(kT), dt=float(DT), pnu=pnu, seed=run_seed)
    if us is not None and n_chains >= 2:
        k, x0 = us
        g0 = [(o, 0) for o in range(length)]
        g1 = [(length + o, 1) for o in range(length)]
        sys.us_on = 1
        sys.bias_list = np.array(g0 + g1, np.int32)
        sys.us_k, sys.us_x0 = float(k), float(x0)
    sys.omp = ff["omp"]
    return sys


# ---- benchmark workloads ---------------------------------------------------
def config_small(seed: int = 1) -> System:
    """44 atoms (2 chains of 22), nMC=20, 40 A box."""
    return make_system(2, 22, 40.0, 20, seed, ff=forcefield(n_mc=20))


def config_plain(seed: int = 2) -> System:
    """1100 atoms (50 chains of 22), nMC=50, 60 A box: the plain drop-in path."""
    return make_system(50, 22, 60.0, 50, seed, ff=forcefield(n_mc=50))


def config_precision(seed: int = 3) -> System:
    """16384 atoms (256 chains of 64), nMC=100, 120 A box, charges +-0.8 e."""
    return make_system(256, 64, 120.0, 100, seed, qmax=0.8, ff=forcefield(n_mc=100))


def config_batched(n_windows: int = 64, seed: int = 4, box: float = 60.0) -> List[System]:
    """64 umbrella windows, 44..1100 atoms each, k=10, r0 from 4 to 16 A, nMC=50."""
    rng = np.random.default_rng(seed)
    ff = forcefield(n_mc=50)
    sizes = rng.integers(2, 51, n_windows)
    x0s = np.linspace(4.0, 16.0, n_windows)
    return [make_system(int(c), 22, box, 50, seed * 1000 + w, ff=ff, us=(10.0, float(x0s[w])))
            for w, c in enumerate(sizes)]


def config_adjoint(n_windows: int = 16, seed: int = 5) -> List[System]:
    """25 chains (550 atoms) in a 50 A box, 16 windows r0 5..12 A, nMC=50."""
    ff = forcefield(n_mc=50)
    base = make_system(25, 22, 50.0, 50, seed, ff=ff, us=(10.0, 5.0))
    out = []
    for w, x0 in enumerate(np.linspace(5.0, 12.0, n_windows)):
        s = base.copy()
        s.us_x0 = float(x0)
        s.omp = base.omp
        out.append(s)
    return out
