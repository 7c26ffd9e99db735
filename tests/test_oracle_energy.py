"""The oracle's energies are the potentials of its forces (CPU only).

* -dU/dx_i by a 4-point central difference in the positions against the
  oracle's conservative force (bonded with 1-4, nonbond LJ + Coulomb + IS-SPA
  correction, umbrella).  The step h = 2^-7 A is exact in float for every
  coordinate in [0, 64) A, so the difference carries only the O(h^4)
  truncation error.  Coordinates with a partner within 3h of the half-box
  distance are skipped: there the minimum image flips the pair force while
  the energy stays continuous, and the stencil straddles the kink.
* The virial sum r . F equals -dU/dlambda under a uniform scaling of the
  coordinates and the box (pair, bonded and restraint terms alike).
"""
import numpy as np

import isspa_gb300.synth as synth
import oracle as O

CONS = slice(2, 11)  # bond .. umbrella


def _system():
    s = synth.make_system(2, 22, 40.0, 20, seed=11, us=(10.0, 6.0))
    s.pos = np.ascontiguousarray(s.pos, np.float32)
    return s


def _potential(s, pos):
    t = s.copy()
    t.pos = pos
    o = O.Oracle(t)
    return o.energies(np.zeros((s.n_atoms, 3)))[CONS].sum()


def test_energy_gradient_is_the_conservative_force():
    s = _system()
    o = O.Oracle(s)
    f = o.bonded(with_14=True) + o.nonbond(7) + o.us()[0]
    h = 2.0 ** -7
    rng = np.random.default_rng(0)
    bias = np.asarray(s.bias_list).reshape(-1, 2)[:, 0]
    atoms = np.unique(np.concatenate([rng.choice(s.n_atoms, 6, replace=False), bias[:2]]))
    err = 0.0
    x = s.pos[:, :3].astype(np.float64)
    half = 0.5 * float(s.box)
    tested = 0
    for i in atoms:
        for d in range(3):
            r = np.abs(x[i, d] - x[:, d])
            r = np.where(r > half, float(s.box) - r, r)
            if np.any(np.abs(r - half) < 3 * h):
                continue
            tested += 1
            U = []
            for k in (-2, -1, 1, 2):
                p = s.pos.copy()
                p[i, d] = np.float32(p[i, d] + k * h)
                assert float(p[i, d]) == float(s.pos[i, d]) + k * h  # exact step
                U.append(_potential(s, p))
            g = (8.0 * (U[2] - U[1]) - (U[3] - U[0])) / (12.0 * h)
            err = max(err, abs(-g - f[i, d]))
    assert tested >= 3 * len(atoms) - 3
    scale = np.abs(f[atoms]).max()
    assert err <= 1e-5 * scale, (err, scale)


def test_virial_is_the_scaling_derivative():
    s = _system()
    o = O.Oracle(s)
    W = o.energies(np.zeros((s.n_atoms, 3)))[11]
    lam = 1e-3

    def U(l):
        t = s.copy()
        t.pos = s.pos.copy()
        t.pos[:, :3] = (s.pos[:, :3].astype(np.float64) * l).astype(np.float32)
        t.box = np.float32(s.box * l)
        e = O.Oracle(t).energies(np.zeros((s.n_atoms, 3)))
        return e[CONS].sum(), np.abs(e[CONS]).sum()

    (up, mag), (um, _) = U(1 + lam), U(1 - lam)
    dU = (up - um) / (2 * lam)
    # float rounding of the scaled coordinates (6e-8 relative) and the O(lam^2)
    # truncation limit the difference to ~1e-5 of the energy scale
    assert abs(-dU - W) <= 1e-4 * mag, (W, -dU, mag)
