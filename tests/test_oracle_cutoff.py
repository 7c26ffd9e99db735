"""The oracle's nonbond cutoff (the engine's optional cutoff mode), on the CPU.

* A cutoff beyond every minimum-image distance gives the all-pairs oracle
  forces exactly (and the energies to the rounding of their threaded sums).
* The truncated forces against an independent numpy evaluation of the same
  sums (FP32 minimum image and squared distance, FP64 pair forces; exclusions
  from the reference's cumulative lists, nonbond_force_cuda.cu:72-108: LJ and
  Coulomb skipped, the IS-SPA correction kept, :153-162).
"""
import math

import numpy as np

import isspa_gb300.synth as synth
import oracle as O

EP = 2.3473  # dielectric constant of the IS-SPA correction (constants.h)


def _mimg(d, L):
    h = np.float32(0.5) * L
    return np.where(np.abs(d) > h, d - np.copysign(L, d), d).astype(np.float32)


def _excluded_pairs(s):
    cum = np.asarray(s.n_excl_cum)
    lst = np.asarray(s.excl_list)
    out = set()
    for a in range(s.n_atoms):
        start = 0 if a == 0 else int(cum[a - 1])
        for e in range(start, int(cum[a])):
            b = int(lst[e])
            if b >= 0:
                out.add((a, b))
                out.add((b, a))
    return out


def _numpy_truncated(s, rc):
    pos = np.asarray(s.pos, np.float32).reshape(-1, 4)
    L = np.float32(s.box)
    cut2 = np.float32(rc) * np.float32(rc)
    rmax = np.asarray(s.rmax, np.float32)[np.asarray(s.isspa_type)]
    lj = np.asarray(s.lj_ab, np.float64).reshape(-1, 2)
    nbp = np.asarray(s.nb_parm_index).reshape(s.n_lj_types, s.n_lj_types)
    ljt = np.asarray(s.lj_type)
    ex = _excluded_pairs(s)
    epf = 1.0 - 1.0 / float(np.float32(EP))
    f = np.zeros((s.n_atoms, 3))
    for i in range(s.n_atoms):
        r = np.stack([_mimg(pos[i, k] - pos[:, k], L) for k in range(3)], axis=1)
        d2 = (r[:, 0] * r[:, 0] + r[:, 1] * r[:, 1] + r[:, 2] * r[:, 2]).astype(np.float32)
        for j in np.nonzero(d2 < cut2)[0]:
            if j == i:
                continue
            dd2 = float(r[j, 0]) ** 2 + float(r[j, 1]) ** 2 + float(r[j, 2]) ** 2
            dd = math.sqrt(dd2)
            qq = float(pos[i, 3]) * float(pos[j, 3])
            rm = float(rmax[j])
            two = np.float32(2.0) * rmax[j]
            if d2[j] > two * two:
                fs = -2.0 * qq * epf / (3.0 * dd2 * dd)
            else:
                fs = -qq * epf * (8.0 * rm - 3.0 * dd) / (24.0 * rm ** 4)
            if (i, j) not in ex:
                A, B = lj[nbp[ljt[i], ljt[j]]]
                r6 = 1.0 / dd2 ** 3
                fs += r6 * (12.0 * A * r6 - 6.0 * B) / dd2 + qq / (dd2 * dd)
            f[i] += fs * r[j].astype(np.float64)
    return f


def test_cutoff_beyond_the_box_equals_all_pairs():
    s = synth.config_small(seed=1)
    o_all = O.Oracle(s)
    o_cut = O.Oracle(s, nonbond_cutoff=s.box * math.sqrt(3.0))
    assert np.array_equal(o_cut.nonbond(), o_all.nonbond())
    f = o_all.nonbond()
    # the energy sums are OpenMP reductions (thread order): equal to rounding
    assert np.allclose(o_cut.energies(f), o_all.energies(f), rtol=1e-12, atol=0)


def test_cutoff_against_numpy():
    s = synth.config_small(seed=1)
    rc = 9.0
    got = O.Oracle(s, nonbond_cutoff=rc).nonbond()
    ref = _numpy_truncated(s, rc)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err
    full = O.Oracle(s).nonbond()
    assert np.abs(full - got).max() > 1e-3 * np.abs(full).max()  # the cutoff removes pairs
