"""isspa_write_isspatop: the written .isspatop reads back bit for bit (CPU).

* the ADI2 fixture's own IS-SPA sections, rewritten and reloaded through the
  reference config loader, give identical types, rmax, tables and radial grids;
* a synthetic system's tables (44 atoms, 5 types, parabolic g(r), LJ mean
  force, analytic field) written in place of ADI2's file load back the same;
* ISSPA_FORCES is written linearly (the values the reader uses).
"""
import os
import shutil

import numpy as np

import isspa_gb300 as ig

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("isspa_type", "rmax", "g_table", "e_table", "f_table", "g_r0", "g_dr", "e_r0", "e_dr", "f_r0", "f_dr")


def _copy_adi2(tmp_path):
    for f in ("ADI2.prmtop", "ADI2.rst7", "ADI2.isspatop", "adi2_config.txt"):
        shutil.copy(os.path.join(GOLDEN, f), tmp_path / f)
    return str(tmp_path / "adi2_config.txt"), str(tmp_path / "ADI2.isspatop")


def _same(a, b):
    # compared as the float32 values the engine is given (a synthetic system may
    # hold its grid origin and spacing as Python doubles)
    for k in FIELDS:
        x, y = np.asarray(getattr(a, k)), np.asarray(getattr(b, k))
        assert x.shape == y.shape, k
        if k == "isspa_type":
            assert np.array_equal(x, y), k
        else:
            assert np.array_equal(x.astype(np.float32), y.astype(np.float32)), k


def test_adi2_round_trip(tmp_path):
    cfg, isspatop = _copy_adi2(tmp_path)
    ref = ig.System.from_config(cfg)
    ref.write_isspatop(isspatop, "PDI")
    back = ig.System.from_config(cfg)
    _same(back, ref)


def test_synthetic_tables_round_trip(tmp_path):
    cfg, isspatop = _copy_adi2(tmp_path)
    s = ig.synth.config_small(seed=4)
    assert s.n_atoms == ig.System.from_config(cfg).n_atoms  # 44 atoms, as ADI2
    s.write_isspatop(isspatop, "synthetic")
    back = ig.System.from_config(cfg)
    _same(back, s)
    assert np.asarray(back.f_table).min() < 0.0  # linear forces, not log(F)
    with open(isspatop) as f:
        text = f.read()
    for flag in ("POINTERS", "ISSPA_TYPE_INDEX", "ISSPA_RMAX", "ISSPA_DENSITIES", "ISSPA_EFIELD", "ISSPA_FORCES"):
        assert f"%FLAG {flag}" in text
