"""Host-side tests (no GPU): the C ABI library, input readers, error paths."""
import ctypes as C
import os
import re
import shutil

import numpy as np
import pytest

import isspa_gb300 as ig
from isspa_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    src = open(os.path.join(ROOT, "include", "isspa_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*([a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 40
    L = C.CDLL(abi.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {s[0] for s in abi.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_reference_call_names_present():
    L = abi.lib()
    for n in ["isspa_force_cuda", "nonbond_force_cuda", "bond_force_cuda", "angle_force_cuda",
              "dih_force_cuda", "leapfrog_cuda", "us_force_cuda"]:
        assert hasattr(L, n)


def test_struct_sizes_match_header():
    # isspa_system_desc: count of members as declared; the ctypes layout must line up
    assert C.sizeof(abi.SystemDesc) % 8 == 0
    assert abi.SystemDesc.seed.offset + 8 == C.sizeof(abi.SystemDesc)
    assert C.sizeof(abi.RunConfig) == 10 * 512 + 7 * 4 + 8 * 4


def test_run_config_parse():
    cfg = ig.read_run_config(os.path.join(GOLDEN, "adi2_config.txt"))
    assert cfg.prmtop == b"ADI2.prmtop"
    assert cfg.n_mc == 1000 and cfg.n_steps == 1 and cfg.seed == 8622
    assert abs(cfg.box - 200.0) < 1e-6
    assert abs(cfg.kT - 298.0 * 0.00198717) < 1e-6
    assert abs(cfg.dt - 0.002 * 20.455) < 1e-7
    assert cfg.pnu_set == 0 and cfg.pnu == 0.0


def test_config_prefix_and_comment_semantics(tmp_path):
    p = tmp_path / "c.txt"
    # velRstFile must not be read as velRst; text after a leading '#' is parsed
    # like the reference's strtok does; pnu given
    p.write_text("velRstFile = v.rst\nvelRst = 1\n#nMC = 7\npnu = 0.02 # comment\n")
    cfg = ig.read_run_config(str(p))
    assert cfg.vel_rst_file == b"v.rst"
    assert cfg.vel_rst == 1
    assert cfg.n_mc == 7
    assert cfg.pnu_set == 1 and abs(cfg.pnu - 0.02) < 1e-9


def test_adi2_prmtop_semantics(adi2):
    s = adi2
    assert s.n_atoms == 44 and s.n_lj_types == 7
    assert len(s.bond_atoms) == 42 and len(s.angle_atoms) == 72 and len(s.dih_atoms) == 134
    assert len(s.excl_list) == 198 and s.n_excl_cum[-1] == 198
    # H masses reset to 12 (read_prmtop.cpp:144-146), raw masses kept
    assert np.all(s.vel[:, 3] >= 2.0)
    assert np.any(s.raw_mass < 2.0)
    # bond constants doubled (read_prmtop.cpp:233)
    assert np.all(s.bond_params[:, 0] > 0)
    # charges: Amber units / sqrt(eps) with eps = 1
    assert abs(s.pos[0, 3] - 2.0463643) < 1e-6
    # isspatop: 16 types, 120 rows, grid from the first two rows
    assert len(s.rmax) == 16 and s.g_table.shape == (16, 120)
    assert abs(s.g_r0 - 0.05) < 1e-7 and abs(s.g_dr - 0.1) < 1e-6
    assert s.isspa_type.min() == 0 and s.isspa_type.max() == 15


def test_us_config_parse(tmp_path, adi2):
    p = tmp_path / "us.cfg"
    p.write_text(open(os.path.join(GOLDEN, "ADI2.us")).read().replace("XXX", "7.5"))
    h = C.c_void_p()
    L = abi.lib()
    abi.check(L.isspa_read_prmtop(os.path.join(GOLDEN, "ADI2.prmtop").encode(), 1.0, C.byref(h)))
    cv = C.create_string_buffer(256)
    abi.check(L.isspa_read_us_config(h, str(p).encode(), cv, 256))
    d = abi.SystemDesc()
    abi.check(L.isspa_system_describe(h, C.byref(d)))
    s = ig.System.from_desc(d)
    L.isspa_system_free(h)
    assert s.us_on == 1 and abs(s.us_k - 20.0) < 1e-6 and abs(s.us_x0 - 7.5) < 1e-6
    assert len(s.bias_list) == 44 and s.bias_list[0].tolist() == [0, 0] and s.bias_list[-1].tolist() == [43, 1]
    assert cv.value == b"ADI2.equil.window.7.5.dat"


@pytest.mark.parametrize("mutate,code", [
    (lambda t: t.replace("%FLAG CHARGE", "%FLAG CHARGX"), abi.ERR_PARSE),  # missing section
    (lambda t: t[: t.index("%FLAG MASS") + 200], abi.ERR_PARSE),           # truncated file
])
def test_malformed_prmtop_is_an_error(tmp_path, mutate, code):
    src = open(os.path.join(GOLDEN, "ADI2.prmtop")).read()
    p = tmp_path / "bad.prmtop"
    p.write_text(mutate(src))
    h = C.c_void_p()
    assert abi.lib().isspa_read_prmtop(str(p).encode(), 1.0, C.byref(h)) == code


def test_missing_files_are_io_errors(tmp_path):
    h = C.c_void_p()
    assert abi.lib().isspa_read_prmtop(str(tmp_path / "nope").encode(), 1.0, C.byref(h)) == abi.ERR_IO
    cfg = abi.RunConfig()
    assert abi.lib().isspa_read_run_config(str(tmp_path / "nope").encode(), C.byref(cfg)) == abi.ERR_IO


def test_malformed_isspatop_is_an_error(tmp_path):
    src = open(os.path.join(GOLDEN, "ADI2.isspatop")).read()
    h = C.c_void_p()
    L = abi.lib()
    abi.check(L.isspa_read_prmtop(os.path.join(GOLDEN, "ADI2.prmtop").encode(), 1.0, C.byref(h)))
    try:
        for bad in [src.replace("%FLAG ISSPA_FORCES", "%FLAG XSSPA_FORCES"),
                    src.replace("  1.19500000e+01", "  nan            ", 1)]:
            p = tmp_path / "bad.isspatop"
            p.write_text(bad)
            assert L.isspa_read_isspatop(h, str(p).encode()) == abi.ERR_PARSE
    finally:
        L.isspa_system_free(h)


def test_engine_create_rejects_bad_descriptions(adi2):
    bad = adi2.copy()
    bad.lj_type = bad.lj_type.copy()
    bad.lj_type[3] = 99
    with pytest.raises(ig.IsspaError) as e:
        ig.Engine(bad)
    assert e.value.status == abi.ERR_ARG
    bad = adi2.copy()
    bad.box = 0.0
    with pytest.raises(ig.IsspaError):
        ig.Engine(bad)


def test_batch_requires_a_shared_force_field():
    a = ig.synth.config_small(seed=1)
    b = a.copy()
    b.rmax = b.rmax * 1.01
    if ig.abi.device_count() == 0:
        pytest.skip("engine creation needs a device after validation")
    with pytest.raises(ig.IsspaError) as e:
        ig.Engine([a, b])
    assert e.value.status == abi.ERR_UNSUPPORTED


def test_synthetic_generator_recipe():
    s = ig.synth.config_small(seed=5)
    assert s.n_atoms == 44 and s.n_mc == 20 and s.box == 40.0
    q = s.pos[:, 3].reshape(2, 22)
    assert np.allclose(q.sum(1), 0.0, atol=1e-3)
    assert np.abs(q).max() <= 0.6 * 18.2223 * 2
    assert len(s.bond_atoms) == 42 and np.allclose(s.bond_params, [[600.0, 1.5]])
    # self-avoiding and non-overlapping chains
    x = s.pos[:, :3]
    d = x[:, None] - x[None]
    d -= s.box * np.round(d / s.box)
    r = np.sqrt((d ** 2).sum(-1))
    idx = np.arange(s.n_atoms)
    far = np.abs(idx[:, None] - idx[None]) >= 4
    assert r[far].min() >= 2.99
    assert s.pnu == pytest.approx(0.02)
