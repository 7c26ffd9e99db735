"""Input readers under corrupted files (CPU).

Seeded mutations of the ADI2 fixture files — truncation at a random line,
deleted or duplicated lines, a numeric field replaced by garbage, a %FLAG line
damaged — fed to the prmtop, isspatop, rst7 and config readers.  Every call
must return OK or one of the library's negative status codes (never crash,
never a positive or unknown code), and a reader that accepts a file must
leave a description it can hand out.

The same cases run a second time against the readers compiled on their own
with AddressSanitizer and UndefinedBehaviorSanitizer (g++), in a subprocess:
any out-of-bounds access or undefined operation fails the test even where it
would not crash.
"""
import ctypes as C
import os
import random
import shutil
import subprocess
import sys

import pytest

from isspa_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
N_CASES = 200
CODES = {0, -1, -2, -3, -4, -5, -6, -7, -8, -9, -10, -11}
READERS = ("prmtop", "isspatop", "rst7", "config")
SOURCE = {"prmtop": "ADI2.prmtop", "isspatop": "ADI2.isspatop", "rst7": "ADI2.rst7", "config": "adi2_config.txt"}
SEED = {"prmtop": 11, "isspatop": 12, "rst7": 13, "config": 14}


def _mutate(lines, rng):
    lines = list(lines)
    kind = rng.randrange(5)
    if kind == 0 and len(lines) > 1:
        lines = lines[:rng.randrange(1, len(lines))]
    elif kind == 1 and len(lines) > 1:
        del lines[rng.randrange(len(lines))]
    elif kind == 2:
        k = rng.randrange(len(lines))
        lines.insert(k, lines[k])
    elif kind == 3:
        k = rng.randrange(len(lines))
        ln = lines[k]
        if ln.strip():
            a = rng.randrange(len(ln))
            b = min(len(ln), a + rng.randrange(1, 17))
            junk = rng.choice(["nan", "inf", "-1e39", "xx", "  ", "99999999", "-7", "1e-45", ""])
            ln = ln[:a] + junk + ln[b:]
        lines[k] = ln
    else:
        flags = [i for i, ln in enumerate(lines) if ln.startswith("%FLAG") or "=" in ln]
        if flags:
            k = rng.choice(flags)
            lines[k] = lines[k][: rng.randrange(len(lines[k]) + 1)]
    return lines


def run_cases(L, which, workdir):
    """Run the mutated inputs of one reader against library L; returns the
    number of files accepted.  L needs only the reader entry points."""
    for name, args, res in (("isspa_read_run_config", [C.c_char_p, C.POINTER(abi.RunConfig)], C.c_int),
                            ("isspa_read_prmtop", [C.c_char_p, C.c_float, C.POINTER(C.c_void_p)], C.c_int),
                            ("isspa_read_isspatop", [C.c_void_p, C.c_char_p], C.c_int),
                            ("isspa_read_rst7", [C.c_void_p, C.c_char_p, C.c_int], C.c_int),
                            ("isspa_system_describe", [C.c_void_p, C.POINTER(abi.SystemDesc)], C.c_int),
                            ("isspa_system_free", [C.c_void_p], None)):
        fn = getattr(L, name)
        fn.argtypes, fn.restype = args, res
    rng = random.Random(SEED[which])
    src = SOURCE[which]
    base = open(os.path.join(GOLDEN, src)).read().splitlines()
    prmtop = os.path.join(GOLDEN, "ADI2.prmtop").encode()
    accepted = 0
    for _ in range(N_CASES):
        p = os.path.join(workdir, src)
        with open(p, "w") as f:
            f.write("\n".join(_mutate(base, rng)) + "\n")
        path = p.encode()
        if which == "config":
            cfg = abi.RunConfig()
            rc = L.isspa_read_run_config(path, C.byref(cfg))
            assert rc in CODES, rc
            accepted += rc == 0
            continue
        h = C.c_void_p()
        if which == "prmtop":
            rc = L.isspa_read_prmtop(path, C.c_float(1.0), C.byref(h))
        else:
            assert L.isspa_read_prmtop(prmtop, C.c_float(1.0), C.byref(h)) == 0
            rc = L.isspa_read_isspatop(h, path) if which == "isspatop" else L.isspa_read_rst7(h, path, 0)
        assert rc in CODES, rc
        if rc == 0 and h.value:
            d = abi.SystemDesc()
            assert L.isspa_system_describe(h, C.byref(d)) in CODES
            assert d.n_atoms >= 0
        if h.value:
            L.isspa_system_free(h)
        accepted += rc == 0
    return accepted


@pytest.mark.parametrize("which", READERS)
def test_readers_survive_corrupted_files(tmp_path, which):
    accepted = run_cases(abi.lib(), which, str(tmp_path))
    print(f"{which}: {accepted} of {N_CASES} mutated files accepted")


def _asan_runtime():
    gxx = shutil.which("g++")
    if not gxx:
        return None, None
    lib = subprocess.run([gxx, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    return gxx, (lib if os.path.isabs(lib) and os.path.exists(lib) else None)


def test_readers_under_address_sanitizer(tmp_path):
    gxx, libasan = _asan_runtime()
    if not libasan:
        pytest.skip("g++ with AddressSanitizer is not available")
    so = tmp_path / "libio_asan.so"
    csrc = os.path.join(ROOT, "isspa-force-cuda_gb300", "csrc")
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-fno-omit-frame-pointer", "-x", "c++", "-D__host__=", "-D__device__=", "-D__forceinline__=inline",
           "-I", os.path.join(ROOT, "include"), "-I", csrc, "-fPIC", "-shared", os.path.join(csrc, "io.cpp"),
           "-o", str(so)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    script = (f"import ctypes, sys; sys.path[:0] = {[HERE, os.path.join(ROOT, 'isspa-force-cuda_gb300')]!r}\n"
              "import test_io_fuzz as T\n"
              f"L = ctypes.CDLL({str(so)!r})\n"
              f"for w in T.READERS: print(w, T.run_cases(L, w, {str(tmp_path)!r}))\n")
    env = dict(os.environ, LD_PRELOAD=libasan, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, env=env, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stderr[-4000:]
    assert "AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr[-4000:]
