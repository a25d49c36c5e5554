"""The drop-in command line: argument parsing against the reference's own
putil.c, and the reference's error paths (no GPU needed)."""
import ctypes as C
import os
import subprocess

import pytest

from conftest import REFERENCE

CASES = ["127", "128", "1e6", "1E6", "2e0", "1e", "2M", "3K", "1G", "1T", "1P", "3k", "5m", "1g", "1t", "1p",
         "5b10", "5B3", "0x7F", "0177", "0", "1e20", "1e19", "18446744073709551615", "18446744073709551616",
         "18446744073709551614", "abc", "12Kx", "1.5e6", "-5", "", "42 ", "9e18", "17P", "16p", "4294967295",
         "4294967296", "2147483647", "2147483646", "1k1", "7b", "1e1x", "0x", "99999999999999999999999"]
RANGES = [(127, 0xFFFFFFFFFFFFFFFF - 1), (128, 0xFFFFFFFFFFFFFFFF), (1, 128), (0, 1000)]
RANGES32 = [(127, 0x7FFFFFFF - 1), (128, 0x7FFFFFFF), (1, 128)]


@pytest.fixture(scope="session")
def refputil():
    import oracle
    if os.path.isdir(REFERENCE):
        try:
            oracle.build_ref(REFERENCE)
        except Exception:
            pass
    r = oracle.ref_putil()
    if r is None:
        pytest.skip("reference tree not present: putil.c checker not built")
    return r


def test_parse_uint64_matches_reference(fslib, refputil):
    L = fslib.lib()
    L.fs_parse_uint64.restype = C.c_int
    L.fs_parse_uint64.argtypes = [C.POINTER(C.c_uint64), C.c_char_p, C.c_uint64, C.c_uint64]
    for s in CASES:
        for lo, hi in RANGES:
            a, b = C.c_uint64(0), C.c_uint64(0)
            ra = L.fs_parse_uint64(C.byref(a), s.encode(), lo, hi)
            rb = refputil.parse_uint64(C.byref(b), s.encode(), lo, hi)
            assert (ra, a.value if ra == 0 else None) == (rb, b.value if rb == 0 else None), (s, lo, hi)


def test_parse_uint_matches_reference(fslib, refputil):
    L = fslib.lib()
    L.fs_parse_uint.restype = C.c_int
    L.fs_parse_uint.argtypes = [C.POINTER(C.c_uint32), C.c_char_p, C.c_uint32, C.c_uint32]
    for s in CASES:
        for lo, hi in RANGES32:
            a, b = C.c_uint32(0), C.c_uint32(0)
            ra = L.fs_parse_uint(C.byref(a), s.encode(), lo, hi)
            rb = refputil.parse_uint(C.byref(b), s.encode(), lo, hi)
            assert (ra, a.value if ra == 0 else None) == (rb, b.value if rb == 0 else None), (s, lo, hi)


def _cli(fslib, args, cwd):
    return subprocess.run([fslib.CLI_PATH] + args, cwd=cwd, capture_output=True, text=True, timeout=60)


def test_cli_help_and_bad_arguments(fslib, tmp_path):
    if not os.path.exists(fslib.CLI_PATH):
        pytest.skip("CLI not built")
    r = _cli(fslib, ["-h"], tmp_path)
    assert r.returncode == 1 and "-n #" in r.stdout and "Start factorial n!+-1" in r.stdout
    r = _cli(fslib, ["-n", "1000", "-N", "2000", "-p", "1e6", "-P", "2x"], tmp_path)
    assert r.returncode == 1 and "invalid argument -P 2x" in r.stdout
    r = _cli(fslib, ["-n", "1000", "-N", "2000", "-p", "100", "-P", "2e6"], tmp_path)
    assert r.returncode == 1 and "out of range argument -p 100" in r.stdout
    r = _cli(fslib, ["-v", "129", "-n", "1000"], tmp_path)
    assert r.returncode == 1 and "out of range argument -v 129" in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["-n", "1000", "-N", "2000"], "-p and -P arguments are required"),
    (["-p", "1e6", "-P", "2e6"], "-n and -N arguments are required"),
    (["-n", "3000", "-N", "2000", "-p", "1e6", "-P", "2e6"], "nmin <= nmax is required"),
    (["-n", "1000", "-N", "2000", "-p", "3e6", "-P", "2e6"], "pmin <= pmax is required"),
    (["-n", "2000", "-N", "3000", "-p", "1000", "-P", "2e6"], "pmin must be >= nmin"),
    # -d/--device is accepted and ignored, as in the reference (main.cpp: handled, not used)
    (["-d", "3", "-n", "3000", "-N", "2000", "-p", "1e6", "-P", "2e6"], "nmin <= nmax is required"),
    (["--device=1", "-n", "3000", "-N", "2000", "-p", "1e6", "-P", "2e6"], "nmin <= nmax is required"),
])
def test_cli_range_checks(fslib, tmp_path, args, msg):
    if not os.path.exists(fslib.CLI_PATH):
        pytest.skip("CLI not built")
    r = _cli(fslib, args, tmp_path)
    assert r.returncode == 1
    assert msg in r.stdout
    assert not (tmp_path / "factors.txt").exists()
