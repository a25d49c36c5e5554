"""The drop-in CLI on the GPU: factors.txt, checksum line, checkpoint files,
resume, and the reference's self test."""
import json
import os
import struct
import subprocess

import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cli(fslib, args, cwd, env=None, timeout=900):
    if not os.path.exists(fslib.CLI_PATH):
        pytest.skip("CLI not built")
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([fslib.CLI_PATH] + args, cwd=cwd, capture_output=True, text=True, timeout=timeout,
                          env=e)


def _gold(name):
    with open(os.path.join(GOLD, f"run_{name}.json")) as fh:
        return json.load(fh)


def _state(pmin, pmax, p, checksum, primecount, factorcount, nmin, nmax, last_trickle=0, bad_sum=False):
    """A 72-byte checkpoint record (cl_sieve.h:9-12) with its additive checksum."""
    M = (1 << 64) - 1
    s = (pmin + pmax + p + checksum + primecount + factorcount + last_trickle + nmin + nmax) & M
    if bad_sum:
        s ^= 1
    return struct.pack("<8Q2I", pmin, pmax, p, checksum, primecount, factorcount, last_trickle, s, nmin, nmax)


def _args(g):
    return ["-n", str(g["nmin"]), "-N", str(g["nmax"]), "-p", str(g["pmin"]), "-P", str(g["pmax"]), "-v", "8"]


def test_cli_config1_output_files(fslib, tmp_path):
    g = _gold("config1")
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = (tmp_path / "factors.txt").read_text().splitlines()
    assert lines == g["factors"] + [g["checksum"]]
    assert f"factors {g['factorcount']}, prime count {g['primecount']}, checksum {g['checksum']}" in r.stdout
    # a checkpoint was written, 72 bytes, finished (p == pmax) and self-consistent
    ck = [f for f in ("stateA.ckp", "stateB.ckp") if (tmp_path / f).exists()]
    assert ck
    rec = (tmp_path / ck[0]).read_bytes()
    assert len(rec) == 72
    v = struct.unpack("<8Q2I", rec)
    assert v[2] == g["pmax"] and v[3] == int(g["checksum"], 16) and v[4] == g["primecount"]
    assert v[7] == (sum(v[:7]) + v[8] + v[9]) % (1 << 64)


def test_cli_no_factors_line(fslib, tmp_path):
    g = _gold("near_2p62")
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert (tmp_path / "factors.txt").read_text().splitlines() == ["no factors", g["checksum"]]


def test_cli_resumes_from_checkpoint(fslib, orc, tmp_path):
    """A checkpoint at p = mid plus the factors found below mid: the resumed run
    ends with exactly the uninterrupted run's factors.txt and checksum."""
    g = _gold("config1")
    mid = 1_500_000
    part = orc.run(g["pmin"], mid, g["nmin"], g["nmax"])
    lines = [f"{int(p)} | {abs(int(nc))}!{'+1' if nc > 0 else '-1'}"
             for p, nc in zip(part["factors"]["p"], part["factors"]["nc"])]
    (tmp_path / "factors.txt").write_text("".join(l + "\n" for l in lines))
    (tmp_path / "stateA.ckp").write_bytes(_state(g["pmin"], g["pmax"], mid, part["checksum"], part["primecount"],
                                                 part["factorcount"], g["nmin"], g["nmax"]))
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Resuming from checkpoint in stateA.ckp" in r.stdout
    assert (tmp_path / "factors.txt").read_text().splitlines() == g["factors"] + [g["checksum"]]


def test_cli_resumes_after_a_kill_between_checkpoint_writes(fslib, orc, tmp_path):
    """Killed while writing the newer checkpoint: stateB.ckp is cut short and
    stateA.ckp holds the last complete one (p = mid).  The run resumes from
    stateA.ckp and ends with the uninterrupted run's factors.txt and checksum."""
    g = _gold("config1")
    mid = 1_500_000
    part = orc.run(g["pmin"], mid, g["nmin"], g["nmax"])
    lines = [f"{int(p)} | {abs(int(nc))}!{'+1' if nc > 0 else '-1'}"
             for p, nc in zip(part["factors"]["p"], part["factors"]["nc"])]
    (tmp_path / "factors.txt").write_text("".join(l + "\n" for l in lines))
    (tmp_path / "stateA.ckp").write_bytes(_state(g["pmin"], g["pmax"], mid, part["checksum"], part["primecount"],
                                                 part["factorcount"], g["nmin"], g["nmax"]))
    newer = _state(g["pmin"], g["pmax"], 1_800_000, 1, 2, 3, g["nmin"], g["nmax"])
    (tmp_path / "stateB.ckp").write_bytes(newer[:50])
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Cannot parse stateB.ckp !!!" in r.stdout
    assert "Resuming from checkpoint in stateA.ckp" in r.stdout
    assert (tmp_path / "factors.txt").read_text().splitlines() == g["factors"] + [g["checksum"]]


@pytest.mark.parametrize("name", ["config1", "near_2p62"])
def test_cli_full_disk_on_factors_file(fslib, tmp_path, name):
    """factors.txt on a full disk (/dev/full: opens, every write fails): the
    factor lines (config 1) or the final checksum line (a range without
    factors) cannot be written, and the run ends with EXIT_FAILURE and the
    reference's message (cl_sieve.cpp:539-541, 758-768)."""
    if not os.path.exists("/dev/full"):
        pytest.skip("no /dev/full")
    g = _gold(name)
    os.symlink("/dev/full", tmp_path / "factors.txt")
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 1, r.stdout + r.stderr
    assert "Cannot write to factors.txt !!!" in r.stderr


def test_cli_ignores_corrupt_checkpoint(fslib, tmp_path):
    g = _gold("config1")
    (tmp_path / "stateA.ckp").write_bytes(_state(g["pmin"], g["pmax"], 1_500_000, 5, 7, 0, g["nmin"], g["nmax"],
                                                 bad_sum=True))
    (tmp_path / "stateB.ckp").write_bytes(b"short")
    (tmp_path / "factors.txt").write_text("stale\n")
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Checksum error in stateA.ckp" in r.stdout
    assert "Cannot parse stateB.ckp" in r.stdout
    assert (tmp_path / "factors.txt").read_text().splitlines() == g["factors"] + [g["checksum"]]


def test_cli_finished_workunit(fslib, tmp_path):
    g = _gold("config1")
    (tmp_path / "stateB.ckp").write_bytes(_state(g["pmin"], g["pmax"], g["pmax"], 1, 2, 0, g["nmin"], g["nmax"]))
    r = _cli(fslib, _args(g), tmp_path)
    assert r.returncode == 0
    assert "Workunit complete." in r.stdout


def test_cli_self_test(fslib, tmp_path):
    r = _cli(fslib, ["-s", "-v", "16"], tmp_path, timeout=1800)
    assert r.returncode == 0, r.stdout[-3000:]
    assert r.stdout.count("passed.") == 5
    assert "All test cases completed successfully!" in r.stdout


def test_cli_top_of_the_p_range(fslib, orc, tmp_path):
    """-P 18446744073709551615, the largest value the parser accepts: candidates up to 2^64 - 1."""
    import factsieve_gb300 as fs
    pmin, pmax, nmin, nmax = (1 << 64) - 400_000, (1 << 64) - 1, 1000, 1333
    want = orc.run(pmin, pmax, nmin, nmax)
    lines = fs.SieveResult(want["factors"], want["checksum"], want["primecount"], want["factorcount"]).lines()
    r = _cli(fslib, ["-n", str(nmin), "-N", str(nmax), "-p", str(pmin), "-P", "18446744073709551615", "-v", "4"],
             tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    got = (tmp_path / "factors.txt").read_text().splitlines()
    assert got == (lines or ["no factors"]) + [f"{want['checksum']:016X}"]
    assert f"prime count {want['primecount']}," in r.stdout


@pytest.mark.parametrize("name,argv", [
    ("config2", ["-n", "1e5", "-N", "2e5", "-p", "1e12", "-P", "1001e9"]),          # suffix spellings of 1e12 + 1e9
    ("config3", ["-n", "1e6", "-N", "101e4", "-p", "9223372036854775808", "-P", "9223372037854775808"]),
])
def test_cli_full_config_matches_oracle_fixture(fslib, tmp_path, name, argv):
    """The drop-in CLI over a whole benchmark configuration (1e9-wide p-range):
    factors.txt and the final line equal the oracle's output for the same range
    (tests/golden/run_<name>.json)."""
    path = os.path.join(GOLD, f"run_{name}.json")
    if not os.path.exists(path):
        pytest.skip(f"fixture {name} not generated")
    g = _gold(name)
    r = _cli(fslib, argv + ["-v", "16"], tmp_path)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = (tmp_path / "factors.txt").read_text().splitlines()
    assert lines == (g["factors"] or ["no factors"]) + [g["checksum"]]
    assert f"factors {g['factorcount']}, prime count {g['primecount']}, checksum {g['checksum']}" in r.stdout
