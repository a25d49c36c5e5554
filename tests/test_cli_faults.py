"""Host fault cases of the command line, no GPU needed: damaged checkpoint
files and an unusable factors.txt.

The reference keeps two checkpoint files and writes the other one each time
(cl_sieve.cpp:100-129), so a run killed while writing one still has the
other; on start it reads both, rejects a file it cannot parse, one for other
ranges and one whose additive state_sum does not match, and resumes from the
newer good one (cl_sieve.cpp:132-222).  A resumed workunit that is already
finished exits at once (cl_sieve.cpp:1000-1013); a factors.txt that cannot be
opened ends the run with EXIT_FAILURE (cl_sieve.cpp:1016-1022).  Every case
here stops before the device is opened.
"""
import os
import struct
import subprocess

import pytest

PMIN, PMAX, NMIN, NMAX = 1_000_000, 2_000_000, 1000, 2000
ARGS = ["-n", str(NMIN), "-N", str(NMAX), "-p", str(PMIN), "-P", str(PMAX)]


def _cli(fslib, cwd):
    if not os.path.exists(fslib.CLI_PATH):
        pytest.skip("CLI not built")
    return subprocess.run([fslib.CLI_PATH] + ARGS, cwd=cwd, capture_output=True, text=True, timeout=60)


def _state(p, checksum=0x188AA0823D, primecount=70456, factorcount=106, pmin=PMIN, pmax=PMAX, nmin=NMIN,
           nmax=NMAX, last_trickle=1, bad_sum=False):
    """A 72-byte checkpoint record (cl_sieve.h:9-12) with its additive checksum."""
    M = (1 << 64) - 1
    s = (pmin + pmax + p + checksum + primecount + factorcount + last_trickle + nmin + nmax) & M
    if bad_sum:
        s ^= 1
    return struct.pack("<8Q2I", pmin, pmax, p, checksum, primecount, factorcount, last_trickle, s, nmin, nmax)


FACTORS = "1000003 | 1234!+1\n"   # whatever a finished run left there: a resume must not touch it


def _finished_a(tmp_path):
    (tmp_path / "stateA.ckp").write_bytes(_state(PMAX))
    (tmp_path / "factors.txt").write_text(FACTORS)


def test_truncated_checkpoint_falls_back_to_the_other(fslib, tmp_path):
    """A run killed while writing stateB.ckp leaves it short: it is rejected
    and the run resumes from stateA.ckp."""
    _finished_a(tmp_path)
    (tmp_path / "stateB.ckp").write_bytes(_state(PMAX)[:40])
    r = _cli(fslib, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Cannot parse stateB.ckp !!!" in r.stdout
    assert "Resuming from checkpoint in stateA.ckp" in r.stdout
    assert "Workunit complete." in r.stdout
    assert (tmp_path / "factors.txt").read_text() == FACTORS


def test_checkpoint_with_a_bad_sum_is_rejected(fslib, tmp_path):
    """A whole record whose state_sum does not add up (garbage, a torn write)."""
    _finished_a(tmp_path)
    (tmp_path / "stateB.ckp").write_bytes(_state(PMAX + 0, bad_sum=True))
    r = _cli(fslib, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Checksum error in stateB.ckp !!!" in r.stdout
    assert "Resuming from checkpoint in stateA.ckp" in r.stdout


def test_garbage_checkpoint_is_rejected(fslib, tmp_path):
    _finished_a(tmp_path)
    (tmp_path / "stateB.ckp").write_bytes(os.urandom(72))
    r = _cli(fslib, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert ("Invalid checkpoint file stateB.ckp !!!" in r.stdout or "Checksum error in stateB.ckp !!!" in r.stdout)
    assert "Workunit complete." in r.stdout


def test_checkpoint_of_other_ranges_is_rejected(fslib, tmp_path):
    _finished_a(tmp_path)
    (tmp_path / "stateB.ckp").write_bytes(_state(PMAX, nmax=NMAX + 1))
    r = _cli(fslib, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Invalid checkpoint file stateB.ckp !!!" in r.stdout
    assert "Resuming from checkpoint in stateA.ckp" in r.stdout


@pytest.mark.parametrize("newer", ["A", "B"])
def test_the_newer_good_checkpoint_wins(fslib, tmp_path, newer):
    """Killed between the two writes: both files are good, the one with the
    larger p (finished here) is taken."""
    older = "B" if newer == "A" else "A"
    (tmp_path / f"state{newer}.ckp").write_bytes(_state(PMAX))
    (tmp_path / f"state{older}.ckp").write_bytes(_state(1_500_000, checksum=5, primecount=30000, factorcount=50))
    (tmp_path / "factors.txt").write_text(FACTORS)
    r = _cli(fslib, tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"Resuming from checkpoint in state{newer}.ckp" in r.stdout
    assert f"Current p: {PMAX}" in r.stdout
    assert "Workunit complete." in r.stdout


def test_unopenable_results_file_fails(fslib, tmp_path):
    """A fresh start truncates factors.txt; when it cannot be opened (here it
    is a directory) the run ends with EXIT_FAILURE and the reference's message."""
    (tmp_path / "factors.txt").mkdir()
    r = _cli(fslib, tmp_path)
    assert r.returncode == 1
    assert "Cannot open factors.txt !!!" in r.stderr
