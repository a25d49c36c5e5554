"""Generate the golden fixtures under tests/golden/ from the CPU oracle.

    python tests/golden/make_golden.py [case ...]      (default: the quick cases)
    python tests/golden/make_golden.py --all            (adds the long ones)
    python tests/golden/make_golden.py config4_slices   (the 64-job mix on 1/1000 p-slices)

Each case writes tests/golden/run_<name>.json with the reference-visible
result of the whole search (primecount, checksum, factorcount), the raw
device-side quantities (sum of s6+s7, hit count) and the kept factor list
(inline when short, else as a SHA-256 of its factors.txt lines).

The five self-test ranges and their golden triples are the reference's own
(cl_sieve.cpp:1283-1364); the script refuses to write a self-test fixture
whose triple disagrees with them, so every fixture derived from the oracle
comes from an oracle pinned to the reference.  The benchmark workloads
(config 1-3: the plain small, plain large and top-of-u64 sieves) have no
reference goldens: their fixtures are oracle output.

Also writes candidates_small.json: exact candidate lists (reference
getsegprimes semantics) for a few short p-ranges, used by the GPU parity
tests of the candidate generator.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

# (name, pmin, pmax, nmin, nmax, reference golden (factorcount, primecount, checksum) or None)
CASES = {
    "selftest1": (100_000_000, 101_000_000, 1_000_000, 2_000_000, (1071, 54211, 0x000004F4F744CA97)),
    "selftest2": (1_000_000_000_000, 1_000_010_000_000, 10_000, 2_000_000, (3, 361727, 0x05052A2D65F3D735)),
    "selftest3": (127, 100_000, 127, 1_000_000, (42770, 9566, 0x0000000065C074F0)),
    "selftest4": (2_000_000_000_000, 2_000_010_000_000, 2_000_000, 6_000_000, (3, 352866, 0x09C9742A908451EB)),
    "selftest5": (1_000_000_000_000, 1_000_001_000_000, 100_000_000, 110_000_000, (3, 36249, 0x0081056DC98DA092)),
    # plain sieve, small: n in [1000, 2000), p in [1e6, 2e6)
    "config1": (1_000_000, 2_000_000, 1000, 2000, None),
    # plain sieve, large: n in [1e5, 2e5), p in [1e12, 1e12 + 1e9)
    "config2": (1_000_000_000_000, 1_001_000_000_000, 100_000, 200_000, None),
    # top of the 64-bit range: p in [2^63, 2^63 + 1e9), n in [1e6, 1.01e6)
    "config3": (1 << 63, (1 << 63) + 1_000_000_000, 1_000_000, 1_010_000, None),
    # a 1/100 slice of config 2 and 3 (used by quicker GPU tests and the CPU baseline)
    "config2_slice100": (1_000_000_000_000, 1_000_010_000_000, 100_000, 200_000, None),
    "config3_slice100": (1 << 63, (1 << 63) + 10_000_000, 1_000_000, 1_010_000, None),
    # edge cases
    "wilson_small": (127, 5_000, 127, 20_000, None),          # p <= nmax everywhere
    "top_of_u64": ((1 << 64) - 2_000_000, (1 << 64) - 1, 127, 1_127, None),
    "near_2p32": ((1 << 32) - 500_000, (1 << 32) + 500_000, 1000, 3000, None),
    "near_2p62": ((1 << 62) - 300_000, (1 << 62) + 300_000, 2000, 3000, None),
    "single_n": (10_000_000, 10_100_000, 5000, 5001, None),
    "nmin_eq_nmax": (10_000_000, 10_050_000, 5000, 5000, None),
}
QUICK = ["selftest3", "config1", "wilson_small", "top_of_u64", "near_2p32", "near_2p62",
         "single_n", "nmin_eq_nmax"]
SLOW = ["selftest1", "selftest5", "config2_slice100", "config3_slice100", "selftest2",
        "selftest4", "config3", "config2"]


def factor_lines(f):
    lines = []
    for p, nc in zip(f["p"].tolist(), f["nc"].tolist()):
        lines.append(f"{p} | {abs(nc)}!{'+1' if nc > 0 else '-1'}")
    return lines


def run_case(name):
    pmin, pmax, nmin, nmax, gold = CASES[name]
    t0 = time.time()
    r = oracle.run(pmin, pmax, nmin, nmax, seg_width=10_000_000)
    dt = time.time() - t0
    assert r["status"] == 0, (name, r["status"])
    assert r["nvalidfail"] == 0
    if gold is not None:
        fc, pc, cs = gold
        got = (r["factorcount"], r["primecount"], r["checksum"])
        if got != (fc, pc, cs):
            raise SystemExit(f"{name}: oracle {got} != reference golden {(fc, pc, cs)}")
    lines = factor_lines(r["factors"])
    rec = {
        "name": name, "pmin": pmin, "pmax": pmax, "nmin": nmin, "nmax": nmax,
        "primecount": r["primecount"], "checksum": f"{r['checksum']:016X}",
        "factorcount": r["factorcount"], "raw_sum": f"{r['raw_sum']:016X}",
        "nhits": r["nhits"], "ndiscarded": r["ndiscarded"],
        "factors_sha256": hashlib.sha256("\n".join(lines).encode()).hexdigest(),
        "reference_golden": gold is not None,
        "oracle_seconds": round(dt, 1), "oracle_threads": oracle.max_threads(),
    }
    if len(lines) <= 2000:
        rec["factors"] = lines
    with open(os.path.join(HERE, f"run_{name}.json"), "w") as fh:
        json.dump(rec, fh, indent=1)
    print(f"{name}: primecount {rec['primecount']} factors {rec['factorcount']} "
          f"checksum {rec['checksum']} ({dt:.1f} s)", flush=True)


def write_config4_slices(div=1000):
    """The 64-job mix (jobs_config4.json, seed 1), each job's p-range cut to its
    first 1/div (at least 2000 wide), searched job by job with the oracle:
    run_config4_slices.json holds each sliced job and its result."""
    with open(os.path.join(HERE, "jobs_config4.json")) as fh:
        jobs = [tuple(j) for j in json.load(fh)["jobs"]]
    out = []
    t0 = time.time()
    for p0, p1, n0, n1 in jobs:
        w = max((p1 - p0) // div, 2000)
        r = oracle.run(p0, p0 + w, n0, n1, seg_width=10_000_000)
        assert r["status"] == 0 and r["nvalidfail"] == 0
        out.append({"pmin": p0, "pmax": p0 + w, "nmin": n0, "nmax": n1, "primecount": r["primecount"],
                    "raw_sum": f"{r['raw_sum']:016X}", "checksum": f"{r['checksum']:016X}",
                    "factorcount": r["factorcount"], "nhits": r["nhits"], "factors": factor_lines(r["factors"])})
    dt = time.time() - t0
    with open(os.path.join(HERE, "run_config4_slices.json"), "w") as fh:
        json.dump({"name": "config4_slices", "slice": f"first 1/{div} of each job's p-range (>= 2000 wide)",
                   "oracle_seconds": round(dt, 1), "oracle_threads": oracle.max_threads(), "jobs": out}, fh,
                  indent=1)
    print(f"run_config4_slices.json: {len(out)} jobs, {sum(j['primecount'] for j in out)} candidates "
          f"({dt:.1f} s)", flush=True)


def write_candidates():
    ranges = [
        (127, 20_000), (1_000_000, 1_030_000), ((1 << 32) - 20_000, (1 << 32) + 20_000),
        ((1 << 62) - 3_000, (1 << 62) + 3_000), ((1 << 63) - 3_000, (1 << 63) + 3_000),
        ((1 << 64) - 30_000, (1 << 64) - 1), (1_000_000_000_000, 1_000_000_050_000),
        (127, 128), (129, 130), (4_294_967_297, 4_294_967_298),
    ]
    out = []
    for lo, hi in ranges:
        c = oracle.candidates(lo, hi)
        out.append({"low": lo, "high": hi, "candidates": [int(x) for x in c]})
    with open(os.path.join(HERE, "candidates_small.json"), "w") as fh:
        json.dump(out, fh)
    print("candidates_small.json:", sum(len(o["candidates"]) for o in out), "candidates")


if __name__ == "__main__":
    args = sys.argv[1:]
    if args == ["--all"]:
        names = QUICK + SLOW
    elif args:
        names = args
    else:
        names = QUICK
    if not args or "--all" in args:
        write_candidates()
    if "config4_slices" in names or "--all" in args:
        write_config4_slices()
    for n in names:
        if n != "config4_slices":
            run_case(n)
