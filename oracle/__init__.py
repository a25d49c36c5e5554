"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of the reference FactSieve search
(mfl0p/FactSieve v1.6): candidate generation (kernels/getsegprimes.cl), the
power table (cl_sieve.cpp:773-838), setup (kernels/setup.cl), iterate
(kernels/iterate.cl), check (kernels/check.cl) and the host post-processing
(cl_sieve.cpp:439-554).  Only tests/, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py`` use it, always as the checker.  The shipped
library never imports it.

``ref()`` returns the reference's own CPU arithmetic (verifyprime.c compiled
from the reference tree by ``make -C oracle ref``) when it was built on this
machine, else None.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_REF = os.path.join(_HERE, "_ref", "libverifyprime.so")
_REF_PUTIL = os.path.join(_HERE, "_ref", "libputil.so")
_lock = threading.Lock()
_lib = None
_ref = None


class OFactor(C.Structure):
    """Reference factor record (cl_sieve.h:3-6): u64 p, i32 nc, 4 bytes pad."""

    _fields_ = [("p", C.c_uint64), ("nc", C.c_int32), ("pad", C.c_int32)]


class OResult(C.Structure):
    _fields_ = [
        ("primecount", C.c_uint64),
        ("checksum", C.c_uint64),
        ("factorcount", C.c_uint64),
        ("raw_sum", C.c_uint64),
        ("nhits", C.c_uint64),
        ("ndiscarded", C.c_uint64),
        ("nvalidfail", C.c_uint64),
        ("status", C.c_int64),
    ]


FACTOR_DTYPE = np.dtype([("p", "<u8"), ("nc", "<i4"), ("pad", "<i4")])


def build(force: bool = False) -> str:
    """Compile liboracle.so in place (gcc + OpenMP)."""
    src = os.path.join(_HERE, "oracle.c")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB


def build_ref(ref_dir: str) -> str | None:
    """Compile the reference's verifyprime.c into oracle/_ref when the tree exists."""
    if not os.path.exists(os.path.join(ref_dir, "verifyprime.c")):
        return None
    subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF_DIR={ref_dir}"], check=True)
    return _REF


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB)
            u64, u32, i32 = C.c_uint64, C.c_uint32, C.c_int32
            P64, P32 = C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)
            L.oracle_invert.restype = u64
            L.oracle_invert.argtypes = [u64]
            L.oracle_mmul.restype = u64
            L.oracle_mmul.argtypes = [u64, u64, u64, u64]
            L.oracle_madd.restype = u64
            L.oracle_madd.argtypes = [u64, u64, u64]
            L.oracle_sprp2.restype = C.c_int
            L.oracle_sprp2.argtypes = [u64]
            L.oracle_small_mask.restype = u32
            L.oracle_small_mask.argtypes = [u32, u32]
            L.oracle_find_wheel_offset.restype = None
            L.oracle_find_wheel_offset.argtypes = [P64, C.POINTER(i32)]
            L.oracle_candidates.restype = u64
            L.oracle_candidates.argtypes = [u64, u64, P64, u64]
            L.oracle_candidates_naive.restype = u64
            L.oracle_candidates_naive.argtypes = [u64, u64, P64, u64]
            L.oracle_power_table.restype = u32
            L.oracle_power_table.argtypes = [u32, P64, P32, P32, u32]
            L.oracle_setup.restype = u64
            L.oracle_setup.argtypes = [u64, P64, P32, P32, u32]
            L.oracle_sieve_list.restype = u64
            L.oracle_sieve_list.argtypes = [P64, u64, u32, u32, P64, P32, P32, u32, P64, P64,
                                            C.POINTER(OFactor), u64, P64, P64]
            L.oracle_verify.restype = C.c_int
            L.oracle_verify.argtypes = [u64, u32, i32]
            L.oracle_is_prime.restype = C.c_int
            L.oracle_is_prime.argtypes = [u64]
            L.oracle_postprocess.restype = C.c_int64
            L.oracle_postprocess.argtypes = [C.POINTER(OFactor), u64, P64, P64]
            L.oracle_set_threads.restype = None
            L.oracle_set_threads.argtypes = [C.c_int]
            L.oracle_max_threads.restype = C.c_int
            L.oracle_max_threads.argtypes = []
            L.oracle_run.restype = C.c_int
            L.oracle_run.argtypes = [u64, u64, u32, u32, u64, C.POINTER(OFactor), u64,
                                     C.POINTER(OResult)]
            _lib = L
    return _lib


def ref():
    """The reference's verifyprime.c (m_mul, add, invert, isPrime, verify), or None."""
    global _ref
    if _ref is None and os.path.exists(_REF):
        R = C.CDLL(_REF)
        u64, u32 = C.c_uint64, C.c_uint32
        # C++ symbols of verifyprime.c (x86-64 and aarch64 Itanium mangling)
        R.m_mul = R._Z5m_mulmmmm
        R.m_mul.restype = u64
        R.m_mul.argtypes = [u64, u64, u64, u64]
        R.add = R._Z3addmmm
        R.add.restype = u64
        R.add.argtypes = [u64, u64, u64]
        R.invert = R._Z6invertm
        R.invert.restype = u64
        R.invert.argtypes = [u64]
        R.isPrime = R._Z7isPrimem
        R.isPrime.restype = C.c_bool
        R.isPrime.argtypes = [u64]
        R.verify = R._Z6verifymji
        R.verify.restype = C.c_bool
        R.verify.argtypes = [u64, u32, C.c_int32]
        _ref = R
    return _ref


def ref_putil():
    """The reference's putil.c (parse_uint64 / parse_uint), or None when not built here."""
    if not os.path.exists(_REF_PUTIL):
        return None
    R = C.CDLL(_REF_PUTIL)
    R.parse_uint64.restype = C.c_int
    R.parse_uint64.argtypes = [C.POINTER(C.c_uint64), C.c_char_p, C.c_uint64, C.c_uint64]
    R.parse_uint.restype = C.c_int
    R.parse_uint.argtypes = [C.POINTER(C.c_uint32), C.c_char_p, C.c_uint32, C.c_uint32]
    return R


def _p64(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _p32(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return lib().oracle_max_threads()


def candidates(low: int, high: int, naive: bool = False) -> np.ndarray:
    """Sorted candidate list of the reference getsegprimes over [low, high)."""
    L = lib()
    fn = L.oracle_candidates_naive if naive else L.oracle_candidates
    width = max(0, high - low)
    cap = width // 3 + 64
    out = np.zeros(cap, dtype=np.uint64)
    n = fn(low, high, _p64(out), cap)
    if n > cap:
        out = np.zeros(n, dtype=np.uint64)
        n = fn(low, high, _p64(out), n)
    return out[:n].copy()


def find_wheel_offset(start: int):
    s = C.c_uint64(start)
    i = C.c_int32(0)
    lib().oracle_find_wheel_offset(C.byref(s), C.byref(i))
    return s.value, i.value


def power_table(nmin: int):
    """Reference compressed power table for nmin!: (primes u64, exp u32, topbit u32)."""
    L = lib()
    cap = nmin // 2 + 64
    tp = np.zeros(cap, dtype=np.uint64)
    te = np.zeros(cap, dtype=np.uint32)
    tb = np.zeros(cap, dtype=np.uint32)
    m = L.oracle_power_table(nmin, _p64(tp), _p32(te), _p32(tb), cap)
    assert m <= cap
    return tp[:m].copy(), te[:m].copy(), tb[:m].copy()


def setup(p: int, table) -> int:
    tp, te, tb = table
    return lib().oracle_setup(p, _p64(tp), _p32(te), _p32(tb), len(tp))


def sieve_list(cand: np.ndarray, nmin: int, nmax: int, table=None, want_residues=False):
    """setup + iterate + check over a candidate list.

    Returns dict(raw_sum, nvalidfail, hits (structured array, unsorted), s6, s7)."""
    L = lib()
    cand = np.ascontiguousarray(cand, dtype=np.uint64)
    if table is None:
        table = power_table(nmin)
    tp, te, tb = table
    raw = C.c_uint64(0)
    bad = C.c_uint64(0)
    fcap = 1 << 16
    while True:
        fac = (OFactor * fcap)()
        s6 = np.zeros(len(cand), dtype=np.uint64) if want_residues else None
        s7 = np.zeros(len(cand), dtype=np.uint64) if want_residues else None
        raw.value = 0
        bad.value = 0
        nh = L.oracle_sieve_list(_p64(cand), len(cand), nmin, nmax, _p64(tp), _p32(te), _p32(tb),
                                 len(tp), C.byref(raw), C.byref(bad), fac, fcap,
                                 _p64(s6) if want_residues else None,
                                 _p64(s7) if want_residues else None)
        if nh <= fcap:
            break
        fcap = int(nh) + 16
    hits = np.frombuffer(fac, dtype=FACTOR_DTYPE, count=nh).copy()
    return {"raw_sum": raw.value, "nvalidfail": bad.value, "hits": hits, "s6": s6, "s7": s7}


def run(pmin: int, pmax: int, nmin: int, nmax: int, seg_width: int = 10_000_000,
        fcap: int = 1 << 20):
    """Whole reference search; returns dict with primecount, checksum, factorcount,
    raw_sum, nhits, ndiscarded, nvalidfail, status and the kept factors (sorted)."""
    L = lib()
    fac = (OFactor * fcap)()
    res = OResult()
    L.oracle_run(pmin, pmax, nmin, nmax, seg_width, fac, fcap, C.byref(res))
    out = {k: getattr(res, k) for k, _ in OResult._fields_}
    kept = np.frombuffer(fac, dtype=FACTOR_DTYPE, count=min(res.factorcount, fcap)).copy()
    out["factors"] = kept
    return out


def is_prime(p: int) -> bool:
    return bool(lib().oracle_is_prime(p))


def verify(p: int, n: int, c: int) -> bool:
    return bool(lib().oracle_verify(p, n, c))


def mmul(a, b, p, q):
    return lib().oracle_mmul(a, b, p, q)


def invert(p):
    return lib().oracle_invert(p)


def sprp2(n):
    return bool(lib().oracle_sprp2(n))


def small_mask(q, r):
    return lib().oracle_small_mask(q, r)


def postprocess(hits: np.ndarray):
    """Reference host post-processing of raw hits: returns (kept, checksum_add, ndiscarded)
    where checksum_add is the n + c sum, or None if a hit fails CPU verification."""
    L = lib()
    n = len(hits)
    fac = (OFactor * max(n, 1))()
    arr = np.frombuffer(fac, dtype=FACTOR_DTYPE, count=n)
    arr[:] = hits
    cs = C.c_uint64(0)
    disc = C.c_uint64(0)
    k = L.oracle_postprocess(fac, n, C.byref(cs), C.byref(disc))
    if k < 0:
        return None
    return arr[:k].copy(), cs.value, disc.value


def exact_small(pmin: int, pmax: int, nmin: int, nmax: int) -> dict:
    """The search by its definition, in pure Python, for small cases at the
    edge of the domain where the reference's own code does not compute it:

    * nmin in {2, 3}: getPower (cl_sieve.cpp:773-788) leaves curBit at 2^31
      when the power of 2 in nmin! is 1, so setup.cl:62-72 squares 2 thirty-one
      more times and the starting residue is not nmin!;
    * nmin = 1: the power table is empty and setup reads an unset entry 0;
    * hits with n < 34: the CPU verifier (verifyprime.c:146-173) starts from
      34! and rejects them, so the reference stops with a verification error.

    Same candidate set (``candidates``); hits are (p, -n) when p | n! - 1 and
    (p, +n) when p | n! + 1 for n in [nmin, nmax); raw_sum adds nmax! R + nmax R
    (R = 2^64, residues mod p) per candidate; the checksum adds n + c for each
    hit whose p is prime (all hits are true, so none is rejected)."""
    cand = [int(x) for x in candidates(pmin, pmax)]
    R = 1 << 64
    M = (1 << 64) - 1
    hits, raw = [], 0
    for p in cand:
        r = 1
        for k in range(2, nmin + 1):
            r = r * k % p
        for n in range(nmin, nmax):
            if r == 1:
                hits.append((p, -n))
            elif r == p - 1:
                hits.append((p, n))
            r = r * (n + 1) % p
        raw += r * R % p + nmax * R % p
    kept = [(p, nc) for p, nc in sorted(hits, key=lambda h: (h[0], abs(h[1]), h[1])) if is_prime(p)]
    cs = raw
    for _, nc in kept:
        cs += (abs(nc) + (1 if nc > 0 else -1)) & 0xFFFFFFFF
    return {"primecount": len(cand), "raw_sum": raw & M, "checksum": cs & M, "factorcount": len(kept),
            "factors": kept, "nhits": len(hits)}
