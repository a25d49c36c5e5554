"""factsieve_gb300 -- GB300-native FactSieve sieve.

Python front end of libfactsieve.so (C ABI in include/factsieve.h).  The
search mirrors the reference's cl_sieve() (cl_sieve.cpp:918-1270): the GPU
produces candidates, residues and hits; the host sorts and verifies hits,
drops 2-PRP factors, and folds n + c into the checksum (cl_sieve.cpp:439-554).

There is no CPU fallback: every entry point needs the compiled library, and
the search entry points need a CUDA device.  A missing library raises
``LibraryMissing``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from dataclasses import dataclass, field

import numpy as np

__all__ = ["lib", "Context", "Tuning", "SieveResult", "FSError", "LibraryMissing", "sieve",
           "power_table", "setup_plan", "is_prime", "verify_factor", "postprocess",
           "find_wheel_offset", "candidate_capacity", "walk_state_words", "FACTOR_DTYPE", "COUNTERS_DTYPE"]

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libfactsieve.so")
CLI_PATH = os.path.join(_HERE, "bin", "factsieve")

FS_OK, FS_E_ARG, FS_E_CUDA, FS_E_OVERFLOW, FS_E_VALIDATION = 0, 1, 2, 3, 4
FS_E_TABLE, FS_E_NOMEM, FS_E_VERIFY, FS_E_STATE, FS_E_LIMIT = 5, 6, 7, 8, 10
FLAG_VALIDATION, FLAG_CAND_OVERFLOW, FLAG_HIT_OVERFLOW, FLAG_TABLE = 1, 2, 4, 8

FACTOR_DTYPE = np.dtype([("p", "<u8"), ("nc", "<i4"), ("pad", "<i4")])
COUNTERS_DTYPE = np.dtype([("raw_sum", "<u8"), ("primecount", "<u8"), ("ncand", "<u4"),
                           ("nhits", "<u4"), ("flags", "<u4"), ("maxcand", "<u4")])


class LibraryMissing(RuntimeError):
    pass


class FSError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {_strerror(code)} ({code})" if what else f"{_strerror(code)} ({code})")


class Factor(C.Structure):
    _fields_ = [("p", C.c_uint64), ("nc", C.c_int32), ("pad", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("sieve_launches", C.c_uint64), ("gen_launches", C.c_uint64),
                ("sieve_ms", C.c_double), ("gen_ms", C.c_double), ("batch_launches", C.c_uint64),
                ("batch_ms", C.c_double)]


class Job(C.Structure):
    _fields_ = [("pmin", C.c_uint64), ("pmax", C.c_uint64), ("nmin", C.c_uint32), ("nmax", C.c_uint32)]


class JobResult(C.Structure):
    _fields_ = [("raw_sum", C.c_uint64), ("primecount", C.c_uint64), ("nhits", C.c_uint64),
                ("flags", C.c_uint32), ("pad", C.c_uint32)]


class Tuning(C.Structure):
    _fields_ = [("sieve_blocks_per_sm", C.c_uint32), ("gen_blocks_per_sm", C.c_uint32),
                ("max_steps_per_launch", C.c_uint32), ("setup_chunks", C.c_uint32),
                ("sieve_variant", C.c_uint32), ("sieve_block_threads", C.c_uint32),
                ("batch_tile_candidates", C.c_uint32)]


class TuneResult(C.Structure):
    _fields_ = [("tuning", Tuning), ("seg_width", C.c_uint64), ("seg_capacity", C.c_uint64),
                ("setup_words", C.c_uint32), ("steps_per_launch", C.c_uint32), ("rate", C.c_double),
                ("shapes_tried", C.c_uint32), ("from_cache", C.c_uint32)]


_lock = threading.Lock()
_lib = None


def _declare(L):
    u64, u32, i32, vp = C.c_uint64, C.c_uint32, C.c_int32, C.c_void_p
    P64, P32, PI32 = C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
    sig = {
        "fs_version": (C.c_int, []),
        "fs_strerror": (C.c_char_p, [C.c_int]),
        "fs_last_error": (C.c_char_p, [vp]),
        "fs_device_count": (C.c_int, [C.POINTER(C.c_int)]),
        "fs_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "fs_destroy": (C.c_int, [vp]),
        "fs_set_stream": (C.c_int, [vp, vp]),
        "fs_get_stream": (vp, [vp]),
        "fs_set_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
        "fs_get_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
        "fs_device_info": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), P64]),
        "fs_synchronize": (C.c_int, [vp]),
        "fs_search_begin": (C.c_int, [vp, u64, u64, u32, u32, u32]),
        "fs_search_segment": (C.c_int, [vp, u64, u64]),
        "fs_search_collect": (C.c_int, [vp, C.POINTER(Factor), u64, P64, P64, P64, P32]),
        "fs_search_range": (C.c_int, [vp, u64, u64, u64]),
        "fs_candidate_capacity": (u64, [u64, u64]),
        "fs_getsegprimes": (C.c_int, [vp, u64, u64, vp, u32, vp]),
        "fs_setup": (C.c_int, [vp, vp, u32, vp, u32, vp]),
        "fs_iterate": (C.c_int, [vp, vp, u32, vp, vp, u32, u32, vp, u32]),
        "fs_check": (C.c_int, [vp, vp, u32, vp, vp, u32]),
        "fs_table_check": (C.c_int, [vp, vp, vp, u32, P64]),
        "fs_plan_check": (C.c_int, [vp, vp, vp, u32, vp, vp, u32, u64, P64]),
        "fs_bench_int_pipe": (C.c_int, [vp, u32, u32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "fs_search_pending": (C.c_int, [vp, P64]),
        "fs_walk_step": (C.c_int, [u64, u64, u32]),
        "fs_setup_form": (C.c_int, [u64, u64]),
        "fs_set_timing": (C.c_int, [vp, C.c_int]),
        "fs_get_stats": (C.c_int, [vp, C.POINTER(Stats)]),
        "fs_reset_stats": (C.c_int, [vp]),
        "fs_batch_prepare": (C.c_int, [vp, C.POINTER(Job), u32, u32]),
        "fs_batch_launch": (C.c_int, [vp]),
        "fs_batch_collect": (C.c_int, [vp, C.POINTER(JobResult), C.POINTER(Factor), u64, P64]),
        "fs_batch_release": (C.c_int, [vp]),
        "fs_autotune": (C.c_int, [vp, u64, u64, u32, u32, C.c_double, C.c_char_p, C.POINTER(TuneResult)]),
        "fs_autotune_batch": (C.c_int, [vp, C.POINTER(Job), u32, u32, C.c_char_p, P32, C.POINTER(C.c_double)]),
        "fs_power_table": (C.c_int, [u32, P64, P32, P32, u32, P32]),
        "fs_setup_plan": (C.c_int, [u32, u32, P64, u64, P64, P32, u32, P32, P64]),
        "fs_setup_plan_chunks": (C.c_int, [u32, u32, P32, P64]),
        "fs_find_wheel_offset": (C.c_int, [P64, PI32]),
        "fs_is_prime": (C.c_int, [u64]),
        "fs_verify_factor": (C.c_int, [u64, u32, i32]),
        "fs_postprocess": (C.c_int, [C.POINTER(Factor), u64, C.c_int, P64, P64, P64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def lib():
    """The loaded libfactsieve.so (raises LibraryMissing if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise LibraryMissing(
                    f"{LIB_PATH} is missing: run `python -m factsieve_gb300.build` (needs nvcc)")
            _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def _strerror(code: int) -> str:
    try:
        return lib().fs_strerror(code).decode()
    except LibraryMissing:
        return f"error {code}"


def _p64(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _p32(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


# ----------------------------------------------------------------- host ---

def power_table(n: int):
    """Reference-format power table for n! (cl_sieve.cpp:773-838)."""
    L = lib()
    ln = C.c_uint32(0)
    L.fs_power_table(n, None, None, None, 0, C.byref(ln))
    m = ln.value
    tp = np.zeros(m, np.uint64)
    te = np.zeros(m, np.uint32)
    tb = np.zeros(m, np.uint32)
    rc = L.fs_power_table(n, _p64(tp), _p32(te), _p32(tb), m, C.byref(ln))
    if rc:
        raise FSError(rc, "fs_power_table")
    return tp, te, tb


def setup_plan(n: int, chunks: int = 1):
    """The bit-layered plan the GPU setup uses: (words, layers[:, 4], deficit)."""
    L = lib()
    nw, nl, d = C.c_uint64(0), C.c_uint32(0), C.c_uint64(0)
    L.fs_setup_plan(n, chunks, None, 0, C.byref(nw), None, 0, C.byref(nl), C.byref(d))
    w = np.zeros(max(nw.value, 1), np.uint64)
    lay = np.zeros((max(nl.value, 1), 4), np.uint32)
    rc = L.fs_setup_plan(n, chunks, _p64(w), nw.value, C.byref(nw), _p32(lay), nl.value, C.byref(nl),
                         C.byref(d))
    if rc:
        raise FSError(rc, "fs_setup_plan")
    return w[:nw.value], lay[:nl.value], d.value


def setup_plan_chunks(n: int, chunks: int):
    """Layer boundaries and deficits of each chunk of the plan for n!."""
    b = np.zeros(chunks + 1, np.uint32)
    d = np.zeros(chunks, np.uint64)
    rc = lib().fs_setup_plan_chunks(n, chunks, _p32(b), _p64(d))
    if rc:
        raise FSError(rc, "fs_setup_plan_chunks")
    return b, d


def walk_step(plo: int, phi: int, kmax: int) -> int:
    """The residue step the sieve runs for p in [plo, phi), multipliers up to kmax
    (6 / 7 / 9 / 4 / 5 / 8 half-offset 32-bit / shifted-window 64-bit / 64-bit
    with the quotient on the FP32 pipe / lazy 64-bit / lazy 96-bit / canonical
    96-bit; 10 / 11 / 12 half-offset with the FP32 quotient over a window sized
    from kmax, s >= 32 / s <= 32 / 96-bit product; 13 the same quotient in the
    half-offset canonical 96-bit step for p >= 2^63; 1 lazy 64-bit, 2 lazy
    96-bit, 3 canonical 96-bit, 0 chosen per candidate)."""
    return int(lib().fs_walk_step(plo, phi, kmax))


def setup_form(plo: int, phi: int) -> int:
    """1 when the setup of p in [plo, phi) folds its products modulo 2^63 + d
    (every p = 2^63 + d with 0 < d < 2^30; four-candidate kernels, 96-bit walks),
    else 0 (Montgomery products)."""
    return int(lib().fs_setup_form(plo, phi))


def find_wheel_offset(start: int):
    s = C.c_uint64(start)
    i = C.c_int32(-1)
    lib().fs_find_wheel_offset(C.byref(s), C.byref(i))
    return s.value, i.value


def is_prime(p: int) -> bool:
    return bool(lib().fs_is_prime(p))


def verify_factor(p: int, n: int, c: int) -> bool:
    return bool(lib().fs_verify_factor(p, n, c))


def candidate_capacity(low: int, high: int) -> int:
    return lib().fs_candidate_capacity(low, high)


def walk_state_words(cap: int) -> int:
    """u64 words of a stage-level residue buffer for cap candidates
    (FS_WALK_STATE_WORDS): cap residues, then cap uint32 walked-n tags."""
    return cap + (cap + 1) // 2


def postprocess(hits: np.ndarray, threads: int = 2):
    """getResults' CPU half: returns (kept factors sorted by (p,|n|), n+c sum, ndiscarded)."""
    L = lib()
    n = len(hits)
    buf = (Factor * max(n, 1))()
    arr = np.frombuffer(buf, dtype=FACTOR_DTYPE, count=n)
    arr[:] = hits
    kept, cs, disc = C.c_uint64(0), C.c_uint64(0), C.c_uint64(0)
    rc = L.fs_postprocess(buf, n, threads, C.byref(kept), C.byref(cs), C.byref(disc))
    if rc:
        raise FSError(rc, "fs_postprocess")
    return arr[:kept.value].copy(), cs.value, disc.value


# --------------------------------------------------------------- device ---

@dataclass
class SieveResult:
    """What the reference reports for a search (cl_sieve.cpp:1258-1263)."""
    factors: np.ndarray            # kept factors, FACTOR_DTYPE, sorted by (p, |n|)
    checksum: int
    primecount: int
    factorcount: int
    raw_sum: int = 0               # sum of (s6 + s7) alone
    nhits: int = 0                 # hits before the 2-PRP filter
    ndiscarded: int = 0
    stats: dict = field(default_factory=dict)

    def lines(self):
        """factors.txt lines: "p | n!+c" (cl_sieve.cpp:539)."""
        return [f"{int(p)} | {abs(int(nc))}!{'+1' if nc > 0 else '-1'}"
                for p, nc in zip(self.factors["p"], self.factors["nc"])]


class Context:
    """One CUDA device context of the library (fs_ctx)."""

    def __init__(self, device: int = 0):
        L = lib()
        h = C.c_void_p()
        rc = L.fs_create(device, C.byref(h))
        if rc:
            raise FSError(rc, f"fs_create(device={device})")
        self._h = h
        self.device = device
        sm, clk, mem = C.c_int(0), C.c_int(0), C.c_uint64(0)
        L.fs_device_info(h, C.byref(sm), C.byref(clk), C.byref(mem))
        self.sm_count, self.clock_khz, self.total_mem = sm.value, clk.value, mem.value

    # lifecycle
    def close(self):
        if getattr(self, "_h", None):
            lib().fs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _chk(self, rc, what):
        if rc:
            detail = lib().fs_last_error(self._h).decode()
            raise FSError(rc, f"{what} {detail}".strip())

    def set_stream(self, stream) -> None:
        """Use a cudaStream_t (int handle, e.g. torch.cuda.Stream().cuda_stream); None: own stream."""
        self._chk(lib().fs_set_stream(self._h, C.c_void_p(stream or 0)), "fs_set_stream")

    def set_tuning(self, sieve_blocks_per_sm=0, gen_blocks_per_sm=0, max_steps_per_launch=0,
                   setup_chunks=0, sieve_variant=0, sieve_block_threads=0, batch_tile_candidates=0) -> None:
        t = Tuning(sieve_blocks_per_sm, gen_blocks_per_sm, max_steps_per_launch, setup_chunks, sieve_variant,
                   sieve_block_threads, batch_tile_candidates)
        self._chk(lib().fs_set_tuning(self._h, C.byref(t)), "fs_set_tuning")

    def tuning(self) -> dict:
        t = Tuning()
        lib().fs_get_tuning(self._h, C.byref(t))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def synchronize(self):
        self._chk(lib().fs_synchronize(self._h), "fs_synchronize")

    # whole search
    def begin(self, pmin, pmax, nmin, nmax, result_cap=0):
        self._chk(lib().fs_search_begin(self._h, pmin, pmax, nmin, nmax, result_cap), "fs_search_begin")

    def segment(self, low, high):
        self._chk(lib().fs_search_segment(self._h, low, high), "fs_search_segment")

    def run_range(self, low, high, seg_width=0):
        self._chk(lib().fs_search_range(self._h, low, high, seg_width), "fs_search_range")

    def collect(self, cap, raise_on_flags=True):
        """Wait, then return (hits, raw_sum, primecount, flags, status) accumulated since
        the last collect; at most `cap` hits are copied (the host buffer is sized to
        what is pending, not to cap)."""
        L = lib()
        nf, rs, pc, fl = C.c_uint64(0), C.c_uint64(0), C.c_uint64(0), C.c_uint32(0)
        pend = np.zeros(1, np.uint64)
        self._chk(L.fs_search_pending(self._h, _p64(pend)), "fs_search_pending")
        cap = min(cap, int(pend[0]))
        buf = (Factor * max(cap, 1))()
        rc = L.fs_search_collect(self._h, buf, cap, C.byref(nf), C.byref(rs), C.byref(pc), C.byref(fl))
        hits = np.frombuffer(buf, dtype=FACTOR_DTYPE, count=min(nf.value, cap)).copy()
        if rc and raise_on_flags:
            self._chk(rc, "fs_search_collect")
        return hits, rs.value, pc.value, fl.value, rc

    def set_timing(self, enable: bool) -> None:
        self._chk(lib().fs_set_timing(self._h, 1 if enable else 0), "fs_set_timing")

    def stats(self) -> dict:
        s = Stats()
        self._chk(lib().fs_get_stats(self._h, C.byref(s)), "fs_get_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def reset_stats(self) -> None:
        self._chk(lib().fs_reset_stats(self._h), "fs_reset_stats")

    def bench_int_pipe(self, kind: int, iters: int = 20000):
        ops, ms = C.c_double(0), C.c_double(0)
        self._chk(lib().fs_bench_int_pipe(self._h, kind, iters, C.byref(ops), C.byref(ms)), "fs_bench_int_pipe")
        return ops.value, ms.value

    # stage-level (device pointers as ints, e.g. torch tensor.data_ptr())
    def getsegprimes(self, low, high, d_cand, cap, d_ctr):
        self._chk(lib().fs_getsegprimes(self._h, low, high, C.c_void_p(d_cand), cap, C.c_void_p(d_ctr)),
                  "fs_getsegprimes")

    def setup(self, d_cand, cap, d_ctr, nstart, d_residue):
        self._chk(lib().fs_setup(self._h, C.c_void_p(d_cand), cap, C.c_void_p(d_ctr), nstart,
                                 C.c_void_p(d_residue)), "fs_setup")

    def iterate(self, d_cand, cap, d_ctr, d_residue, nstart, nend, d_hits, hitcap):
        self._chk(lib().fs_iterate(self._h, C.c_void_p(d_cand), cap, C.c_void_p(d_ctr), C.c_void_p(d_residue),
                                   nstart, nend, C.c_void_p(d_hits), hitcap), "fs_iterate")

    def check(self, d_cand, cap, d_ctr, d_residue, nmax):
        self._chk(lib().fs_check(self._h, C.c_void_p(d_cand), cap, C.c_void_p(d_ctr), C.c_void_p(d_residue),
                                 nmax), "fs_check")

    def table_check(self, d_cand, d_ctr, nmin):
        out = np.zeros(2, np.uint64)
        self._chk(lib().fs_table_check(self._h, C.c_void_p(d_cand), C.c_void_p(d_ctr), nmin, _p64(out)),
                  "fs_table_check")
        return int(out[0]), int(out[1])

    # batches of uneven jobs
    def batch_prepare(self, jobs, hitcap=1 << 20):
        """jobs: sequence of (pmin, pmax, nmin, nmax)."""
        arr = (Job * len(jobs))(*[Job(*map(int, j)) for j in jobs])
        self._njobs = len(jobs)
        self._batch_hitcap = hitcap
        self._chk(lib().fs_batch_prepare(self._h, arr, len(jobs), hitcap), "fs_batch_prepare")

    def batch_launch(self):
        self._chk(lib().fs_batch_launch(self._h), "fs_batch_launch")

    def batch_collect(self, raise_on_flags=True):
        """Per-job results (list of dicts) and all hits (pad = job index)."""
        res = (JobResult * self._njobs)()
        cap = self._batch_hitcap
        buf = (Factor * cap)()
        nh = C.c_uint64(0)
        rc = lib().fs_batch_collect(self._h, res, buf, cap, C.byref(nh))
        if rc and raise_on_flags:
            self._chk(rc, "fs_batch_collect")
        hits = np.frombuffer(buf, dtype=FACTOR_DTYPE, count=min(nh.value, cap)).copy()
        out = [{k: getattr(r, k) for k, _ in JobResult._fields_} for r in res]
        return out, hits, rc

    def batch_release(self):
        self._chk(lib().fs_batch_release(self._h), "fs_batch_release")

    def batch_sieve(self, jobs, threads=2, hitcap=1 << 20):
        """Run many jobs in one persistent launch; one SieveResult per job."""
        self.batch_prepare(jobs, hitcap)
        self.batch_launch()
        res, hits, rc = self.batch_collect()
        out = []
        for k, r in enumerate(res):
            mine = hits[hits["pad"] == k].copy()
            mine["pad"] = 0
            kept, cs_add, disc = postprocess(mine, threads)
            out.append(SieveResult(kept, (r["raw_sum"] + cs_add) & 0xFFFFFFFFFFFFFFFF, r["primecount"], len(kept),
                                   r["raw_sum"], len(mine), disc))
        return out

    # measured launch sizing (fs_autotune / fs_autotune_batch)
    def autotune(self, pmin, pmax, nmin, nmax, target_ms=1000.0, cache_path=None) -> dict:
        """Time launch shapes on a sample of this search, apply the fastest to the
        context, and return it with the segment width for target_ms of kernel time."""
        r = TuneResult()
        path = cache_path.encode() if cache_path else None
        self._chk(lib().fs_autotune(self._h, pmin, pmax, nmin, nmax, target_ms, path, C.byref(r)), "fs_autotune")
        out = {k: getattr(r, k) for k, _ in TuneResult._fields_ if k != "tuning"}
        out["tuning"] = {k: getattr(r.tuning, k) for k, _ in Tuning._fields_}
        return out

    def autotune_batch(self, jobs, scale_down=16, cache_path=None) -> dict:
        """Time the batch kernel's tile sizes on the job mix (p-ranges narrowed
        scale_down times) and apply the fastest; returns {tile, ms}."""
        arr = (Job * len(jobs))(*[Job(*map(int, j)) for j in jobs])
        tile, ms = C.c_uint32(0), C.c_double(0)
        path = cache_path.encode() if cache_path else None
        self._chk(lib().fs_autotune_batch(self._h, arr, len(jobs), scale_down, path, C.byref(tile), C.byref(ms)),
                  "fs_autotune_batch")
        return {"tile": tile.value, "ms": ms.value}

    def plan_check(self, d_cand, d_ctr, nmin, d_words, d_layers4, nlayers, deficit):
        out = np.zeros(2, np.uint64)
        self._chk(lib().fs_plan_check(self._h, C.c_void_p(d_cand), C.c_void_p(d_ctr), nmin, C.c_void_p(d_words),
                                      C.c_void_p(d_layers4), nlayers, deficit, _p64(out)), "fs_plan_check")
        return int(out[0]), int(out[1])

    # the reference's whole search
    def sieve(self, pmin, pmax, nmin, nmax, threads=2, seg_width=0, result_cap=0) -> SieveResult:
        """Search p in [pmin, pmax), n in [nmin, nmax) like cl_sieve(); returns the
        reference-visible result (factors, checksum, primecount, factorcount)."""
        self.begin(pmin, pmax, nmin, nmax, result_cap)
        self.run_range(pmin, pmax, seg_width)
        cap = result_cap or (30_000_000 if pmin < 0xFFFFFFFF else 1_000_000)
        hits, raw, pc, flags, rc = self.collect(cap)
        kept, cs_add, disc = postprocess(hits, threads)
        checksum = (raw + cs_add) & 0xFFFFFFFFFFFFFFFF
        return SieveResult(kept, checksum, pc, len(kept), raw, len(hits), disc)


def sieve(pmin, pmax, nmin, nmax, device=0, threads=2, seg_width=0) -> SieveResult:
    with Context(device) as ctx:
        return ctx.sieve(pmin, pmax, nmin, nmax, threads=threads, seg_width=seg_width)
