"""fs_segment_noalloc, the allocation-free segment search, against fs_search_segment.

Callers that cannot allocate device memory -- code running inside a stream
capture, services whose device memory all belongs to a pool, embedders that
lend preallocated buffers -- call fs_segment_noalloc with their own device
buffers; its only scratch is a fixed array compiled into the library.  Here
it runs six segments in a row on one stream (p from 1e6 to just below 2^64),
with no synchronisation between the calls (so each call starts on the
previous call's leftovers in that array), and each result must equal the
allocating entry point's exactly:
same hit list, same sum of (s6 + s7), same candidate count (integer work, so
the tolerance is zero).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEGMENTS = [
    # (low, high, nmin, nmax): a small-p segment with many hits, then a large-p one
    (1_000_000, 1_400_000, 1000, 2600),
    (1_000_000_000_000, 1_000_004_000_000, 100_000, 101_000),
    # p crossing 2^32, and near 2^62, 2^63 (folded setup products) and 2^64 - 1
    ((1 << 32) - 2_000_000, (1 << 32) + 2_000_000, 5_000, 5_400),
    ((1 << 62) - 3_000_000, (1 << 62) + 1_000_000, 100_000, 100_300),
    ((1 << 63) + 1, (1 << 63) + 3_000_001, 1_000_000, 1_000_200),
    ((1 << 64) - 4_000_000, (1 << 64) - 1, 20_000, 20_200),
]


def _entry(fs):
    f = fs.lib().fs_segment_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                  C.c_uint64, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    return f


def _existing(fs, low, high, nmin, nmax):
    with fs.Context(0) as ctx:
        ctx.begin(low, high, nmin, nmax)
        ctx.segment(low, high)
        hits, raw, pc, flags, rc = ctx.collect(1 << 20)
    assert rc == 0 and flags == 0
    return sorted(zip(hits["p"].tolist(), hits["nc"].tolist())), raw, pc


def test_noalloc_equals_search_segment_two_calls_in_a_row():
    import torch
    import factsieve_gb300 as fs
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    want = [_existing(fs, *s) for s in SEGMENTS]
    assert want[0][0], "the first segment should produce hits"

    f = _entry(fs)
    hitcap = 1 << 16
    bufs = []
    for low, high, nmin, nmax in SEGMENTS:
        words, layers, deficit = fs.setup_plan(nmin)
        bufs.append({
            "words": torch.from_numpy(words.view(np.int64).copy()).cuda(),
            "layers": torch.from_numpy(layers.astype(np.uint32).reshape(-1).view(np.int32).copy()).cuda(),
            "nlayers": len(layers), "deficit": deficit,
            "hits": torch.zeros(2 * hitcap, dtype=torch.int64, device="cuda"),
            "ctr": torch.zeros(4, dtype=torch.int64, device="cuda"),
        })
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    for (low, high, nmin, nmax), b in zip(SEGMENTS, bufs):
        rc = f(low, high, nmin, nmax, b["words"].data_ptr(), b["layers"].data_ptr(), b["nlayers"], b["deficit"],
               b["hits"].data_ptr(), hitcap, b["ctr"].data_ptr(), stream.cuda_stream)
        assert rc == 0, fs.lib().fs_strerror(rc)
    torch.cuda.synchronize()

    for (wh, wraw, wpc), b in zip(want, bufs):
        ctr = np.frombuffer(b["ctr"].cpu().numpy().tobytes(), dtype=fs.COUNTERS_DTYPE)[0]
        assert int(ctr["flags"]) == 0
        assert int(ctr["primecount"]) == wpc
        assert int(ctr["raw_sum"]) == wraw
        n = int(ctr["nhits"])
        got = np.frombuffer(b["hits"].cpu().numpy().tobytes(), dtype=fs.FACTOR_DTYPE, count=n)
        assert sorted(zip(got["p"].tolist(), got["nc"].tolist())) == wh


def test_noalloc_rejects_a_segment_beyond_its_scratch():
    import torch
    import factsieve_gb300 as fs
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    f = _entry(fs)
    low, high = 10**12, 10**12 + 10**9          # ~3.6e7 candidates > FS_NOALLOC_MAX_CANDIDATES
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    rc = f(low, high, 1000, 2000, None, None, 0, 0, None, 0, ctr.data_ptr(), None)
    assert rc == 10   # FS_E_LIMIT
    assert fs.lib().fs_strerror(rc).decode() == "request exceeds a fixed size limit"


@pytest.mark.parametrize("low,high,nmin,nmax", [
    (1_000_000, 1_100_000, 0, 1000),       # nmin = 0
    (1_000_000, 1_100_000, 2000, 1000),    # nmin > nmax
    (1_000_000, 1_100_000, 2_000_000, 2_000_100),   # p below nmin
])
def test_noalloc_rejects_what_a_search_rejects(low, high, nmin, nmax):
    """The range checks of fs_search_begin (the reference's setupSearch,
    cl_sieve.cpp:561-589) apply: FS_E_ARG, and nothing runs."""
    import torch
    import factsieve_gb300 as fs
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    f = _entry(fs)
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    rc = f(low, high, nmin, nmax, None, None, 0, 0, None, 0, ctr.data_ptr(), None)
    assert rc == 1   # FS_E_ARG
    torch.cuda.synchronize()
    assert int(ctr.abs().sum()) == 0
