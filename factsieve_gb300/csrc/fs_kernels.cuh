// fs_kernels.cuh -- device data structures shared by the kernels and the C-ABI.
#pragma once
#include <stdint.h>
#include "fs_arith.cuh"

namespace fs {

// Reference factor record (cl_sieve.h:3-6): u64 p; i32 nc; 4 bytes padding.
// nc = -n for p | n! - 1, +n for p | n! + 1 (iterate.cl:69-73).
struct Factor {
    u64 p;
    int nc;
    int pad;
};

// Device-side counters of one search (the reference keeps these in
// g_primecount[6] and g_sum[], cl_sieve.cpp:439-467).
struct Counters {
    u64 raw_sum;      // sum of (s6 + s7) over finished candidates, wrapping
    u64 primecount;   // candidates produced by the generator (all segments)
    u32 ncand;        // candidates of the current segment (may exceed capacity)
    u32 nhits;        // factor hits (may exceed capacity)
    u32 flags;        // FLAG_* below
    u32 maxcand;      // largest per-segment candidate count seen
};

enum : u32 {
    FLAG_VALIDATION = 1u,   // nmax round trip failed (check.cl:67-78)
    FLAG_CAND_OVERFLOW = 2u,
    FLAG_HIT_OVERFLOW = 4u,
    FLAG_TABLE = 8u,        // power table disagrees with the direct product
};

// Setup plan layer (words [begin, end), dbl = double after squaring).
struct Layer {
    u32 begin, end, dbl, pad;
};

// Per-launch description of the setup plan.
struct PlanDev {
    const u64* words;
    const Layer* layers;
    u32 layer_begin, layer_end;   // layers of one chunk (or all for 1 chunk)
    u64 deficit;
};

}  // namespace fs
