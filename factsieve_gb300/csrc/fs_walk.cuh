// fs_walk.cuh -- the sieve's per-candidate device code, shared by the
// translation units that instantiate its kernels (fs_sieve2.cu, fs_sieve4.cu,
// fs_multi.cu, fs_kernels.cu): hit staging, setup-plan products, the walk
// regimes behind one interface, and the fused sieve kernel template.
//
//   sieve_kernel<S,F,B,W,P>  per candidate p: starting residue nstart!*R mod p
//                       from the bit-layered power table (setup.cl:49-103),
//                       the residue walk r <- r*(n+1) with the +-1 hit test
//                       for n in [nstart, nend) (iterate.cl:54-80), and on the
//                       last n-chunk the checksum s6 + s7 and the nmax round
//                       trip (check.cl:50-109).  S selects where the starting
//                       residue comes from, F whether this chunk finishes, B
//                       the resident blocks per SM it is built for, W the walk
//                       step, P the candidates per thread (2 or 4).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_arith.cuh"
#include "fs_kernels.cuh"
#include "fs_launch.h"

namespace fs {

constexpr int kSieveThreads = 256;
constexpr int kHitStage = 128;

struct HitStage {
    Factor buf[kHitStage];
    u32 n;
};

// Record a hit: lanes that hit together take consecutive slots of the block's
// shared-memory stage with one shared atomic (warp-ballot compaction); a full
// stage spills straight to the global list.
static __device__ __noinline__ void record_hit(HitStage& st, u64 p, int nc, Factor* hits, u32 hitcap,
                                        Counters* ctr, int tag) {
    const u32 mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const u32 rank = __popc(mask & ((1u << lane) - 1u));
    u32 base = 0;
    if (lane == leader) base = atomicAdd(&st.n, (u32)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    const u32 slot = base + rank;
    if (slot < kHitStage) {
        st.buf[slot].p = p;
        st.buf[slot].nc = nc;
        st.buf[slot].pad = tag;
    } else {
        u32 g = atomicAdd(&ctr->nhits, 1u);
        if (g < hitcap) {
            hits[g].p = p;
            hits[g].nc = nc;
            hits[g].pad = tag;
        } else {
            atomicOr(&ctr->flags, FLAG_HIT_OVERFLOW);
        }
    }
}

// Product of one plan chunk's layers for candidate c, with its R^-deficit.
__device__ __forceinline__ u64 plan_product(const Prime& c, const u64* __restrict__ words,
                                            const Layer* __restrict__ layers, u32 lb, u32 le) {
    const u64 p = c.p, pinv = c.pinv;
    u64 x = c.one;
    for (u32 l = lb; l < le; ++l) {
        const Layer L = layers[l];
        if (l != lb) x = mont_mul(x, x, p, pinv);
        if (L.dbl) x = mod_add(x, x, p);
        u32 i = L.begin;
        if ((i & 1) && i < L.end) x = mont_mul(x, __ldg(words + i++), p, pinv);
        for (; i + 2 <= L.end; i += 2) {
            const ulonglong2 w2 = __ldg(reinterpret_cast<const ulonglong2*>(words + i));
            x = mont_mul(x, w2.x, p, pinv);
            x = mont_mul(x, w2.y, p, pinv);
        }
        if (i < L.end) x = mont_mul(x, __ldg(words + i), p, pinv);
    }
    return x;
}

// The same for two candidates at once: two independent product chains share
// every (warp-uniform) table load.
__device__ __forceinline__ void plan_product2(const Prime& a, const Prime& b, const u64* __restrict__ words,
                                              const Layer* __restrict__ layers, u32 lb, u32 le, u64& xa,
                                              u64& xb) {
    u64 x = a.one, y = b.one;
    for (u32 l = lb; l < le; ++l) {
        const Layer L = layers[l];
        if (l != lb) {
            x = mont_mul(x, x, a.p, a.pinv);
            y = mont_mul(y, y, b.p, b.pinv);
        }
        if (L.dbl) {
            x = mod_add(x, x, a.p);
            y = mod_add(y, y, b.p);
        }
        u32 i = L.begin;
        if ((i & 1) && i < L.end) {
            const u64 w = __ldg(words + i++);
            x = mont_mul(x, w, a.p, a.pinv);
            y = mont_mul(y, w, b.p, b.pinv);
        }
        for (; i + 2 <= L.end; i += 2) {
            const ulonglong2 w2 = __ldg(reinterpret_cast<const ulonglong2*>(words + i));
            x = mont_mul(x, w2.x, a.p, a.pinv);
            y = mont_mul(y, w2.x, b.p, b.pinv);
            x = mont_mul(x, w2.y, a.p, a.pinv);
            y = mont_mul(y, w2.y, b.p, b.pinv);
        }
        if (i < L.end) {
            const u64 w = __ldg(words + i);
            x = mont_mul(x, w, a.p, a.pinv);
            y = mont_mul(y, w, b.p, b.pinv);
        }
    }
    xa = x;
    xb = y;
}

// The same for four candidates, each product split over two chains (even
// and odd words of a layer, the odd chain started at R = one so that joining
// them with one more Montgomery product leaves the deficit unchanged): eight
// independent chains per thread and one table load per four candidates.
__device__ __forceinline__ void plan_product4(const Prime (&c)[4], const u64* __restrict__ words,
                                              const Layer* __restrict__ layers, u32 lb, u32 le, u64 (&x)[4]) {
#pragma unroll
    for (int h = 0; h < 4; ++h) x[h] = c[h].one;
    for (u32 l = lb; l < le; ++l) {
        const Layer L = layers[l];
        if (l != lb) {
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], x[h], c[h].p, c[h].pinv);
        }
        if (L.dbl) {
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mod_add(x[h], x[h], c[h].p);
        }
        u32 i = L.begin;
        if ((i & 1) && i < L.end) {
            const u64 w = __ldg(words + i++);
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], w, c[h].p, c[h].pinv);
        }
        if (i + 2 <= L.end) {
            u64 y[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) y[h] = c[h].one;
            for (; i + 2 <= L.end; i += 2) {
                const ulonglong2 w2 = __ldg(reinterpret_cast<const ulonglong2*>(words + i));
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    x[h] = mont_mul(x[h], w2.x, c[h].p, c[h].pinv);
                    y[h] = mont_mul(y[h], w2.y, c[h].p, c[h].pinv);
                }
            }
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], y[h], c[h].p, c[h].pinv);
        }
        if (i < L.end) {
            const u64 w = __ldg(words + i);
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], w, c[h].p, c[h].pinv);
        }
    }
}

// plan_product4 for p = 2^63 + d (0 < d < 2^30) with the folding product
// pm_mul in place of Montgomery's: plain residues from 1, no R^-1 deficit;
// x[h] ends as n! mod p, lazy (any 64-bit value congruent to it).
__device__ __forceinline__ void plan_product4_pm(const Prime (&c)[4], const u64* __restrict__ words,
                                                 const Layer* __restrict__ layers, u32 lb, u32 le, u64 (&x)[4]) {
    PMod m[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        m[h] = make_pmod(c[h].p);
        x[h] = 1;
    }
    for (u32 l = lb; l < le; ++l) {
        const Layer L = layers[l];
        if (l != lb) {
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = pm_mul(x[h], x[h], m[h]);
        }
        if (L.dbl) {
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = pm_mul(x[h], 2, m[h]);
        }
        u32 i = L.begin;
        if ((i & 1) && i < L.end) {
            const u64 w = __ldg(words + i++);
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = pm_mul(x[h], w, m[h]);
        }
        if (i + 2 <= L.end) {
            u64 y[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) y[h] = 1;
            for (; i + 2 <= L.end; i += 2) {
                const ulonglong2 w2 = __ldg(reinterpret_cast<const ulonglong2*>(words + i));
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    x[h] = pm_mul(x[h], w2.x, m[h]);
                    y[h] = pm_mul(y[h], w2.y, m[h]);
                }
            }
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = pm_mul(x[h], y[h], m[h]);
        }
        if (i < L.end) {
            const u64 w = __ldg(words + i);
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = pm_mul(x[h], w, m[h]);
        }
    }
}

struct WalkOut {
    HitStage* st;
    Factor* hits;
    u32 hitcap;
    Counters* ctr;
    int tag;   // stored in each hit record's pad word (job index in a batch, else 0)
};

// The Barrett walk regimes behind one interface.  enter / leave convert a
// canonical n! R into the regime's residue form and back; hit classifies a
// canonical residue of that form: -1 for n! = 1 (p | n! - 1), +1 for n! = -1
// (p | n! + 1), 0 for neither.
struct RegT64 {
    using K = Lazy64;
    static __device__ __forceinline__ K make(const Prime& c, u32, u64) { return make_lazy(c); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return lazy_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return lazy_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return lazy_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime&, const K&) { return r; }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime&, const K& X) { return lazy_canon(r, X); }
    static __device__ __forceinline__ int hit(u64 c, const K& X) {
        return c == X.one ? -1 : (c == X.p - X.one ? 1 : 0);
    }
};
struct RegL96 {
    using K = Lazy96;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_lazy96(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return lazy96_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return lazy96_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return lazy96_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime&, const K&) { return r; }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime&, const K& X) { return lazy96_canon(r, X); }
    static __device__ __forceinline__ int hit(u64 c, const K& X) {
        return c == X.one ? -1 : (c == X.p - X.one ? 1 : 0);
    }
};
struct RegC96 {
    using K = Canon96;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_canon96(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return canon96_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return canon96_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K&) { return r; }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime&, const K&) { return r; }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime&, const K&) { return r; }
    static __device__ __forceinline__ int hit(u64 c, const K& X) {
        return c == X.one ? -1 : (c == X.p - X.one ? 1 : 0);
    }
};
struct RegH64 {
    using K = Half64;
    static __device__ __forceinline__ K make(const Prime& c, u32, u64) { return make_half(c); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return half_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return half_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return half_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(half_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegHF {
    using K = HalfF;
    static __device__ __forceinline__ K make(const Prime& c, u32, u64 f) { return make_halff(c, f); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return halff_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return halff_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return halff_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(halff_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
// The float quotient with the window chosen from k_max (make_halfg): HG on
// the halff_walk8x2 block, HGL and HG96 on their own blocks.
struct RegHG {
    using K = HalfF;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_halfg(c, kmax, 0); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return halff_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return halff_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return halff_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(halff_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegHGL {
    using K = HalfF;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_halfg(c, kmax, 1); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return halfgl_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return halfgl_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return halff_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(halff_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegHG96 {
    using K = HalfF;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_halfg(c, kmax, 2); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return halfg96_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return halfg96_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return halff_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(halff_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegH32 {
    using K = Half32;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_half32(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return half32_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return half32_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return half32_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(half32_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegHM {
    using K = Half96;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_halfmid(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return halfmid_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return halfmid_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return half96_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(half96_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegC96H {
    using K = Canon96H;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_canon96h(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return canon96h_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return canon96h_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K&) { return r; }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K&) { return half_leave(r, c); }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegC96G {
    using K = Canon96G;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_canon96g(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return canon96g_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return canon96g_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K&) { return r; }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K&) { return half_leave(r, c); }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};
struct RegH96 {
    using K = Half96;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax, u64) { return make_half96(c, kmax); }
    static __device__ __forceinline__ u32 block(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const K& A, const K& B) {
        return half96_walk8x2(al, ah, bl, bh, k1, A, B);
    }
    static __device__ __forceinline__ u64 step(u64 r, u32 k, const K& X) { return half96_step(r, k, X); }
    static __device__ __forceinline__ u64 canon(u64 r, const K& X) { return half96_canon(r, X); }
    static __device__ __forceinline__ u64 enter(u64 r, const Prime& c, const K& X) { return half_enter(r, c, X.x); }
    static __device__ __forceinline__ u64 leave(u64 r, const Prime& c, const K& X) {
        return half_leave(half96_canon(r, X), c);
    }
    static __device__ __forceinline__ int hit(u64 c, const K& X) { return c == X.x ? -1 : (c == X.x + 1 ? 1 : 0); }
};

// Exact +-1 test of a walk residue at n, recording a hit.
template <class Reg>
__device__ __forceinline__ void reg_check(u64 r, u32 n, const typename Reg::K& X, const WalkOut& o) {
    const int h = Reg::hit(Reg::canon(r, X), X);
    if (h) record_hit(*o.st, X.p, h * (int)n, o.hits, o.hitcap, o.ctr, o.tag);
}

// Replay N steps from r at n0 with exact tests (the PTX blocks saw a
// possible hit in them); the residues are the same bits as the blocks'.
template <class Reg, int N>
__device__ __noinline__ void reg_replay(u64 r, u32 n0, typename Reg::K X, WalkOut o) {
    for (u32 j = 0; j < N; ++j) {
        reg_check<Reg>(r, n0 + j, X, o);
        r = Reg::step(r, n0 + j + 1, X);
    }
}
template <class Reg>
__device__ __forceinline__ void reg_replay8(u64 r, u32 n0, const typename Reg::K& X, const WalkOut& o) {
    reg_replay<Reg, 8>(r, n0, X, o);
}

// Walk two candidates of one regime over [nstart, nend); residues in and out
// are in the regime's form (out not yet canonical).  real_b = false: b
// duplicates a and its hits are dropped.
template <class Reg>
__device__ __forceinline__ void walk_reg2(u64& ra, u64& rb, const typename Reg::K& A, const typename Reg::K& B,
                                          bool real_b, u32 nstart, u32 nend, const WalkOut& o) {
    u32 al = (u32)ra, ah = (u32)(ra >> 32), bl = (u32)rb, bh = (u32)(rb >> 32);
    u32 n = nstart;
    for (; n + 8 <= nend; n += 8) {
        const u32 sal = al, sah = ah, sbl = bl, sbh = bh;
        if (Reg::block(al, ah, bl, bh, n + 1, A, B)) {
            reg_replay8<Reg>(((u64)sah << 32) | sal, n, A, o);
            if (real_b) reg_replay8<Reg>(((u64)sbh << 32) | sbl, n, B, o);
        }
    }
    u64 a = ((u64)ah << 32) | al, b = ((u64)bh << 32) | bl;
    for (; n < nend; ++n) {
        reg_check<Reg>(a, n, A, o);
        a = Reg::step(a, n + 1, A);
        if (real_b) {
            reg_check<Reg>(b, n, B, o);
            b = Reg::step(b, n + 1, B);
        }
    }
    ra = a;
    if (real_b) rb = b;
}

template <class Reg>
__device__ __forceinline__ void walk_reg_pair(u64& ra, u64& rb, const Prime& a, const Prime& b, bool real_b,
                                              u32 nstart, u32 nend, const WalkOut& o) {
    const typename Reg::K A = Reg::make(a, nend, a.p);
    const typename Reg::K B = real_b ? Reg::make(b, nend, b.p) : A;
    u64 wa = Reg::enter(ra, a, A);
    u64 wb = real_b ? Reg::enter(rb, b, B) : wa;
    walk_reg2<Reg>(wa, wb, A, B, real_b, nstart, nend, o);
    ra = Reg::leave(wa, a, A);
    if (real_b) rb = Reg::leave(wb, b, B);
}

// Generic walk for any p < 2^64 and n < 2^31: multiply by the Montgomery
// image of n+1, advanced by R each step (the reference's own step).
__device__ __forceinline__ u64 walk_generic(u64 r, const Prime& c, u32 nstart, u32 nend, const WalkOut& o) {
    const u64 p = c.p, one = c.one, nmo = p - one;
    if (nstart >= nend) return r;
    u64 k = to_mont((u64)nstart + 1, c);
    for (u32 n = nstart; n < nend; ++n) {
        if (r == one || r == nmo) record_hit(*o.st, p, r == one ? -(int)n : (int)n, o.hits, o.hitcap, o.ctr, o.tag);
        r = mont_mul(r, k, p, c.pinv);
        k = mod_add(k, one, p);
    }
    return r;
}

// Walk regime of one candidate for multipliers up to kmax: 6 / 7 / 4 / 5 / 8
// 32-bit / shifted-window 64-bit / lazy 64-bit / lazy 96-bit / canonical
// 96-bit in half-offset form, 1 lazy 64-bit, 2 lazy 96-bit, 3 canonical
// 96-bit, 0 generic Montgomery.  (The float-quotient step runs only where
// the host has shown it valid for a whole launch: per candidate it would
// add little and cost the mixed-step kernel registers.)
__device__ __forceinline__ int walk_regime(u64 p, u32 kmax) {
    if (half32_ok(p, kmax)) return 6;
    if (halfmid_ok(p, kmax)) return 7;
    if (canon96h_ok(p, kmax)) return 8;
    if (half_ok(p, kmax)) return 4;
    if (lazy_ok(p, kmax)) return 1;
    if (half96_ok(p, kmax)) return 5;
    if (lazy96_ok(p, kmax)) return 2;
    if (canon96_ok(p, kmax)) return 3;
    return 0;
}

__device__ __forceinline__ void walk_one(u64& r, const Prime& c, int reg, u32 nstart, u32 nend, const WalkOut& o) {
    u64 dup = r;
    switch (reg) {
        case 1: walk_reg_pair<RegT64>(r, dup, c, c, false, nstart, nend, o); break;
        case 2: walk_reg_pair<RegL96>(r, dup, c, c, false, nstart, nend, o); break;
        case 3: walk_reg_pair<RegC96>(r, dup, c, c, false, nstart, nend, o); break;
        case 4: walk_reg_pair<RegH64>(r, dup, c, c, false, nstart, nend, o); break;
        case 5: walk_reg_pair<RegH96>(r, dup, c, c, false, nstart, nend, o); break;
        case 6: walk_reg_pair<RegH32>(r, dup, c, c, false, nstart, nend, o); break;
        case 7: walk_reg_pair<RegHM>(r, dup, c, c, false, nstart, nend, o); break;
        case 8: walk_reg_pair<RegC96H>(r, dup, c, c, false, nstart, nend, o); break;
        default: r = walk_generic(r, c, nstart, nend, o); break;
    }
}

// Walk both candidates of a pair with one step the host has shown valid for
// every candidate of the launch (WALK_T64 / WALK_L96 / WALK_C96), or, for
// WALK_ANY, each with the fastest step that applies to it.
template <int WALK>
__device__ __forceinline__ void walk_pair_as(u64& ra, u64& rb, const Prime& a, const Prime& b, bool real_b,
                                             u32 nstart, u32 nend, const WalkOut& o);

// Walk both candidates of a pair, each with the fastest step that applies.
__device__ __forceinline__ void walk_pair(u64& ra, u64& rb, const Prime& a, const Prime& b, bool real_b,
                                          u32 nstart, u32 nend, const WalkOut& o) {
    if (nstart >= nend) return;
    const int ga = walk_regime(a.p, nend);
    const int gb = real_b ? walk_regime(b.p, nend) : ga;
    if (ga == gb && ga != 0) {
        switch (ga) {
            case 1: walk_reg_pair<RegT64>(ra, rb, a, b, real_b, nstart, nend, o); return;
            case 2: walk_reg_pair<RegL96>(ra, rb, a, b, real_b, nstart, nend, o); return;
            case 4: walk_reg_pair<RegH64>(ra, rb, a, b, real_b, nstart, nend, o); return;
            case 5: walk_reg_pair<RegH96>(ra, rb, a, b, real_b, nstart, nend, o); return;
            case 6: walk_reg_pair<RegH32>(ra, rb, a, b, real_b, nstart, nend, o); return;
            case 7: walk_reg_pair<RegHM>(ra, rb, a, b, real_b, nstart, nend, o); return;
            case 8: walk_reg_pair<RegC96H>(ra, rb, a, b, real_b, nstart, nend, o); return;
            default: walk_reg_pair<RegC96>(ra, rb, a, b, real_b, nstart, nend, o); return;
        }
    }
    walk_one(ra, a, ga, nstart, nend, o);
    if (real_b) walk_one(rb, b, gb, nstart, nend, o);
}

template <int WALK>
__device__ __forceinline__ void walk_pair_as(u64& ra, u64& rb, const Prime& a, const Prime& b, bool real_b,
                                             u32 nstart, u32 nend, const WalkOut& o) {
    if (nstart >= nend) return;
    if (WALK == WALK_HF) walk_reg_pair<RegHF>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_HG) walk_reg_pair<RegHG>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_HGL) walk_reg_pair<RegHGL>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_HG96) walk_reg_pair<RegHG96>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_H64) walk_reg_pair<RegH64>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_H96) walk_reg_pair<RegH96>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_H32) walk_reg_pair<RegH32>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_HM) walk_reg_pair<RegHM>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_C96H) walk_reg_pair<RegC96H>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_C96G) walk_reg_pair<RegC96G>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_T64) walk_reg_pair<RegT64>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_L96) walk_reg_pair<RegL96>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_C96) walk_reg_pair<RegC96>(ra, rb, a, b, real_b, nstart, nend, o);
    else walk_pair(ra, rb, a, b, real_b, nstart, nend, o);
}

// Walk four candidates of one regime over [nstart, nend) as two pairs whose
// PTX blocks have no dependence on each other, so four residue chains are in
// flight per thread.  Candidates h >= nreal duplicate candidate 0: they are
// walked (the warp stays converged) but never tested or returned.
//
// The candidates' Montgomery constants are not kept across the walk (they
// would cost the registers that a third resident block needs): c is rebuilt
// from p after it, for leave() and the caller's final check.
template <class Reg>
__device__ __forceinline__ void walk_reg4(u64 (&r)[4], Prime (&c)[4], u32 nreal, u32 nstart, u32 nend,
                                          const WalkOut& o) {
    // the thread's least candidate: one floor for all four keeps shared constants in shared registers
    const u64 f = umin64(umin64(c[0].p, c[1].p), umin64(c[2].p, c[3].p));
    const typename Reg::K K0 = Reg::make(c[0], nend, f), K1 = Reg::make(c[1], nend, f);
    const typename Reg::K K2 = Reg::make(c[2], nend, f), K3 = Reg::make(c[3], nend, f);
    const u64 w0 = Reg::enter(r[0], c[0], K0), w1 = Reg::enter(r[1], c[1], K1);
    const u64 w2 = Reg::enter(r[2], c[2], K2), w3 = Reg::enter(r[3], c[3], K3);
    u32 l0 = (u32)w0, h0 = (u32)(w0 >> 32), l1 = (u32)w1, h1 = (u32)(w1 >> 32);
    u32 l2 = (u32)w2, h2 = (u32)(w2 >> 32), l3 = (u32)w3, h3 = (u32)(w3 >> 32);
    u32 n = nstart;
    for (; n + 8 <= nend; n += 8) {
        const u64 s0 = ((u64)h0 << 32) | l0, s1 = ((u64)h1 << 32) | l1;
        const u64 s2 = ((u64)h2 << 32) | l2, s3 = ((u64)h3 << 32) | l3;
        const u32 f1 = Reg::block(l0, h0, l1, h1, n + 1, K0, K1);
        const u32 f2 = Reg::block(l2, h2, l3, h3, n + 1, K2, K3);
        if (f1 | f2) {
            if (f1) {
                reg_replay8<Reg>(s0, n, K0, o);
                if (nreal > 1) reg_replay8<Reg>(s1, n, K1, o);
            }
            if (f2 && nreal > 2) {
                reg_replay8<Reg>(s2, n, K2, o);
                if (nreal > 3) reg_replay8<Reg>(s3, n, K3, o);
            }
        }
    }
    u64 x0 = ((u64)h0 << 32) | l0, x1 = ((u64)h1 << 32) | l1;
    u64 x2 = ((u64)h2 << 32) | l2, x3 = ((u64)h3 << 32) | l3;
    for (; n < nend; ++n) {
        reg_check<Reg>(x0, n, K0, o);
        x0 = Reg::step(x0, n + 1, K0);
        if (nreal > 1) {
            reg_check<Reg>(x1, n, K1, o);
            x1 = Reg::step(x1, n + 1, K1);
        }
        if (nreal > 2) {
            reg_check<Reg>(x2, n, K2, o);
            x2 = Reg::step(x2, n + 1, K2);
        }
        if (nreal > 3) {
            reg_check<Reg>(x3, n, K3, o);
            x3 = Reg::step(x3, n + 1, K3);
        }
    }
    c[0] = make_prime(K0.p);
    c[1] = make_prime(K1.p);
    c[2] = make_prime(K2.p);
    c[3] = make_prime(K3.p);
    r[0] = Reg::leave(x0, c[0], K0);
    if (nreal > 1) r[1] = Reg::leave(x1, c[1], K1);
    if (nreal > 2) r[2] = Reg::leave(x2, c[2], K2);
    if (nreal > 3) r[3] = Reg::leave(x3, c[3], K3);
}

// Four candidates with a step valid for all of them (WALK_T64 / WALK_L96 /
// WALK_C96), or, for WALK_ANY, as two pairs one after the other.
template <int WALK>
__device__ __forceinline__ void walk_quad_as(u64 (&r)[4], Prime (&c)[4], u32 nreal, u32 nstart, u32 nend,
                                             const WalkOut& o) {
    if (nstart >= nend) return;
    if (WALK == WALK_HF) walk_reg4<RegHF>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_HG) walk_reg4<RegHG>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_HGL) walk_reg4<RegHGL>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_HG96) walk_reg4<RegHG96>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_H64) walk_reg4<RegH64>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_H96) walk_reg4<RegH96>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_H32) walk_reg4<RegH32>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_HM) walk_reg4<RegHM>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_C96H) walk_reg4<RegC96H>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_C96G) walk_reg4<RegC96G>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_T64) walk_reg4<RegT64>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_L96) walk_reg4<RegL96>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_C96) walk_reg4<RegC96>(r, c, nreal, nstart, nend, o);
    else {
        walk_pair(r[0], r[1], c[0], c[1], nreal > 1, nstart, nend, o);
        if (nreal > 2) walk_pair(r[2], r[3], c[2], c[3], nreal > 3, nstart, nend, o);
    }
}

// The same with the step chosen at run time (one job's code, uniform over a
// block's tile).
__device__ __forceinline__ void walk_quad_rt(int walk, u64 (&r)[4], Prime (&c)[4], u32 nreal, u32 nstart, u32 nend,
                                             const WalkOut& o) {
    switch (walk) {
        case WALK_HF: walk_quad_as<WALK_HF>(r, c, nreal, nstart, nend, o); break;
        case WALK_HG: walk_quad_as<WALK_HG>(r, c, nreal, nstart, nend, o); break;
        case WALK_HGL: walk_quad_as<WALK_HGL>(r, c, nreal, nstart, nend, o); break;
        case WALK_HG96: walk_quad_as<WALK_HG96>(r, c, nreal, nstart, nend, o); break;
        case WALK_H64: walk_quad_as<WALK_H64>(r, c, nreal, nstart, nend, o); break;
        case WALK_H96: walk_quad_as<WALK_H96>(r, c, nreal, nstart, nend, o); break;
        case WALK_H32: walk_quad_as<WALK_H32>(r, c, nreal, nstart, nend, o); break;
        case WALK_HM: walk_quad_as<WALK_HM>(r, c, nreal, nstart, nend, o); break;
        case WALK_C96H: walk_quad_as<WALK_C96H>(r, c, nreal, nstart, nend, o); break;
        case WALK_C96G: walk_quad_as<WALK_C96G>(r, c, nreal, nstart, nend, o); break;
        case WALK_T64: walk_quad_as<WALK_T64>(r, c, nreal, nstart, nend, o); break;
        case WALK_L96: walk_quad_as<WALK_L96>(r, c, nreal, nstart, nend, o); break;
        case WALK_C96: walk_quad_as<WALK_C96>(r, c, nreal, nstart, nend, o); break;
        default: walk_quad_as<WALK_ANY>(r, c, nreal, nstart, nend, o); break;
    }
}

// The last three of four candidates of a thread, duplicates of the first
// where the list ends.
__device__ __forceinline__ u32 load_quad(const u64* cand, u32 i0, u32 n, Prime (&c)[4]) {
    const u32 nreal = n - i0 < 4 ? n - i0 : 4;
    c[0] = make_prime(cand[i0]);
#pragma unroll
    for (int h = 1; h < 4; ++h) c[h] = (u32)h < nreal ? make_prime(cand[i0 + h]) : c[0];
    return nreal;
}

// s6 + s7 of one finished candidate and its nmax round trip (check.cl:50-109).
// n is the n the candidate's residue stands at: its walked[] tag from the
// launches before, plus the steps of this one.  s7 = n R mod p is then
// the reference's s7 (its Montgomery image of n, advanced by R once per step
// across every iterate chunk, iterate.cl:67-68), and converting it back must
// give nmax, with the reference's allowance for p <= nmax.  A chunk of n that
// was skipped or walked twice fails the round trip and changes the checksum,
// as it does in the reference.
__device__ __forceinline__ void final_check(const Prime& c, u64 r, u32 n, u32 nmax, u64& sum, u32& bad) {
    const u64 s7 = to_mont(n, c);
    u32 back = (u32)mont_mul(s7, 1, c.p, c.pinv);
    if (c.p <= nmax && nmax % c.p == back) back = nmax;
    bad += back != nmax;
    sum += r + s7;
}

// Starting residue of candidate i (SETUP mode), before the walk.
template <int SETUP>
__device__ __forceinline__ u64 start_residue_one(const SieveArgs& a, const Prime& c, u32 i) {
    u64 r;
    if (SETUP == SETUP_PLAN) {
        r = plan_product(c, a.plan.words, a.plan.layers, a.plan.layer_begin, a.plan.layer_end);
        r = mont_mul(r, mont_pow(c.r2, a.plan.deficit, c), c.p, c.pinv);
    } else if (SETUP == SETUP_PARTIALS) {
        r = a.partials[i];
        for (u32 k = 1; k < a.nchunks; ++k) r = mont_mul(r, a.partials[(u64)k * a.cap + i], c.p, c.pinv);
        r = mont_mul(r, mont_pow(c.r2, a.plan.deficit, c), c.p, c.pinv);
    } else {
        r = a.residue[i];
    }
    return r;
}

// The n candidate i's residue stands at when the launch starts: its tag when
// it comes from an earlier launch (SETUP_LOAD with tags), else nstart.
template <int SETUP>
__device__ __forceinline__ u32 start_n(const SieveArgs& a, u32 i) {
    return (SETUP == SETUP_LOAD && a.walked) ? a.walked[i] : a.nstart;
}

template <int SETUP, bool FINAL, int MINB, int WALK, int PPT>
__global__ void __launch_bounds__(kSieveThreads, MINB) sieve_kernel(SieveArgs a) {
    __shared__ HitStage st;
    __shared__ u64 wsum[kSieveThreads / 32];
    __shared__ u32 wbad[kSieveThreads / 32];
    // With the float-quotient steps, each thread's checksum and validation
    // count stay in shared memory across the walk (volatile: not promoted to
    // registers), so that the walk loop of a checking kernel is allocated like
    // a storing one's: in registers they cost config 2's fused launch 1.2 %
    // and a 96-bit float-quotient launch 1.5 %.  The 96-bit steps for
    // p >= 2^63 keep them in registers (shared costs config 3 2.9 %).
    constexpr bool kAccShared = FINAL && PPT == 4 &&
                                (WALK == WALK_HF || WALK == WALK_HG || WALK == WALK_HGL || WALK == WALK_HG96);
    __shared__ u64 tsum_[kAccShared ? kSieveThreads : 1];
    __shared__ u32 tbad_[kAccShared ? kSieveThreads : 1];
    volatile u64* tsum = tsum_;
    volatile u32* tbad = tbad_;
    if (kAccShared) {
        tsum[threadIdx.x] = 0;
        tbad[threadIdx.x] = 0;
    }
    u64 sum = 0;
    u32 bad = 0;
    if (threadIdx.x == 0) st.n = 0;
    __syncthreads();
    const u32 ncand = *a.ncand;
    const u32 n = ncand < a.cap ? ncand : a.cap;
    const WalkOut o{&st, a.hits, a.hitcap, a.ctr, 0};
    // every residue of the launch advances by the launch's steps
    const u32 steps = a.nend > a.nstart ? a.nend - a.nstart : 0;
    const u32 stride = gridDim.x * blockDim.x;
    if constexpr (PPT == 4) {
        // four candidates per thread: two interleaved pairs
        const u32 nquads = (n + 3) / 4;
        for (u32 j = blockIdx.x * blockDim.x + threadIdx.x; j < nquads; j += stride) {
            const u32 i0 = 4 * j;
            const u32 nreal = n - i0 < 4 ? n - i0 : 4;
            Prime c[4];
            c[0] = make_prime(a.cand[i0]);
#pragma unroll
            for (int h = 1; h < 4; ++h) c[h] = (u32)h < nreal ? make_prime(a.cand[i0 + h]) : c[0];
            u64 r[4];
            if constexpr (SETUP == SETUP_PLAN) {
                plan_product4(c, a.plan.words, a.plan.layers, a.plan.layer_begin, a.plan.layer_end, r);
#pragma unroll
                for (int h = 0; h < 4; ++h)
                    r[h] = mont_mul(r[h], mont_pow(c[h].r2, a.plan.deficit, c[h]), c[h].p, c[h].pinv);
            } else if constexpr (SETUP == SETUP_PLAN_PM) {
                // p = 2^63 + d, d < 2^30 over the launch, one plan chunk: plain n! mod p, then n! R
                plan_product4_pm(c, a.plan.words, a.plan.layers, a.plan.layer_begin, a.plan.layer_end, r);
#pragma unroll
                for (int h = 0; h < 4; ++h) r[h] = to_mont(pm_canon(r[h], c[h].p), c[h]);
            } else {
                r[0] = start_residue_one<SETUP>(a, c[0], i0);
#pragma unroll
                for (int h = 1; h < 4; ++h) r[h] = (u32)h < nreal ? start_residue_one<SETUP>(a, c[h], i0 + h) : r[0];
            }
            walk_quad_as<WALK>(r, c, nreal, a.nstart, a.nend, o);
            u64 qsum = 0;
            u32 qbad = 0;
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                if ((u32)h >= nreal) break;
                const u32 nw = start_n<SETUP>(a, i0 + h) + steps;
                if (FINAL) {
                    final_check(c[h], r[h], nw, a.nmax, qsum, qbad);
                } else {
                    a.residue[i0 + h] = r[h];
                    if (a.walked) a.walked[i0 + h] = nw;
                }
            }
            if (kAccShared) {
                tsum[threadIdx.x] = tsum[threadIdx.x] + qsum;
                tbad[threadIdx.x] = tbad[threadIdx.x] + qbad;
            } else if (FINAL) {
                sum += qsum;
                bad += qbad;
            }
        }
    } else {
    const u32 npairs = (n + 1) / 2;
    for (u32 j = blockIdx.x * blockDim.x + threadIdx.x; j < npairs; j += stride) {
        const u32 ia = 2 * j, ib = 2 * j + 1;
        const bool real_b = ib < n;
        const Prime ca = make_prime(a.cand[ia]);
        const Prime cb = real_b ? make_prime(a.cand[ib]) : ca;
        u64 ra, rb;
        if (SETUP == SETUP_PLAN) {
            plan_product2(ca, cb, a.plan.words, a.plan.layers, a.plan.layer_begin, a.plan.layer_end, ra, rb);
            ra = mont_mul(ra, mont_pow(ca.r2, a.plan.deficit, ca), ca.p, ca.pinv);
            rb = mont_mul(rb, mont_pow(cb.r2, a.plan.deficit, cb), cb.p, cb.pinv);
        } else {
            ra = start_residue_one<SETUP>(a, ca, ia);
            rb = real_b ? start_residue_one<SETUP>(a, cb, ib) : ra;
        }
        walk_pair_as<WALK>(ra, rb, ca, cb, real_b, a.nstart, a.nend, o);
        const u32 nwa = start_n<SETUP>(a, ia) + steps;
        const u32 nwb = real_b ? start_n<SETUP>(a, ib) + steps : nwa;
        if (FINAL) {
            // s7 from the n each walk reached, the reference's final Montgomery image of n
            final_check(ca, ra, nwa, a.nmax, sum, bad);
            if (real_b) final_check(cb, rb, nwb, a.nmax, sum, bad);
        } else {
            a.residue[ia] = ra;
            if (real_b) a.residue[ib] = rb;
            if (a.walked) {
                a.walked[ia] = nwa;
                if (real_b) a.walked[ib] = nwb;
            }
        }
    }
    }
    if (FINAL) {
        if (kAccShared) {
            sum = tsum[threadIdx.x];
            bad = tbad[threadIdx.x];
        }
        // warp then block reduction of the checksum, one atomic per block
#pragma unroll
        for (int d = 16; d; d >>= 1) {
            sum += __shfl_xor_sync(0xffffffffu, sum, d);
            bad += __shfl_xor_sync(0xffffffffu, bad, d);
        }
        if ((threadIdx.x & 31) == 0) {
            wsum[threadIdx.x >> 5] = sum;
            wbad[threadIdx.x >> 5] = bad;
        }
    }
    __syncthreads();
    if (FINAL && threadIdx.x == 0) {
        u64 s = 0;
        u32 b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {   // blocks of 256 or 128 threads
            s += wsum[w];
            b += wbad[w];
        }
        if (s) atomicAdd(&a.ctr->raw_sum, s);
        if (b) atomicOr(&a.ctr->flags, FLAG_VALIDATION);
        if (blockIdx.x == 0 && a.count_candidates) {
            atomicAdd(&a.ctr->primecount, (u64)ncand);
            atomicMax(&a.ctr->maxcand, ncand);
            if (ncand > a.cap) atomicOr(&a.ctr->flags, FLAG_CAND_OVERFLOW);
        }
    }
    // flush the staged hits
    const u32 nh = st.n < kHitStage ? st.n : kHitStage;
    if (nh) {
        __shared__ u32 gbase;
        if (threadIdx.x == 0) gbase = atomicAdd(&a.ctr->nhits, nh);
        __syncthreads();
        for (u32 j = threadIdx.x; j < nh; j += blockDim.x) {
            const u32 g = gbase + j;
            if (g < a.hitcap)
                a.hits[g] = st.buf[j];
            else
                atomicOr(&a.ctr->flags, FLAG_HIT_OVERFLOW);
        }
    }
}

}  // namespace fs
