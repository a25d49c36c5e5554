// fs_kernels.cu -- the GPU kernels of the FactSieve search path (sm_103a).
//
//   gen_kernel          candidate generation: odd numbers of [low, high) with
//                       no prime factor <= 113 that pass the base-2 strong
//                       PRP test (reference kernels/getsegprimes.cl:170-239)
//   sieve_kernel<S,F>   per candidate p: starting residue nstart!*R mod p from
//                       the bit-layered power table (setup.cl:49-103), the
//                       residue walk r <- r*(n+1) with the +-1 hit test for n
//                       in [nstart, nend) (iterate.cl:54-80), and on the last
//                       n-chunk the checksum s6 + s7 and the nmax round trip
//                       (check.cl:50-109).  S selects where the starting
//                       residue comes from, F whether this chunk finishes.
//   setup_partial_kernel  one chunk of the power table for a tile of
//                       candidates, into a per-chunk partial product (used
//                       when there are too few candidates to fill the GPU)
//   table_check_kernel  one-shot check of the setup plan against the direct
//                       product 2*3*...*n mod the first candidate
//                       (verifyslow/verifypow/verifyreduce/verifyresult.cl)
//   imad_bench_kernel   dependency-free integer streams that measure the
//                       IMAD / ALU pipe rates used as the roofline
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_arith.cuh"
#include "fs_kernels.cuh"
#include "fs_launch.h"

namespace fs {

// ============================================================ generator ====

// Odd primes whose multiples the generator removes before the PRP test: the
// mod-30 wheel (3, 5) and the reference's mask primes 7..113.
static __device__ constexpr u32 kSmallQ[29] = {3,  5,  7,  11, 13, 17, 19, 23, 29,  31,  37,  41,  43,  47, 53,
                                    59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};

// Bits at 0, q, 2q, ... below 32: the divisibility pattern of 32 consecutive
// odd numbers by q, anchored at a multiple of q.
__host__ __device__ constexpr u32 pattern_of(u32 q) {
    u32 m = 0;
    for (u32 i = 0; i < 32; i += q) m |= 1u << i;
    return m;
}

constexpr int kGenWarps = 8;
constexpr int kGenQueue = 32 * 32;   // one slot per odd number of the warp's 32 words (at most 18 per word survive)

// One "word" = 32 consecutive odd numbers o0 + 64 w + 2 i, i in [0, 32).
__global__ void __launch_bounds__(kGenWarps * 32) gen_kernel(GenArgs a) {
    __shared__ u32 queue[kGenWarps][kGenQueue];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 stride = (u64)gridDim.x * blockDim.x;
    for (u64 wb = (u64)blockIdx.x * blockDim.x; wb < a.nwords; wb += stride) {
        const u64 w = wb + threadIdx.x;
        const u32 w32 = (u32)w;          // the host keeps nwords below 2^32
        u32 sv = 0;
        if (w < a.nwords) {
            u32 comp = 0;
#pragma unroll
            for (int j = 0; j < 29; ++j) {
                const u32 q = kSmallQ[j];
                // residue of the word's first number o0 + 64 w
                u32 r = (a.r0[j] + 64u * (w32 % q)) % q;
                // first i with q | r + 2i: i0 = (q - r) * (q+1)/2 mod q
                u32 i0 = ((q - r) * ((q + 1) >> 1)) % q;
                comp |= i0 < 32 ? (pattern_of(q) << i0) : 0u;
            }
            sv = ~comp;
            const u64 base = a.o0 + 64 * w;
            const u64 room = a.high - base;              // > 0 since base < high
            const u64 nvalid = (room + 1) >> 1;         // odd numbers below high
            if (nvalid < 32) sv &= (1u << nvalid) - 1u;
        }
        // warp-wide exclusive scan of survivor counts
        const u32 cnt = __popc(sv);
        u32 incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            u32 v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += v;
        }
        const u32 total = __shfl_sync(0xffffffffu, incl, 31);
        u32 off = incl - cnt;
        while (sv) {
            int i = __ffs(sv) - 1;
            sv &= sv - 1;
            queue[warp][off++] = w32 * 32u + (u32)i;   // odd index relative to o0
        }
        __syncwarp();
        for (u32 jb = 0; jb < total; jb += 32) {
            const u32 j = jb + lane;
            bool pass = false;
            u64 n = 0;
            if (j < total) {
                n = a.o0 + 2 * (u64)queue[warp][j];
                pass = sprp2(n);
            }
            const u32 bal = __ballot_sync(0xffffffffu, pass);
            if (bal) {
                u32 base = 0;
                if (lane == 0) base = atomicAdd(&a.ctr->ncand, (u32)__popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (pass) {
                    u32 slot = base + __popc(bal & ((1u << lane) - 1u));
                    if (slot < a.cap) a.cand[slot] = n;
                }
            }
        }
        __syncwarp();
    }
}

// ================================================================ sieve ====

constexpr int kSieveThreads = 256;
constexpr int kHitStage = 128;

struct HitStage {
    Factor buf[kHitStage];
    u32 n;
};

// Record a hit: lanes that hit together take consecutive slots of the block's
// shared-memory stage with one shared atomic (warp-ballot compaction); a full
// stage spills straight to the global list.
__device__ __noinline__ void record_hit(HitStage& st, u64 p, int nc, Factor* hits, u32 hitcap,
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

// The same for four candidates: four independent product chains per table
// load, for the four-candidate sieve kernel.
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
        for (; i + 2 <= L.end; i += 2) {
            const ulonglong2 w2 = __ldg(reinterpret_cast<const ulonglong2*>(words + i));
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], w2.x, c[h].p, c[h].pinv);
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], w2.y, c[h].p, c[h].pinv);
        }
        if (i < L.end) {
            const u64 w = __ldg(words + i);
#pragma unroll
            for (int h = 0; h < 4; ++h) x[h] = mont_mul(x[h], w, c[h].p, c[h].pinv);
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
    static __device__ __forceinline__ K make(const Prime& c, u32) { return make_lazy(c); }
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
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax) { return make_lazy96(c, kmax); }
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
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax) { return make_canon96(c, kmax); }
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
    static __device__ __forceinline__ K make(const Prime& c, u32) { return make_half(c); }
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
struct RegH96 {
    using K = Half96;
    static __device__ __forceinline__ K make(const Prime& c, u32 kmax) { return make_half96(c, kmax); }
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

// Replay eight steps from r at n0 with exact tests (the PTX block saw a
// possible hit in them); the residues are the same bits as the block's.
template <class Reg>
__device__ __noinline__ void reg_replay8(u64 r, u32 n0, typename Reg::K X, WalkOut o) {
    for (u32 j = 0; j < 8; ++j) {
        reg_check<Reg>(r, n0 + j, X, o);
        r = Reg::step(r, n0 + j + 1, X);
    }
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
    const typename Reg::K A = Reg::make(a, nend);
    const typename Reg::K B = real_b ? Reg::make(b, nend) : A;
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

// Walk regime of one candidate for multipliers up to kmax: 4 / 5 lazy 64-bit
// / 96-bit in half-offset form, 1 lazy 64-bit, 2 lazy 96-bit, 3 canonical
// 96-bit, 0 generic Montgomery.
__device__ __forceinline__ int walk_regime(u64 p, u32 kmax) {
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
    if (WALK == WALK_H64) walk_reg_pair<RegH64>(ra, rb, a, b, real_b, nstart, nend, o);
    else if (WALK == WALK_H96) walk_reg_pair<RegH96>(ra, rb, a, b, real_b, nstart, nend, o);
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
    const typename Reg::K K0 = Reg::make(c[0], nend), K1 = Reg::make(c[1], nend);
    const typename Reg::K K2 = Reg::make(c[2], nend), K3 = Reg::make(c[3], nend);
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
    if (WALK == WALK_H64) walk_reg4<RegH64>(r, c, nreal, nstart, nend, o);
    else if (WALK == WALK_H96) walk_reg4<RegH96>(r, c, nreal, nstart, nend, o);
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
        case WALK_H64: walk_quad_as<WALK_H64>(r, c, nreal, nstart, nend, o); break;
        case WALK_H96: walk_quad_as<WALK_H96>(r, c, nreal, nstart, nend, o); break;
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
__device__ __forceinline__ void final_check(const Prime& c, u64 r, u32 nmax, u64& sum, u32& bad) {
    const u64 s7 = to_mont(nmax, c);
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

template <int SETUP, bool FINAL, int MINB, int WALK, int PPT>
__global__ void __launch_bounds__(kSieveThreads, MINB) sieve_kernel(SieveArgs a) {
    __shared__ HitStage st;
    __shared__ u64 wsum[kSieveThreads / 32];
    __shared__ u32 wbad[kSieveThreads / 32];
    if (threadIdx.x == 0) st.n = 0;
    __syncthreads();
    const u32 ncand = *a.ncand;
    const u32 n = ncand < a.cap ? ncand : a.cap;
    const WalkOut o{&st, a.hits, a.hitcap, a.ctr, 0};
    u64 sum = 0;
    u32 bad = 0;
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
            if (SETUP == SETUP_PLAN) {
                plan_product4(c, a.plan.words, a.plan.layers, a.plan.layer_begin, a.plan.layer_end, r);
#pragma unroll
                for (int h = 0; h < 4; ++h)
                    r[h] = mont_mul(r[h], mont_pow(c[h].r2, a.plan.deficit, c[h]), c[h].p, c[h].pinv);
            } else {
                r[0] = start_residue_one<SETUP>(a, c[0], i0);
#pragma unroll
                for (int h = 1; h < 4; ++h) r[h] = (u32)h < nreal ? start_residue_one<SETUP>(a, c[h], i0 + h) : r[0];
            }
            walk_quad_as<WALK>(r, c, nreal, a.nstart, a.nend, o);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                if ((u32)h >= nreal) break;
                if (FINAL) {
                    const u64 s7 = to_mont(a.nmax, c[h]);
                    u32 back = (u32)mont_mul(s7, 1, c[h].p, c[h].pinv);
                    if (c[h].p <= a.nmax && a.nmax % c[h].p == back) back = a.nmax;
                    bad += back != a.nmax;
                    sum += r[h] + s7;
                    if (a.store_final) a.residue[i0 + h] = r[h];
                } else {
                    a.residue[i0 + h] = r[h];
                }
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
        if (FINAL) {
            // s7 = nmax*R mod p, the reference's final Montgomery image of n
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (h == 1 && !real_b) break;
                const Prime& c = h ? cb : ca;
                const u64 r = h ? rb : ra;
                const u64 s7 = to_mont(a.nmax, c);
                u32 back = (u32)mont_mul(s7, 1, c.p, c.pinv);
                if (c.p <= a.nmax && a.nmax % c.p == back) back = a.nmax;
                bad += back != a.nmax;
                sum += r + s7;
            }
            if (a.store_final) {
                a.residue[ia] = ra;
                if (real_b) a.residue[ib] = rb;
            }
        } else {
            a.residue[ia] = ra;
            if (real_b) a.residue[ib] = rb;
        }
    }
    }
    if (FINAL) {
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
        for (int w = 0; w < kSieveThreads / 32; ++w) {
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

// One chunk of the plan for candidates [0, n): partials[chunk * cap + i].
__global__ void __launch_bounds__(kSieveThreads) setup_partial_kernel(SieveArgs a) {
    const u32 ncand = *a.ncand;
    const u32 n = ncand < a.cap ? ncand : a.cap;
    const u32 chunk = blockIdx.y;
    const PlanChunkDev pc = a.chunks[chunk];
    const u32 stride = gridDim.x * blockDim.x;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const Prime c = make_prime(a.cand[i]);
        a.partials[(u64)chunk * a.cap + i] =
            plan_product(c, a.plan.words, a.plan.layers, pc.layer_begin, pc.layer_end);
    }
}

// ============================================================ batches ====

// Persistent kernel over many uneven jobs.  A tile is kTileCandidates
// candidates of one job, four per thread; blocks take tiles from a global
// counter until the batch is done.  The host orders jobs by estimated work
// per candidate, heaviest first, so the long tiles start early and the tail
// is made of short ones.  Each job carries the walk step valid for its whole
// p-range, uniform over a tile.
constexpr int kBatchMaxJobs = 1024;

__global__ void __launch_bounds__(kSieveThreads, 2) batch_sieve_kernel(BatchArgs a) {
    __shared__ HitStage st;
    __shared__ u32 tile_end[kBatchMaxJobs];   // inclusive prefix sum of tiles per job
    __shared__ u32 s_tile;
    __shared__ u64 wsum[kSieveThreads / 32];
    __shared__ u32 wbad[kSieveThreads / 32];
    const u32 per_tile = kTileCandidates;
    if (threadIdx.x == 0) {
        st.n = 0;
        u32 acc = 0;
        for (u32 j = 0; j < a.njobs; ++j) {
            const u32 nc = a.ctr[j].ncand;
            const u32 n = nc < a.jobs[j].cap ? nc : a.jobs[j].cap;
            acc += (n + per_tile - 1) / per_tile;
            tile_end[j] = acc;
        }
    }
    __syncthreads();
    const u32 total = tile_end[a.njobs - 1];
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const u32 t = s_tile;
        __syncthreads();
        if (t >= total) break;
        // job of tile t: first j with tile_end[j] > t (binary search)
        u32 lo = 0, hi = a.njobs - 1;
        while (lo < hi) {
            const u32 mid = (lo + hi) >> 1;
            if (tile_end[mid] > t) hi = mid;
            else lo = mid + 1;
        }
        const u32 j = lo;
        const BatchJob& J = a.jobs[j];
        const u32 nc = a.ctr[j].ncand;
        const u32 n = nc < J.cap ? nc : J.cap;
        const u32 i0 = (t - (j ? tile_end[j - 1] : 0)) * per_tile + 4 * threadIdx.x;
        u64 sum = 0;
        u32 bad = 0;
        if (i0 < n) {
            const WalkOut o{&st, a.hits, a.hitcap, a.gctr, (int)j};
            Prime c[4];
            const u32 nreal = load_quad(J.cand, i0, n, c);
            u64 r[4];
            plan_product4(c, a.words, a.layers, J.layer_begin, J.layer_end, r);
#pragma unroll
            for (int h = 0; h < 4; ++h) r[h] = mont_mul(r[h], mont_pow(c[h].r2, J.deficit, c[h]), c[h].p, c[h].pinv);
            walk_quad_rt((int)J.walk, r, c, nreal, J.nstart, J.nend, o);
#pragma unroll
            for (int h = 0; h < 4; ++h)
                if ((u32)h < nreal) final_check(c[h], r[h], J.nend, sum, bad);
        }
#pragma unroll
        for (int d = 16; d; d >>= 1) {
            sum += __shfl_xor_sync(0xffffffffu, sum, d);
            bad += __shfl_xor_sync(0xffffffffu, bad, d);
        }
        if ((threadIdx.x & 31) == 0) {
            wsum[threadIdx.x >> 5] = sum;
            wbad[threadIdx.x >> 5] = bad;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 s = 0;
            u32 b = 0;
            for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
                s += wsum[w];
                b += wbad[w];
            }
            if (s) atomicAdd(&a.ctr[j].raw_sum, s);
            if (b) atomicOr(&a.ctr[j].flags, FLAG_VALIDATION);
        }
    }
    __syncthreads();
    const u32 nh = st.n < kHitStage ? st.n : kHitStage;
    if (nh) {
        __shared__ u32 gbase;
        if (threadIdx.x == 0) gbase = atomicAdd(&a.gctr->nhits, nh);
        __syncthreads();
        for (u32 k = threadIdx.x; k < nh; k += blockDim.x) {
            const u32 g = gbase + k;
            if (g < a.hitcap)
                a.hits[g] = st.buf[k];
            else
                atomicOr(&a.gctr->flags, FLAG_HIT_OVERFLOW);
        }
    }
}

// ============================================================ serving ====

// One round of the serving loop: a list of tiles, each up to kTileCandidates
// candidates of one job in one phase (starting residue from the plan, a
// chunk of the walk, the final checksum), four per thread, taken from a
// global counter by persistent blocks.  Residues live in each job's device
// buffer between rounds.
__global__ void __launch_bounds__(kSieveThreads, 2) serve_round_kernel(ServeArgs a) {
    __shared__ HitStage st;
    __shared__ u32 s_tile;
    __shared__ u64 wsum[kSieveThreads / 32];
    __shared__ u32 wbad[kSieveThreads / 32];
    if (threadIdx.x == 0) st.n = 0;
    __syncthreads();
    const u32 per_tile = kTileCandidates;
    const u32 ntiles = a.nchunks ? a.chunks[a.nchunks - 1].tile_end : 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const u32 t = s_tile;
        __syncthreads();
        if (t >= ntiles) break;
        // chunk of tile t: first c with tile_end > t
        u32 lo = 0, hi = a.nchunks - 1;
        while (lo < hi) {
            const u32 mid = (lo + hi) >> 1;
            if (a.chunks[mid].tile_end > t) hi = mid;
            else lo = mid + 1;
        }
        const ServeChunk T = a.chunks[lo];
        const u32 tile0 = lo ? a.chunks[lo - 1].tile_end : 0;
        const u32 i0 = T.first + (t - tile0) * per_tile + 4 * threadIdx.x;
        const u32 end = T.first + T.count;
        u64 sum = 0;
        u32 bad = 0;
        if (i0 < end) {
            const WalkOut o{&st, a.hits, a.hitcap, a.gctr, (int)T.tag};
            Prime c[4];
            const u32 nreal = load_quad(T.cand, i0, end, c);
            u64 r[4];
            if (T.flags & SERVE_SETUP) {
                plan_product4(c, T.words, T.layers, T.layer_begin, T.layer_end, r);
#pragma unroll
                for (int h = 0; h < 4; ++h)
                    r[h] = mont_mul(r[h], mont_pow(c[h].r2, T.deficit, c[h]), c[h].p, c[h].pinv);
            } else {
                r[0] = T.residue[i0];
#pragma unroll
                for (int h = 1; h < 4; ++h) r[h] = (u32)h < nreal ? T.residue[i0 + h] : r[0];
            }
            walk_quad_rt((int)T.walk, r, c, nreal, T.nstart, T.nend, o);
            if (T.flags & SERVE_FINAL) {
#pragma unroll
                for (int h = 0; h < 4; ++h)
                    if ((u32)h < nreal) final_check(c[h], r[h], T.nend, sum, bad);
            } else {
#pragma unroll
                for (int h = 0; h < 4; ++h)
                    if ((u32)h < nreal) T.residue[i0 + h] = r[h];
            }
        }
    if (T.flags & SERVE_FINAL) {
#pragma unroll
            for (int d = 16; d; d >>= 1) {
                sum += __shfl_xor_sync(0xffffffffu, sum, d);
                bad += __shfl_xor_sync(0xffffffffu, bad, d);
            }
            if ((threadIdx.x & 31) == 0) {
                wsum[threadIdx.x >> 5] = sum;
                wbad[threadIdx.x >> 5] = bad;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                u64 s = 0;
                u32 b = 0;
                for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
                    s += wsum[w];
                    b += wbad[w];
                }
                if (s) atomicAdd(&T.ctr->raw_sum, s);
                if (b) atomicOr(&T.ctr->flags, FLAG_VALIDATION);
            }
        }
    }
    __syncthreads();
    const u32 nh = st.n < kHitStage ? st.n : kHitStage;
    if (nh) {
        __shared__ u32 gbase;
        if (threadIdx.x == 0) gbase = atomicAdd(&a.gctr->nhits, nh);
        __syncthreads();
        for (u32 k = threadIdx.x; k < nh; k += blockDim.x) {
            const u32 g = gbase + k;
            if (g < a.hitcap)
                a.hits[g] = st.buf[k];
            else
                atomicOr(&a.gctr->flags, FLAG_HIT_OVERFLOW);
        }
    }
}

// ========================================================== table check ====

// Direct product 2*3*...*n0 mod the first candidate, reduced over the grid
// (the last block to finish combines), against the plan's product.
__global__ void __launch_bounds__(256) table_check_kernel(TableCheckArgs a) {
    __shared__ u64 part[256];
    __shared__ bool last;
    if (*a.ncand == 0) return;
    const Prime c = make_prime(a.cand[0]);
    u64 acc = c.one;   // deficit grows by one per factor k
    const u32 stride = gridDim.x * blockDim.x;
    for (u64 k = 2 + blockIdx.x * blockDim.x + threadIdx.x; k <= a.n0; k += stride)
        acc = mont_mul(acc, k, c.p, c.pinv);
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s; s >>= 1) {
        if (threadIdx.x < s) part[threadIdx.x] = mont_mul(part[threadIdx.x], part[threadIdx.x + s], c.p, c.pinv);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.scratch[blockIdx.x] = part[0];
        __threadfence();
        u32 done = atomicAdd(a.done, 1u);
        last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    u64 direct = c.one;
    for (u32 b = 0; b < gridDim.x; ++b) direct = mont_mul(direct, ((volatile u64*)a.scratch)[b], c.p, c.pinv);
    const u64 nk = a.n0 >= 2 ? (u64)a.n0 - 1 : 0;
    direct = mont_mul(direct, mont_pow(c.r2, nk, c), c.p, c.pinv);
    u64 table = c.one;
    for (u32 k = 0; k < a.nchunks; ++k) {
        const u64 part_k = plan_product(c, a.words, a.layers, a.chunks[k].layer_begin, a.chunks[k].layer_end);
        table = mont_mul(table, part_k, c.p, c.pinv);
    }
    // the chunks' deficits add; table now carries R^(1 - D) with one extra R^-1
    // per combining product beyond the first -- combining started from one:
    // mont_mul(one, x) = x, so no extra deficit.
    table = mont_mul(table, mont_pow(c.r2, a.deficit, c), c.p, c.pinv);
    a.result[0] = direct;
    a.result[1] = table;
    *a.done = 0;
    if (direct != table) atomicOr(&a.ctr->flags, FLAG_TABLE);
}

// ============================================================ IMAD rate ====

// kind 0: IMAD (mad.lo.u32), 1: IMAD.WIDE (mad.wide.u32), 2: IMAD.HI
// (mul.hi.u32), 3: integer ALU (lop3/xor-add).  Eight independent chains per
// thread; the result is stored so the work cannot be dropped.
__global__ void __launch_bounds__(256) imad_bench_kernel(u32 iters, u32 kind, u32 seed, u32* sink) {
    u32 a0 = seed ^ threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    u32 a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const u32 b = 0x9E3779B1u ^ seed, cc = 0x7F4A7C15u;
    if (kind == 0) {
        for (u32 it = 0; it < iters; ++it) {
            asm volatile(
                "mad.lo.u32 %0, %0, %8, %9;\n\tmad.lo.u32 %1, %1, %8, %9;\n\t"
                "mad.lo.u32 %2, %2, %8, %9;\n\tmad.lo.u32 %3, %3, %8, %9;\n\t"
                "mad.lo.u32 %4, %4, %8, %9;\n\tmad.lo.u32 %5, %5, %8, %9;\n\t"
                "mad.lo.u32 %6, %6, %8, %9;\n\tmad.lo.u32 %7, %7, %8, %9;"
                : "+r"(a0), "+r"(a1), "+r"(a2), "+r"(a3), "+r"(a4), "+r"(a5), "+r"(a6), "+r"(a7)
                : "r"(b), "r"(cc));
        }
    } else if (kind == 1) {
        u64 w0 = a0, w1 = a1, w2 = a2, w3 = a3, w4 = a4, w5 = a5, w6 = a6, w7 = a7;
        for (u32 it = 0; it < iters; ++it) {
            asm volatile(
                "{.reg .u32 l0,l1,l2,l3,l4,l5,l6,l7;\n\t"
                "cvt.u32.u64 l0, %0;\n\tcvt.u32.u64 l1, %1;\n\tcvt.u32.u64 l2, %2;\n\tcvt.u32.u64 l3, %3;\n\t"
                "cvt.u32.u64 l4, %4;\n\tcvt.u32.u64 l5, %5;\n\tcvt.u32.u64 l6, %6;\n\tcvt.u32.u64 l7, %7;\n\t"
                "mad.wide.u32 %0, l0, %8, %0;\n\tmad.wide.u32 %1, l1, %8, %1;\n\t"
                "mad.wide.u32 %2, l2, %8, %2;\n\tmad.wide.u32 %3, l3, %8, %3;\n\t"
                "mad.wide.u32 %4, l4, %8, %4;\n\tmad.wide.u32 %5, l5, %8, %5;\n\t"
                "mad.wide.u32 %6, l6, %8, %6;\n\tmad.wide.u32 %7, l7, %8, %7;}"
                : "+l"(w0), "+l"(w1), "+l"(w2), "+l"(w3), "+l"(w4), "+l"(w5), "+l"(w6), "+l"(w7)
                : "r"(b));
        }
        a0 = (u32)(w0 ^ (w0 >> 32)) ^ (u32)(w1 ^ (w1 >> 32)) ^ (u32)(w2 ^ (w2 >> 32)) ^ (u32)(w3 ^ (w3 >> 32));
        a1 = (u32)(w4 ^ (w4 >> 32)) ^ (u32)(w5 ^ (w5 >> 32)) ^ (u32)(w6 ^ (w6 >> 32)) ^ (u32)(w7 ^ (w7 >> 32));
        a2 = a3 = a4 = a5 = a6 = a7 = 0;
    } else if (kind == 2) {
        for (u32 it = 0; it < iters; ++it) {
            asm volatile(
                "mul.hi.u32 %0, %0, %8;\n\tmul.hi.u32 %1, %1, %8;\n\t"
                "mul.hi.u32 %2, %2, %8;\n\tmul.hi.u32 %3, %3, %8;\n\t"
                "mul.hi.u32 %4, %4, %8;\n\tmul.hi.u32 %5, %5, %8;\n\t"
                "mul.hi.u32 %6, %6, %8;\n\tmul.hi.u32 %7, %7, %8;"
                : "+r"(a0), "+r"(a1), "+r"(a2), "+r"(a3), "+r"(a4), "+r"(a5), "+r"(a6), "+r"(a7)
                : "r"(b | 0x80000000u));
        }
    } else {
        for (u32 it = 0; it < iters; ++it) {
            asm volatile(
                "lop3.b32 %0, %0, %8, %9, 0x96;\n\tlop3.b32 %1, %1, %8, %9, 0x96;\n\t"
                "lop3.b32 %2, %2, %8, %9, 0x96;\n\tlop3.b32 %3, %3, %8, %9, 0x96;\n\t"
                "lop3.b32 %4, %4, %8, %9, 0x96;\n\tlop3.b32 %5, %5, %8, %9, 0x96;\n\t"
                "lop3.b32 %6, %6, %8, %9, 0x96;\n\tlop3.b32 %7, %7, %8, %9, 0x96;"
                : "+r"(a0), "+r"(a1), "+r"(a2), "+r"(a3), "+r"(a4), "+r"(a5), "+r"(a6), "+r"(a7)
                : "r"(b), "r"(cc));
        }
    }
    const u32 x = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
    if (x == seed) sink[blockIdx.x] = x;   // practically never true, but not provable
}

// ======================================================= ceilings ====
//
// The sieve's own arithmetic with nothing else: register-resident chains at
// full occupancy, no loads, no stores but one guarded word.  Their rates
// are the speed of light of that instruction mix on this GPU, the
// denominator of the sieve kernel's roofline.
//   kind 4  Montgomery products (mont_mul), 8 chains per thread
//   kind 5  half-offset lazy steps (the half_walk8x2 block), 4 chains
//   kind 6  lazy 64-bit steps (lazy_walk8x2), 4 chains
//   kind 7  lazy 96-bit steps (lazy96_walk8x2), 4 chains
//   kind 8  canonical 96-bit steps (canon96_walk8x2), 4 chains
//   kind 9  generic Montgomery steps (mont_mul by kR, k advanced by R), 4 chains
//   kind 10 half-offset lazy 96-bit steps (half96_walk8x2), 4 chains
constexpr u32 kCeilUnits[11] = {0, 0, 0, 0, 8, 32, 32, 32, 32, 4, 32};

template <u32 kind>
__global__ void __launch_bounds__(256) ceiling_kernel(u32 iters, u32 seed, u32* sink) {
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x;
    // moduli in each regime's range (odd; the arithmetic is exact for any odd modulus)
    u64 base;
    switch (kind) {
        case 5: base = 1000000000000ull; break;           // p kmax <= 2^60
        case 6: base = (1ull << 34) + 1; break;           // 2^33 < p, p kmax <= 2^62
        case 7: base = 1000000000000000ull; break;        // p kmax > 2^62, p < 2^63
        case 10: base = 1000000000000000ull; break;       // p kmax > 2^60, p < 2^63
        case 8: base = (1ull << 63) + 1; break;           // p >= 2^63
        default: base = (1ull << 63) + 1; break;
    }
    Prime c[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) c[h] = make_prime((base + 2ull * (4ull * tid + h) + 2ull * seed) | 1ull);
    const u32 k0 = 100001;   // multipliers k0 .. k0 + 8 iters: below 2^28 and p k below each regime's bound
    u32 acc = 0;
    if constexpr (kind == 4) {
        u64 x[8];
#pragma unroll
        for (int h = 0; h < 8; ++h) x[h] = c[h & 3].one + h;
        const u64 y = c[0].r2;
        for (u32 it = 0; it < iters; ++it) {
#pragma unroll
            for (int h = 0; h < 8; ++h) x[h] = mont_mul(x[h], y, c[h & 3].p, c[h & 3].pinv);
        }
#pragma unroll
        for (int h = 0; h < 8; ++h) acc ^= (u32)x[h] ^ (u32)(x[h] >> 32);
    } else if constexpr (kind == 9) {
        u64 r[4], k[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            r[h] = c[h].one;
            k[h] = to_mont(k0, c[h]);
        }
        for (u32 it = 0; it < iters; ++it) {
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                acc += (r[h] == c[h].one) | (r[h] == c[h].p - c[h].one);
                r[h] = mont_mul(r[h], k[h], c[h].p, c[h].pinv);
                k[h] = mod_add(k[h], c[h].one, c[h].p);
            }
        }
#pragma unroll
        for (int h = 0; h < 4; ++h) acc ^= (u32)r[h];
    } else {
        u32 l[4], hh[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            l[h] = (u32)c[h].one;
            hh[h] = (u32)(c[h].one >> 32);
        }
        if constexpr (kind == 5) {
            const Half64 A = make_half(c[0]), B = make_half(c[1]), C = make_half(c[2]), D = make_half(c[3]);
            for (u32 it = 0; it < iters; ++it) {
                acc += half_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += half_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 6) {
            const Lazy64 A = make_lazy(c[0]), B = make_lazy(c[1]), C = make_lazy(c[2]), D = make_lazy(c[3]);
            for (u32 it = 0; it < iters; ++it) {
                acc += lazy_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += lazy_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 10) {
            const u32 kmax = k0 + 8 * iters;
            const Half96 A = make_half96(c[0], kmax), B = make_half96(c[1], kmax);
            const Half96 C = make_half96(c[2], kmax), D = make_half96(c[3], kmax);
            for (u32 it = 0; it < iters; ++it) {
                acc += half96_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += half96_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 7) {
            const u32 kmax = k0 + 8 * iters;
            const Lazy96 A = make_lazy96(c[0], kmax), B = make_lazy96(c[1], kmax);
            const Lazy96 C = make_lazy96(c[2], kmax), D = make_lazy96(c[3], kmax);
            for (u32 it = 0; it < iters; ++it) {
                acc += lazy96_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += lazy96_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else {
            const u32 kmax = k0 + 8 * iters;
            const Canon96 A = make_canon96(c[0], kmax), B = make_canon96(c[1], kmax);
            const Canon96 C = make_canon96(c[2], kmax), D = make_canon96(c[3], kmax);
            for (u32 it = 0; it < iters; ++it) {
                acc += canon96_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += canon96_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        }
#pragma unroll
        for (int h = 0; h < 4; ++h) acc ^= l[h] ^ hh[h];
    }
    if (acc == 0x9E3779B9u) sink[blockIdx.x & 4095] = acc;   // keeps the work; practically never stores
}

// ============================================================== launches ===

cudaError_t launch_gen(const GenArgs& a, int grid, cudaStream_t s) {
    gen_kernel<<<grid, kGenWarps * 32, 0, s>>>(a);
    return cudaGetLastError();
}

template <int MINB, int WALK, int PPT = 2>
static void launch_sieve_w(const SieveArgs& a, int setup, bool fin, int grid, cudaStream_t s) {
    const int t = kSieveThreads;
    if (setup == SETUP_PLAN) {
        if (fin) sieve_kernel<SETUP_PLAN, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
        else sieve_kernel<SETUP_PLAN, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
    } else if (setup == SETUP_PARTIALS) {
        if (fin) sieve_kernel<SETUP_PARTIALS, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
        else sieve_kernel<SETUP_PARTIALS, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
    } else {
        if (fin) sieve_kernel<SETUP_LOAD, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
        else sieve_kernel<SETUP_LOAD, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
    }
}

// variant v: the kernel compiled for v resident blocks per SM (register cap
// 65536 / (256 v)); 0 picks the default.  walk: a step valid for every
// candidate of the launch (WALK_ANY: chosen per candidate).  The specialised
// walks are built for the default variant only.
cudaError_t launch_sieve(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s,
                         int variant, int walk) {
    if (variant == 2) {
        launch_sieve_w<2, WALK_ANY>(a, setup, final_chunk, grid, s);
    } else if (variant == 4) {
        launch_sieve_w<4, WALK_ANY>(a, setup, final_chunk, grid, s);
    } else if (variant == 5 || variant == 6) {
        // four candidates per thread, 2 (variant 5) or 3 (variant 6) blocks per SM
        switch (walk * 2 + (variant == 6)) {
            case WALK_H64 * 2: launch_sieve_w<2, WALK_H64, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_H64 * 2 + 1: launch_sieve_w<3, WALK_H64, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_H96 * 2: launch_sieve_w<2, WALK_H96, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_H96 * 2 + 1: launch_sieve_w<3, WALK_H96, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_T64 * 2: launch_sieve_w<2, WALK_T64, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_L96 * 2: launch_sieve_w<2, WALK_L96, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_C96 * 2: launch_sieve_w<2, WALK_C96, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_T64 * 2 + 1: launch_sieve_w<3, WALK_T64, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_L96 * 2 + 1: launch_sieve_w<3, WALK_L96, 4>(a, setup, final_chunk, grid, s); break;
            case WALK_C96 * 2 + 1: launch_sieve_w<3, WALK_C96, 4>(a, setup, final_chunk, grid, s); break;
            default: launch_sieve_w<3, WALK_ANY>(a, setup, final_chunk, grid, s); break;
        }
    } else {
        switch (walk) {
            case WALK_H64: launch_sieve_w<3, WALK_H64>(a, setup, final_chunk, grid, s); break;
            case WALK_H96: launch_sieve_w<3, WALK_H96>(a, setup, final_chunk, grid, s); break;
            case WALK_T64: launch_sieve_w<3, WALK_T64>(a, setup, final_chunk, grid, s); break;
            case WALK_L96: launch_sieve_w<3, WALK_L96>(a, setup, final_chunk, grid, s); break;
            case WALK_C96: launch_sieve_w<3, WALK_C96>(a, setup, final_chunk, grid, s); break;
            default: launch_sieve_w<3, WALK_ANY>(a, setup, final_chunk, grid, s); break;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_setup_partial(const SieveArgs& a, int grid_x, int nchunks, cudaStream_t s) {
    dim3 g(grid_x, nchunks);
    setup_partial_kernel<<<g, kSieveThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchArgs& a, int grid, cudaStream_t s) {
    if (a.njobs == 0 || a.njobs > (u32)kBatchMaxJobs) return cudaErrorInvalidValue;
    batch_sieve_kernel<<<grid, kSieveThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t batch_occupancy(int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, batch_sieve_kernel, kSieveThreads, 0);
}

int batch_max_jobs() { return kBatchMaxJobs; }

cudaError_t launch_serve_round(const ServeArgs& a, int grid, cudaStream_t s) {
    serve_round_kernel<<<grid, kSieveThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t serve_occupancy(int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, serve_round_kernel, kSieveThreads, 0);
}

cudaError_t launch_table_check(const TableCheckArgs& a, int grid, cudaStream_t s) {
    table_check_kernel<<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_imad_bench(u32 iters, u32 kind, u32 seed, u32* sink, int grid, cudaStream_t s) {
    switch (kind) {
        case 4: ceiling_kernel<4><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 5: ceiling_kernel<5><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 6: ceiling_kernel<6><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 7: ceiling_kernel<7><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 8: ceiling_kernel<8><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 9: ceiling_kernel<9><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 10: ceiling_kernel<10><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        default: imad_bench_kernel<<<grid, 256, 0, s>>>(iters, kind, seed, sink); break;
    }
    return cudaGetLastError();
}

double bench_units_per_thread_iter(u32 kind) { return kind < 4 ? 8.0 : (kind < 11 ? kCeilUnits[kind] : 0.0); }

int walk_for_range(uint64_t plo, uint64_t phi, uint32_t kmax) {
    if (phi <= plo || kmax == 0) return WALK_ANY;
    const uint64_t pmax = phi - 1;
    const int kb = 32 - __builtin_clz(kmax);
    // the half-offset lazy step needs p >= 2^36 and p kmax <= 2^62 (half_ok)
    if (plo >= (1ull << 36) && pmax <= ((1ull << 62) / kmax)) return WALK_H64;
    // the lazy 64-bit step needs p > 2^33 and p kmax <= 2^62 (lazy_ok)
    if (plo > (1ull << 33) && pmax <= ((1ull << 62) / kmax)) return WALK_T64;
    // the half-offset lazy 96-bit step needs 2^33 < p < 2^63, kmax < 2^26 and
    // bitlen(p) + bitlen(kmax) >= 61 (half96_ok)
    if (kb <= 26 && plo > (1ull << 33) && (pmax >> 63) == 0 && (64 - __builtin_clzll(plo)) + kb >= 61)
        return WALK_H96;
    if (kb <= 28 && plo > (1ull << 33) && (pmax >> 63) == 0) return WALK_L96;
    if (kb <= 28 && (plo >> 63) != 0) return WALK_C96;
    return WALK_ANY;
}

int sieve_threads() { return kSieveThreads; }
int gen_threads() { return kGenWarps * 32; }

cudaError_t sieve_occupancy(int* blocks_per_sm, int variant) {
    switch (variant) {
        case 2: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 2, WALK_ANY, 2>, kSieveThreads, 0);
        case 4: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 4, WALK_ANY, 2>, kSieveThreads, 0);
        case 5: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 2, WALK_T64, 4>, kSieveThreads, 0);
        case 6: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 3, WALK_T64, 4>, kSieveThreads, 0);
        default: return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                    blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 3, WALK_ANY, 2>, kSieveThreads, 0);
    }
}

}  // namespace fs
