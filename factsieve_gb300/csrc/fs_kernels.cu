// fs_kernels.cu -- the GPU kernels of the FactSieve search path (sm_103a).
//
//   gen_kernel          candidate generation: odd numbers of [low, high) with
//                       no prime factor <= 113 that pass the base-2 strong
//                       PRP test (reference kernels/getsegprimes.cl:170-239)
//   (the fused sieve kernel is in fs_walk.cuh, built by fs_sieve2.cu and
//   fs_sieve4.cu; the batch and serving kernels are in fs_multi.cu)
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
#include "fs_walk.cuh"

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
        const u32 w32 = (u32)w;          // the host keeps nwords below 2^31
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
        // Odd index relative to the block's first word wb: below 256 * 32, so
        // it fits a u32 for any segment width (an index relative to o0 would
        // wrap once w reaches 2^27).
        while (sv) {
            int i = __ffs(sv) - 1;
            sv &= sv - 1;
            queue[warp][off++] = (u32)threadIdx.x * 32u + (u32)i;
        }
        __syncwarp();
        const u64 block_o = a.o0 + 64 * wb;
        for (u32 jb = 0; jb < total; jb += 32) {
            const u32 j = jb + lane;
            bool pass = false;
            u64 n = 0;
            if (j < total) {
                n = block_o + 2 * (u64)queue[warp][j];
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

// ========================================================== table check ====

// Direct product 2*3*...*n0 mod the first candidate, reduced over the grid
// (the last block to finish combines), against the plan's product.
__global__ void __launch_bounds__(256) table_check_kernel(TableCheckArgs a) {
    __shared__ u64 part[256];
    __shared__ bool last;
    // the segment's first candidate, as the reference checks; a segment without
    // candidates checks against the prime 2^61 - 1 instead, so the check never
    // passes silently
    const Prime c = make_prime(*a.ncand ? a.cand[0] : 2305843009213693951ull);
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
//   kind 11 32-bit half-offset steps (half32_walk8x2), 4 chains
//   kind 12 shifted-window half-offset 64-bit steps (halfmid_walk8x2), 4 chains
//   kind 13 half-offset canonical 96-bit steps (canon96h_walk8x2), 4 chains
//   kind 14 half-offset 64-bit steps, quotient on the FP32 pipe (halff_walk8x2), 4 chains
//   kind 15 folding products modulo p = 2^63 + d (pm_mul), 8 chains
//   kind 16 float-quotient steps, k_max-aware window, s >= 32 (HG: halff_walk8x2), 4 chains
//   kind 17 the same with s <= 32 (HGL: halfgl_walk8x2), 4 chains
//   kind 18 the same with a 96-bit t (HG96: halfg96_walk8x2), 4 chains
//   kind 19 half-offset 96-bit steps for p >= 2^63 with that quotient
//           (canon96g_walk8x2), 4 chains
constexpr u32 kCeilUnits[20] = {0, 0, 0, 0, 8, 32, 32, 32, 32, 4, 32, 32, 32, 32, 32, 8, 32, 32, 32, 32};

template <u32 kind>
__global__ void __launch_bounds__(256) ceiling_kernel(u32 iters, u32 seed, u32* sink) {
    const u32 tid = blockIdx.x * blockDim.x + threadIdx.x;
    // moduli in each regime's range (odd; the arithmetic is exact for any odd modulus)
    u64 base;
    switch (kind) {
        case 5: base = 1000000000000ull; break;           // 2^36 <= p, p kmax <= 2^62
        case 14: base = 1000000000000ull; break;          // 2^38 <= p, 19 p kmax < 2^(bitlen(p) + 23)
        case 16: base = 1000000000000ull; break;          // window shift s >= 32, t < 2^64
        case 17: base = (1ull << 34) + 1; break;          // window shift s <= 32
        case 18: base = 1000000000000000ull; break;       // t beyond 2^64, p < 2^63
        case 6: base = (1ull << 34) + 1; break;           // 2^33 < p < 2^36
        case 7: base = 1000000000000000ull; break;        // p kmax > 2^62, p < 2^63
        case 10: base = 1000000000000000ull; break;       // p kmax > 2^60, p < 2^63
        case 11: base = 1000000001ull; break;             // p < 2^31
        case 12: base = (1ull << 33) + 1; break;          // 2^31 <= p < 2^36
        case 13: base = (1ull << 63) + 1; break;          // p >= 2^63
        case 8: base = (1ull << 63) + 1; break;           // p >= 2^63
        default: base = (1ull << 63) + 1; break;
    }
    Prime c[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) c[h] = make_prime((base + 2ull * (4ull * tid + h) + 2ull * seed) | 1ull);
    const u32 k0 = 100001;   // multipliers k0 .. k0 + 8 iters: below 2^28 and p k below each regime's bound
    u32 acc = 0;
    if constexpr (kind == 15) {
        // moduli 2^63 + d with d < 2^30: base + 2 (4 tid + h) + 2 seed stays below 2^63 + 2^30
        // for the grids of fs_bench_int_pipe (8 blocks of 256 threads per SM)
        u64 x[8];
        PMod m[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) m[h] = make_pmod(c[h].p);
#pragma unroll
        for (int h = 0; h < 8; ++h) x[h] = c[h & 3].one + h;
        const u64 y = c[0].r2;
        for (u32 it = 0; it < iters; ++it) {
#pragma unroll
            for (int h = 0; h < 8; ++h) x[h] = pm_mul(x[h], y, m[h & 3]);
        }
#pragma unroll
        for (int h = 0; h < 8; ++h) acc ^= (u32)x[h] ^ (u32)(x[h] >> 32);
    } else if constexpr (kind == 4) {
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
        } else if constexpr (kind == 14) {
            const u64 f = umin64(umin64(c[0].p, c[1].p), umin64(c[2].p, c[3].p));
            const HalfF A = make_halff(c[0], f), B = make_halff(c[1], f);
            const HalfF C = make_halff(c[2], f), D = make_halff(c[3], f);
            for (u32 it = 0; it < iters; ++it) {
                acc += halff_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += halff_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 16 || kind == 17 || kind == 18) {
            const u32 kmax = k0 + 8 * iters;
            const int form = kind == 16 ? 0 : (kind == 17 ? 1 : 2);
            const HalfF A = make_halfg(c[0], kmax, form), B = make_halfg(c[1], kmax, form);
            const HalfF C = make_halfg(c[2], kmax, form), D = make_halfg(c[3], kmax, form);
            for (u32 it = 0; it < iters; ++it) {
                if constexpr (kind == 16) {
                    acc += halff_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                    acc += halff_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
                } else if constexpr (kind == 17) {
                    acc += halfgl_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                    acc += halfgl_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
                } else {
                    acc += halfg96_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                    acc += halfg96_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
                }
            }
        } else if constexpr (kind == 6) {
            const Lazy64 A = make_lazy(c[0]), B = make_lazy(c[1]), C = make_lazy(c[2]), D = make_lazy(c[3]);
            for (u32 it = 0; it < iters; ++it) {
                acc += lazy_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += lazy_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 11) {
            const u32 kmax = k0 + 8 * iters;
            const Half32 A = make_half32(c[0], kmax), B = make_half32(c[1], kmax);
            const Half32 C = make_half32(c[2], kmax), D = make_half32(c[3], kmax);
            for (u32 h = 0; h < 4; ++h) hh[h] = 0;
            for (u32 h = 0; h < 4; ++h) l[h] = (u32)(c[h].one % c[h].p);
            for (u32 it = 0; it < iters; ++it) {
                acc += half32_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += half32_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 12) {
            const u32 kmax = k0 + 8 * iters;
            const Half96 A = make_halfmid(c[0], kmax), B = make_halfmid(c[1], kmax);
            const Half96 C = make_halfmid(c[2], kmax), D = make_halfmid(c[3], kmax);
            for (u32 it = 0; it < iters; ++it) {
                acc += halfmid_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += halfmid_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 13) {
            const u32 kmax = k0 + 8 * iters;
            const Canon96H A = make_canon96h(c[0], kmax), B = make_canon96h(c[1], kmax);
            const Canon96H C = make_canon96h(c[2], kmax), D = make_canon96h(c[3], kmax);
            for (u32 it = 0; it < iters; ++it) {
                acc += canon96h_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += canon96h_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
            }
        } else if constexpr (kind == 19) {
            const u32 kmax = k0 + 8 * iters;
            const Canon96G A = make_canon96g(c[0], kmax), B = make_canon96g(c[1], kmax);
            const Canon96G C = make_canon96g(c[2], kmax), D = make_canon96g(c[3], kmax);
            for (u32 it = 0; it < iters; ++it) {
                acc += canon96g_walk8x2(l[0], hh[0], l[1], hh[1], k0 + 8 * it, A, B);
                acc += canon96g_walk8x2(l[2], hh[2], l[3], hh[3], k0 + 8 * it, C, D);
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

cudaError_t launch_setup_partial(const SieveArgs& a, int grid_x, int nchunks, cudaStream_t s) {
    dim3 g(grid_x, nchunks);
    setup_partial_kernel<<<g, kSieveThreads, 0, s>>>(a);
    return cudaGetLastError();
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
        case 11: ceiling_kernel<11><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 12: ceiling_kernel<12><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 13: ceiling_kernel<13><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 14: ceiling_kernel<14><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 15: ceiling_kernel<15><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 16: ceiling_kernel<16><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 17: ceiling_kernel<17><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 18: ceiling_kernel<18><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        case 19: ceiling_kernel<19><<<grid, 256, 0, s>>>(iters, seed, sink); break;
        default: imad_bench_kernel<<<grid, 256, 0, s>>>(iters, kind, seed, sink); break;
    }
    return cudaGetLastError();
}

double bench_units_per_thread_iter(u32 kind) { return kind < 4 ? 8.0 : (kind < 20 ? kCeilUnits[kind] : 0.0); }

// bitlen(ceil(23 p kmax / 16)) - 24: the window shift of make_halfg.
static int halfg_window_host(uint64_t p, uint32_t kmax) {
    const unsigned __int128 T = ((unsigned __int128)23 * p * kmax + 15) / 16;
    const uint64_t th = (uint64_t)(T >> 64), tl = (uint64_t)T;
    return (th ? 128 - __builtin_clzll(th) : 64 - __builtin_clzll(tl)) - 24;
}

int walk_for_range(uint64_t plo, uint64_t phi, uint32_t kmax) {
    if (phi <= plo || kmax == 0) return WALK_ANY;
    const uint64_t pmax = phi - 1;
    const int kb = 32 - __builtin_clz(kmax);
    // the 32-bit half-offset step needs 2 < p < 2^31 and kmax < 2^26 (half32_ok)
    if (plo > 2 && pmax < (1ull << 31) && kb <= 26) return WALK_H32;
    // the float-quotient half-offset step needs p >= 2^38, p kmax <= 2^62,
    // 19 kmax <= 2^23 and 19 pmax kmax < 2^(bitlen(plo) + 23) (the bounds
    // of halff_walk8x2 with s taken from a thread's least candidate; launch-
    // wide only, no per-candidate test)
    if (plo >= (1ull << 38) && pmax <= ((1ull << 62) / kmax) && 19ull * kmax <= (1ull << 23) &&
        (unsigned __int128)19 * pmax * kmax < ((unsigned __int128)1 << ((64 - __builtin_clzll(plo)) + 23)))
        return WALK_HF;
    // the float-quotient steps with a k_max-aware window (make_halfg) need
    // p >= 2^31 and 46 kmax < 7 2^23, and every candidate's window shift
    // s = bitlen(ceil(23 p kmax / 16)) - 24 on one side of 32: s <= 32 with
    // t < 2^64 (HGL), s >= 32 with t < 2^64 (HG), s in [32, 64) with p < 2^63
    // (HG96, t up to 96 bits)
    if (plo >= (1ull << 31) && (pmax >> 63) == 0 && kmax <= kHalfGMaxK) {
        const int slo = halfg_window_host(plo, kmax), shi = halfg_window_host(pmax, kmax);
        const bool t64 = ((unsigned __int128)23 * pmax * kmax + 15) / 16 < ((unsigned __int128)1 << 64);
        if (t64 && shi <= 32) return WALK_HGL;
        if (t64 && slo >= 32) return WALK_HG;
        if (slo >= 32 && shi < 64 && (pmax >> 63) == 0) return WALK_HG96;
    }
    // the shifted-window half-offset step needs 2^31 <= p < 2^36 and kmax < 2^25 (halfmid_ok);
    // HGL runs the same range 14 % faster and is taken first where it holds
    if (plo >= (1ull << 31) && pmax < (1ull << 36) && kb <= 25) return WALK_HM;
    // the half-offset lazy step needs p >= 2^36 and p kmax <= 2^62 (half_ok)
    if (plo >= (1ull << 36) && pmax <= ((1ull << 62) / kmax)) return WALK_H64;
    // the lazy 64-bit step needs p > 2^33 and p kmax <= 2^62 (lazy_ok)
    if (plo > (1ull << 33) && pmax <= ((1ull << 62) / kmax)) return WALK_T64;
    // the half-offset lazy 96-bit step needs 2^33 < p < 2^63, kmax < 2^26 and
    // bitlen(p) + bitlen(kmax) >= 61 (half96_ok)
    if (kb <= 26 && plo > (1ull << 33) && (pmax >> 63) == 0 && (64 - __builtin_clzll(plo)) + kb >= 61)
        return WALK_H96;
    if (kb <= 28 && plo > (1ull << 33) && (pmax >> 63) == 0) return WALK_L96;
    // the same with the float quotient for p >= 2^63 (canon96g_ok): 46 kmax < 7 2^23
    if ((plo >> 63) != 0 && kmax <= kHalfGMaxK) return WALK_C96G;
    // the half-offset canonical 96-bit step needs p >= 2^63 and kmax < 2^26 (canon96h_ok)
    if (kb <= 26 && (plo >> 63) != 0) return WALK_C96H;
    if (kb <= 28 && (plo >> 63) != 0) return WALK_C96;
    return WALK_ANY;
}

int pm_setup_for_range(uint64_t plo, uint64_t phi) {
    // candidates are odd, so p >= 2^63 means d >= 1
    if (phi <= plo) return 0;
    return plo >= (1ull << 63) && phi - 1 < (1ull << 63) + (1ull << 30) ? 1 : 0;
}

int sieve_threads() { return kSieveThreads; }
int gen_threads() { return kGenWarps * 32; }

// variant 3: two candidates per thread at 3 resident blocks per SM, every
// walk step (WALK_ANY: chosen per candidate); variant 5: four candidates per
// thread at 2 blocks per SM, for a step valid over the whole launch (a
// WALK_ANY launch runs variant 3).
cudaError_t launch_sieve(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s,
                         int variant, int walk, int threads) {
    if (variant == 5 && walk != WALK_ANY) return launch_sieve_quad(a, setup, final_chunk, grid, s, walk, threads);
    return launch_sieve_pair(a, setup, final_chunk, grid, s, walk, threads);
}

cudaError_t sieve_occupancy(int* blocks_per_sm, int variant, int threads) {
    return variant == 5 ? sieve_quad_occupancy(blocks_per_sm, threads) : sieve_pair_occupancy(blocks_per_sm, threads);
}

}  // namespace fs
