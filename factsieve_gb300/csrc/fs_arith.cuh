// fs_arith.cuh -- exact 64-bit modular arithmetic for the FactSieve kernels.
//
// Residues live in Montgomery form with R = 2^64, the representation the
// reference's kernels use and checksum (kernels/iterate.cl:36-49): a value x
// is held as x*R mod p, always fully reduced into [0, p).  Three products
// are used:
//
//   mont_mul(a, b)     a*b/R mod p for a < p, b < 2^64.  Setup and the PRP test.
//   lazy_step(r, k)    r*k mod p for a 32-bit k by a Barrett step on residues
//                      kept in [0, 2p), valid when p > 2^33 and p*k <= 2^62.
//                      The iterate hot loop: the multiplier k = n+1 is a plain
//                      integer, so multiplying a Montgomery-form residue by it
//                      keeps the form and needs no Montgomery image of n.
//   mont_mul with kR   generic iterate step for every other (p, n) (the
//                      reference's own step: multiply by the Montgomery image
//                      of n+1, which advances by R each step).
//
// Residues leave every routine canonical (the lazy walk folds [0, 2p) back
// into [0, p) at its end), so any mix of them yields the reference's bits.
#pragma once
#include <stdint.h>

typedef unsigned long long u64;
typedef unsigned int u32;

namespace fs {

// ---------------------------------------------------------------- basics --

__device__ __forceinline__ u64 mulhi64(u64 a, u64 b) { return __umul64hi(a, b); }

// p^-1 mod 2^64 (p odd) by Newton's iteration x <- x(2 - p x).  p*p = 1 mod 8,
// so x0 = p is good to 3 bits; five steps reach 96 > 64 bits.
__device__ __forceinline__ u64 inv64(u64 p) {
    u64 x = p;
#pragma unroll
    for (int i = 0; i < 5; ++i) x *= 2 - p * x;
    return x;
}

// a*b/R mod p, result in [0, p); needs a*b < p*R (a < p suffices).
// (a*b - m*p)/R with m = (a*b mod R)*p^-1: the low halves cancel exactly,
// the high halves differ by less than p, one conditional add folds it.
__device__ __forceinline__ u64 mont_mul(u64 a, u64 b, u64 p, u64 pinv) {
    const unsigned __int128 x = (unsigned __int128)a * b;
    u64 lo = (u64)x;
    u64 hi = (u64)(x >> 64);
    u64 m = lo * pinv;
    u64 mp = mulhi64(m, p);
    u64 r = hi - mp;
    return hi < mp ? r + p : r;
}

// a + b mod p for a, b < p.
__device__ __forceinline__ u64 mod_add(u64 a, u64 b, u64 p) {
    u64 s = a + b;
    u64 t = s - p;
    // a + b >= p  <=>  a >= p - b  (no wrap reasoning needed)
    return (a >= p - b) ? t : s;
}

// Per-prime constants.  one = R mod p, r2 = R^2 mod p.
struct Prime {
    u64 p, pinv, one, r2;
};

__device__ __forceinline__ Prime make_prime(u64 p) {
    Prime c;
    c.p = p;
    c.pinv = inv64(p);
    // R mod p: for p > 2^63 it is 2^64 - p, else a single 64-bit remainder.
    c.one = (p >> 63) ? (0ull - p) : ((0ull - p) % p);
    // R^2 mod p: start from 4R, five Montgomery squarings give 4^32 * R.
    u64 two = mod_add(c.one, c.one, p);
    u64 r = mod_add(two, two, p);
#pragma unroll
    for (int i = 0; i < 5; ++i) r = mont_mul(r, r, p, c.pinv);
    c.r2 = r;
    return c;
}

// Montgomery image of a plain value x < 2^64: x*R mod p.
__device__ __forceinline__ u64 to_mont(u64 x, const Prime& c) { return mont_mul(x, c.r2, c.p, c.pinv); }

// base^e in the Montgomery domain (base and result in Montgomery form).
__device__ __forceinline__ u64 mont_pow(u64 base, u64 e, const Prime& c) {
    u64 a = c.one;
    if (e == 0) return a;
    int top = 63 - __clzll(e);
    a = base;
    for (int b = top - 1; b >= 0; --b) {
        a = mont_mul(a, a, c.p, c.pinv);
        if ((e >> b) & 1) a = mont_mul(a, base, c.p, c.pinv);
    }
    return a;
}

// ----------------- setup: products modulo p = 2^63 + d, 0 < d < 2^30 --
//
// For p just above 2^63, 2^64 = 2p - 2d, so 2^64 = -e (mod p) with e = 2d
// < 2^31, and a product folds down without Montgomery's second wide product:
//   x = a b = X1 2^64 + X0            = X0 - e X1
//   W = e X1 = W1 2^64 + W0 (W1 < e)  = W0 - e W1
//   u = X0 - W0 = u' - b 2^64         = u' + b e      (b the borrow)
// so a b = u' + e (W1 + b) (mod p), where e (W1 + b) < 2^62.  If that
// last sum carries out of 64 bits, its value is y' + 2^64 = y' + (p - e),
// and y' + p - e < 2^64.  The result is a 64-bit value congruent to a b,
// for any 64-bit a and b (lazy: pm_canon makes it canonical).  Cost: one
// full 64x64->128 product and three 32x32->64 ones, against the Montgomery
// product's full product, 64x64 low product and 64x64 high product.
struct PMod {
    u32 e;          // 2d
    u32 pe0, pe1;   // p - e = 2^63 - d, two words
};

__device__ __forceinline__ PMod make_pmod(u64 p) {
    PMod m;
    const u64 d = p - (1ull << 63);
    m.e = (u32)(d << 1);
    const u64 pe = p - 2 * d;
    m.pe0 = (u32)pe;
    m.pe1 = (u32)(pe >> 32);
    return m;
}

__device__ __forceinline__ u64 pm_mul(u64 a, u64 b, const PMod& m) {
    const unsigned __int128 x = (unsigned __int128)a * b;
    const u64 x0 = (u64)x, x1 = (u64)(x >> 64);                     // a b = x1 2^64 + x0
    const u64 t0 = (u64)m.e * (u32)x1;
    const u64 t1 = (u64)m.e * (u32)(x1 >> 32) + (t0 >> 32);         // e x1 = (t1 >> 32) 2^64 + w0
    const u64 w0 = (t1 << 32) | (u32)t0;
    const u64 u = x0 - w0;
    const u32 w1b = (u32)(t1 >> 32) + (x0 < w0 ? 1u : 0u);         // W1 + borrow < 2^31
    const u64 v = (u64)m.e * w1b;                                    // < 2^62
    const u64 y = u + v;
    const u64 pe = ((u64)m.pe1 << 32) | m.pe0;
    return y < u ? y + pe : y;                                       // a carry out: + (p - e)
}

// The canonical residue of a pm_mul result (< 2^64 < 2p).
__device__ __forceinline__ u64 pm_canon(u64 y, u64 p) { return y >= p ? y - p : y; }

// Base-2 strong probable-prime test of odd n > 2 (the candidate filter of
// kernels/getsegprimes.cl:79-108): 2^d by a left-to-right ladder whose
// doublings are modular additions, then up to t-1 squarings looking for -1.
__device__ __forceinline__ bool sprp2(u64 n) {
    if (n < 3) return false;
    const u64 pinv = inv64(n);
    const u64 one = (n >> 63) ? (0ull - n) : ((0ull - n) % n);
    const u64 nmo = n - one;
    const int t = __ffsll((long long)(n - 1)) - 1;
    const u64 d = (n - 1) >> t;
    u64 a = mod_add(one, one, n);          // 2 in Montgomery form
    if (d > 1) {
        int top = 63 - __clzll(d);
        for (int b = top - 1; b >= 0; --b) {
            a = mont_mul(a, a, n, pinv);
            if ((d >> b) & 1) a = mod_add(a, a, n);
        }
    }
    if (a == one || a == nmo) return true;
    for (int s = 1; s < t; ++s) {
        a = mont_mul(a, a, n, pinv);
        if (a == nmo) return true;
    }
    return false;
}

// ------------------------------------------- iterate: lazy Barrett step --
//
// For p in (2^33, 2^62 / kmax] the walk keeps r in [0, 2p) ("lazy") and
// multiplies by the plain 32-bit k = n + 1 (p * k <= 2^62, so t = r k < 2^63):
//
//   z  = floor(t / 2^32)            (< 2^31)
//   M  = floor(2^64 / p)            (< 2^31)
//   qe = floor(z M / 2^32)          = floor(t/p) or one less, since
//                                    t/p - z M / 2^32 < 2^32/p + z/2^32 < 1
//   r' = t - qe p                   (in [0, 2p); computed mod 2^64 as t + qe (2^64 - p))
//
// Three 32-bit multiply groups (t, qe, qe p) and no correction step.  The
// +-1 test looks at the low word of r against the four values one, one + p,
// nmo, nmo + p that r can take when r = +-R mod p; a match is checked exactly
// on the slow path.
struct Lazy64 {
    u64 p, one;               // one = R mod p
    u32 np0, np1, M;          // 2^64 - p (two words), floor(2^64 / p)
    u32 c0, c1, c2, c3;       // low words of one, one + p, p - one, 2p - one
};

__device__ __forceinline__ Lazy64 make_lazy(const Prime& c) {
    Lazy64 L;
    L.p = c.p;
    L.one = c.one;
    const u64 np = 0ull - c.p;
    L.np0 = (u32)np;
    L.np1 = (u32)(np >> 32);
    L.M = (u32)((~0ull) / c.p);
    const u64 nmo = c.p - c.one;
    L.c0 = (u32)c.one;
    L.c1 = (u32)(c.one + c.p);
    L.c2 = (u32)nmo;
    L.c3 = (u32)(nmo + c.p);
    return L;
}

// p qualifies for the lazy step for every multiplier up to kmax.
__device__ __forceinline__ bool lazy_ok(u64 p, u32 kmax) {
    return p > (1ull << 33) && p <= ((1ull << 62) / (u64)(kmax ? kmax : 1));
}

// One lazy step r <- r*k (r in [0, 2p)), bit-identical to the PTX block below.
__device__ __forceinline__ u64 lazy_step(u64 r, u32 k, const Lazy64& L) {
    const u64 t = r * (u64)k;
    const u32 qe = __umulhi((u32)(t >> 32), L.M);
    return t + (u64)qe * (((u64)L.np1 << 32) | L.np0);
}

__device__ __forceinline__ u64 lazy_canon(u64 r, const Lazy64& L) { return r >= L.p ? r - L.p : r; }

// Eight lazy steps on two independent residues (A in %0:%1, B in %2:%3)
// with multipliers k1 .. k1+7.  Before each multiply the low words are
// compared with the four hit values; the comparisons OR into one predicate
// returned as 0/1 (a hit, or a 2^-30-rare low-word coincidence, somewhere in
// the eight steps).
#define FS_LZ_TEST(RL, C0, C1, C2, C3)                 \
    "setp.eq.or.u32 P, " RL ", " C0 ", P;\n\t"         \
    "setp.eq.or.u32 P, " RL ", " C1 ", P;\n\t"         \
    "setp.eq.or.u32 P, " RL ", " C2 ", P;\n\t"         \
    "setp.eq.or.u32 P, " RL ", " C3 ", P;\n\t"
// r' = t + q (2^64 - p) is formed by a mad.lo.cc / madc.hi carry pair and
// one mad.lo rather than by a mad.wide with a 64-bit addend: on GB300 the
// latter costs two more integer ALU instructions per step (ncu), and these
// walk blocks are bound by instruction issue as much as by the multiply pipe
// (lazy 64-bit ceiling +17 %, half-offset +6 %, float quotient +8 %).  The
// blocks that keep the multiply pipe above 90 % busy (the half-offset 96-bit
// step and the half-offset canonical 96-bit step) keep the mad.wide form,
// where the extra lo/hi pipe cycles cost more than the saved ALU work.
#define FS_LZ_MUL(RL, RH, NP0, NP1, MM, T, R, TL, TH, Q)          \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                          \
    "mov.b64 {" TL ", " TH "}, " T ";\n\t"                         \
    "mad.lo.u32 " TH ", " RH ", kk, " TH ";\n\t"                   \
    "mul.hi.u32 " Q ", " TH ", " MM ";\n\t"                        \
    "mad.lo.cc.u32 " RL ", " Q ", " NP0 ", " TL ";\n\t"          \
    "madc.hi.u32 " TH ", " Q ", " NP0 ", " TH ";\n\t"            \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " TH ";\n\t"
#define FS_LZ_STEP2(J)                                              \
    "add.u32 kk, %5, " #J ";\n\t"                                   \
    FS_LZ_TEST("%0", "%9", "%10", "%11", "%12")                     \
    FS_LZ_TEST("%2", "%16", "%17", "%18", "%19")                    \
    FS_LZ_MUL("%0", "%1", "%6", "%7", "%8", "TA", "RA", "aL", "aH", "qA") \
    FS_LZ_MUL("%2", "%3", "%13", "%14", "%15", "TB", "RB", "bL", "bH", "qB")

__device__ __forceinline__ u32 lazy_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Lazy64& A,
                                            const Lazy64& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, aL, aH, qA, bL, bH, qB;\n\t"
        ".reg .u64 TA, RA, TB, RB;\n\t"
        ".reg .pred P;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_LZ_STEP2(0) FS_LZ_STEP2(1) FS_LZ_STEP2(2) FS_LZ_STEP2(3)
        FS_LZ_STEP2(4) FS_LZ_STEP2(5) FS_LZ_STEP2(6) FS_LZ_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "r"(A.M), "r"(A.c0), "r"(A.c1), "r"(A.c2), "r"(A.c3),
          "r"(B.np0), "r"(B.np1), "r"(B.M), "r"(B.c0), "r"(B.c1), "r"(B.c2), "r"(B.c3));
    return flag;
}

// ---------------------------------- iterate: 96-bit Barrett steps --
//
// When p k_max > 2^62 the product t = r k needs a third 32-bit word.  The
// quotient estimate takes 31 bits of t from bit s on, z = floor(t / 2^s),
// and a 32-bit reciprocal M = floor(2^(32+s) / p):
//
//   qe = floor(z M / 2^32),   t/p - z M / 2^32 < 2^s/p + z/2^32 < 1/2 + 1/2,
//
// so qe is floor(t/p) or one less, provided k_max < 2^28 (2^s/p <= 2^(kb-29)).
//
//   lazy96   p in (2^33, 2^63): r kept in [0, 2p) like the 64-bit lazy step,
//            s = bitlen(p) + 1 + bitlen(k_max) - 31, r' = (t - qe p) mod 2^64.
//   canon96  p in [2^63, 2^64): r canonical in [0, p), s = bitlen(p) +
//            bitlen(k_max) - 31; r' = t - qe p in [0, 2p) needs 65 bits, so
//            it is formed over three words and folded once.

// floor(2^e / p) for 64 <= e <= 95 and odd p > 1, when it fits 32 bits.
__device__ __forceinline__ u32 recip_pow2(u64 p, int e) {
    u64 q = (~0ull) / p;                    // floor(2^64 / p)
    u64 rem = 0ull - q * p;                 // 2^64 - q p, in [1, p)
    for (int i = 64; i < e; ++i) {
        const u64 top = rem >> 63;
        rem <<= 1;
        q <<= 1;
        if (top || rem >= p) {
            rem -= p;
            q |= 1;
        }
    }
    return (u32)q;
}

__device__ __forceinline__ int bitlen64(u64 x) { return 64 - __clzll(x); }
__device__ __forceinline__ int bitlen32(u32 x) { return 32 - __clz(x); }
__device__ __forceinline__ u64 umin64(u64 a, u64 b) { return a < b ? a : b; }

struct Lazy96 {
    u64 p, one;
    u32 np0, np1, M, sh;      // 2^64 - p, reciprocal, shift s - 32
    u32 c0, c1, c2, c3;       // low words of one, one + p, p - one, 2p - one
};

struct Canon96 {
    u64 p, one;
    u32 p0, p1, M, sh;
    u32 c0, c2;               // low words of one and p - one
};

__device__ __forceinline__ bool lazy96_ok(u64 p, u32 kmax) {
    return p > (1ull << 33) && (p >> 63) == 0 && bitlen32(kmax) <= 28;
}
__device__ __forceinline__ bool canon96_ok(u64 p, u32 kmax) { return (p >> 63) != 0 && bitlen32(kmax) <= 28; }

__device__ __forceinline__ Lazy96 make_lazy96(const Prime& c, u32 kmax) {
    Lazy96 L;
    L.p = c.p;
    L.one = c.one;
    const u64 np = 0ull - c.p;
    L.np0 = (u32)np;
    L.np1 = (u32)(np >> 32);
    const int s = bitlen64(c.p) + 1 + bitlen32(kmax) - 31;
    L.sh = (u32)(s - 32);
    L.M = recip_pow2(c.p, 32 + s);
    const u64 nmo = c.p - c.one;
    L.c0 = (u32)c.one;
    L.c1 = (u32)(c.one + c.p);
    L.c2 = (u32)nmo;
    L.c3 = (u32)(nmo + c.p);
    return L;
}

__device__ __forceinline__ Canon96 make_canon96(const Prime& c, u32 kmax) {
    Canon96 C;
    C.p = c.p;
    C.one = c.one;
    C.p0 = (u32)c.p;
    C.p1 = (u32)(c.p >> 32);
    const int s = bitlen64(c.p) + bitlen32(kmax) - 31;
    C.sh = (u32)(s - 32);
    C.M = recip_pow2(c.p, 32 + s);
    C.c0 = (u32)c.one;
    C.c2 = (u32)(c.p - c.one);
    return C;
}

// z = bits [32 + sh, 64 + sh) of t = hi:lo, as shf.r.clamp takes them
__device__ __forceinline__ u32 top_bits(u64 lo, u64 hi, u32 sh) {
    const u64 t12 = (hi << 32) | (lo >> 32);
    return (u32)(t12 >> sh);
}

__device__ __forceinline__ u64 lazy96_step(u64 r, u32 k, const Lazy96& L) {
    const u64 lo = r * (u64)k, hi = __umul64hi(r, (u64)k);
    const u32 q = __umulhi(top_bits(lo, hi, L.sh), L.M);
    return lo + (u64)q * (((u64)L.np1 << 32) | L.np0);
}
__device__ __forceinline__ u64 lazy96_canon(u64 r, const Lazy96& L) { return r >= L.p ? r - L.p : r; }

__device__ __forceinline__ u64 canon96_step(u64 r, u32 k, const Canon96& C) {
    const u64 lo = r * (u64)k, hi = __umul64hi(r, (u64)k);
    const u32 q = __umulhi(top_bits(lo, hi, C.sh), C.M);
    const u64 qlo = (u64)q * C.p, qhi = __umul64hi((u64)q, C.p);
    const u64 rl = lo - qlo;
    const u64 r2 = hi - qhi - (lo < qlo ? 1ull : 0ull);
    return (r2 || rl >= C.p) ? rl - C.p : rl;
}

// Eight lazy96 steps on two residues (operands as lazy_walk8x2 plus shifts).
#define FS_L96_MUL(RL, RH, NP0, NP1, MM, SH, T, U, R, CC, T0, C, T1, T2, Z, Q)  \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                                        \
    "mov.b64 {" T0 ", " C "}, " T ";\n\t"                                        \
    "mad.lo.cc.u32 " T1 ", " RH ", kk, " C ";\n\t"                               \
    "madc.hi.u32 " T2 ", " RH ", kk, zr;\n\t"                                       \
    "shf.r.clamp.b32 " Z ", " T1 ", " T2 ", " SH ";\n\t"                         \
    "mul.hi.u32 " Q ", " Z ", " MM ";\n\t"                                       \
    "mad.lo.cc.u32 " RL ", " Q ", " NP0 ", " T0 ";\n\t"                          \
    "madc.hi.u32 " T1 ", " Q ", " NP0 ", " T1 ";\n\t"                            \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " T1 ";\n\t"
#define FS_L96_STEP2(J)                                                                        \
    "add.u32 kk, %5, " #J ";\n\t"                                                              \
    FS_LZ_TEST("%0", "%10", "%11", "%12", "%13")                                               \
    FS_LZ_TEST("%2", "%18", "%19", "%20", "%21")                                               \
    FS_L96_MUL("%0", "%1", "%6", "%7", "%8", "%9", "TA", "UA", "RA", "CA", "a0", "ac", "a1", "a2", "az", "aq") \
    FS_L96_MUL("%2", "%3", "%14", "%15", "%16", "%17", "TB", "UB", "RB", "CB", "b0", "bc", "b1", "b2", "bz", "bq")

__device__ __forceinline__ u32 lazy96_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Lazy96& A,
                                              const Lazy96& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, zr, a0, ac, a1, a2, az, aq, b0, bc, b1, b2, bz, bq;\n\t"
        ".reg .u64 TA, UA, RA, CA, TB, UB, RB, CB;\n\t"
        ".reg .pred P;\n\t"
        "mov.u32 zr, 0;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_L96_STEP2(0) FS_L96_STEP2(1) FS_L96_STEP2(2) FS_L96_STEP2(3)
        FS_L96_STEP2(4) FS_L96_STEP2(5) FS_L96_STEP2(6) FS_L96_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "r"(A.M), "r"(A.sh), "r"(A.c0), "r"(A.c1), "r"(A.c2), "r"(A.c3),
          "r"(B.np0), "r"(B.np1), "r"(B.M), "r"(B.sh), "r"(B.c0), "r"(B.c1), "r"(B.c2), "r"(B.c3));
    return flag;
}

// Eight canon96 steps on two residues; the +-1 test needs two compares
// (canonical residue) and the fold uses a 65-bit comparison.
#define FS_C96_TEST(RL, C0, C2)                        \
    "setp.eq.or.u32 P, " RL ", " C0 ", P;\n\t"         \
    "setp.eq.or.u32 P, " RL ", " C2 ", P;\n\t"
#define FS_C96_MUL(RL, RH, P0, P1, MM, SH, PP, T, U, A, B, CC, R64, T0, C, T1, T2, Z, Q, X0, X1, Y1, Y2, W2, G) \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                                        \
    "mov.b64 {" T0 ", " C "}, " T ";\n\t"                                        \
    "mad.lo.cc.u32 " T1 ", " RH ", kk, " C ";\n\t"                               \
    "madc.hi.u32 " T2 ", " RH ", kk, zr;\n\t"                                       \
    "shf.r.clamp.b32 " Z ", " T1 ", " T2 ", " SH ";\n\t"                         \
    "mul.hi.u32 " Q ", " Z ", " MM ";\n\t"                                       \
    "mul.wide.u32 " A ", " Q ", " P0 ";\n\t"                                     \
    "mov.b64 {" X0 ", " X1 "}, " A ";\n\t"                                       \
    "mad.lo.cc.u32 " Y1 ", " Q ", " P1 ", " X1 ";\n\t"                           \
    "madc.hi.u32 " Y2 ", " Q ", " P1 ", zr;\n\t"                                       \
    "sub.cc.u32 " RL ", " T0 ", " X0 ";\n\t"                                     \
    "subc.cc.u32 " RH ", " T1 ", " Y1 ";\n\t"                                    \
    "subc.u32 " W2 ", " T2 ", " Y2 ";\n\t"                                       \
    "mov.b64 " R64 ", {" RL ", " RH "};\n\t"                                     \
    "setp.ge.u64 " G ", " R64 ", " PP ";\n\t"                                    \
    "setp.ne.or.u32 " G ", " W2 ", 0, " G ";\n\t"                                \
    "@" G " sub.cc.u32 " RL ", " RL ", " P0 ";\n\t"                              \
    "@" G " subc.u32 " RH ", " RH ", " P1 ";\n\t"
#define FS_C96_STEP2(J)                                                                                 \
    "add.u32 kk, %5, " #J ";\n\t"                                                                       \
    FS_C96_TEST("%0", "%10", "%11")                                                                     \
    FS_C96_TEST("%2", "%16", "%17")                                                                     \
    FS_C96_MUL("%0", "%1", "%6", "%7", "%8", "%9", "PA", "TA", "UA", "AA", "BA", "CA", "RA", "a0", "ac", "a1", \
               "a2", "az", "aq", "ax0", "ax1", "ay1", "ay2", "aw", "GA")                                \
    FS_C96_MUL("%2", "%3", "%12", "%13", "%14", "%15", "PB", "TB", "UB", "AB", "BB", "CB", "RB", "b0", "bc", "b1", \
               "b2", "bz", "bq", "bx0", "bx1", "by1", "by2", "bw", "GB")

__device__ __forceinline__ u32 canon96_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Canon96& A,
                                               const Canon96& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, zr, a0, ac, a1, a2, az, aq, ax0, ax1, ay1, ay2, aw;\n\t"
        ".reg .u32 b0, bc, b1, b2, bz, bq, bx0, bx1, by1, by2, bw;\n\t"
        ".reg .u64 TA, UA, AA, BA, CA, RA, PA, TB, UB, AB, BB, CB, RB, PB;\n\t"
        ".reg .pred P, GA, GB;\n\t"
        "mov.u32 zr, 0;\n\t"
        "mov.b64 PA, {%6, %7};\n\t"
        "mov.b64 PB, {%12, %13};\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_C96_STEP2(0) FS_C96_STEP2(1) FS_C96_STEP2(2) FS_C96_STEP2(3)
        FS_C96_STEP2(4) FS_C96_STEP2(5) FS_C96_STEP2(6) FS_C96_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.p0), "r"(A.p1), "r"(A.M), "r"(A.sh), "r"(A.c0), "r"(A.c2),
          "r"(B.p0), "r"(B.p1), "r"(B.M), "r"(B.sh), "r"(B.c0), "r"(B.c2));
    return flag;
}

// ------------------------- iterate: lazy 64-bit steps, half-offset form --
//
// The lazy 64-bit step with the residue held as n! x mod p for
// x = (p - 1)/2 = -1/2 mod p instead of n! R.  Then n! = +1 gives x and
// n! = -1 gives -x = x + 1, two adjacent values.  The quotient estimate of
// the lazy step falls short of floor(t/p) by at most one, and only when
// t mod p < d p with d < 2^32/p + z/2^32 (z = t >> 32): the step leaves r in
// [0, (1 + d) p).  If r < (1 + e) p then z < (1 + e) p kmax / 2^32, so for
// p >= 2^36 and p kmax <= 2^62, d < 1/16 + (1 + e)/4, whose fixed point is
// e = 5/12: starting canonical, r stays below (17/12) p < x + p, never
// reaches x + p or x + 1 + p, and the exact hit test is r in {x, x + 1}: two
// compares of the low word per step instead of the four the [0, 2p) window
// needs.
struct Half64 {
    u64 p, x;                 // x = (p - 1) / 2
    u32 np0, np1, M;          // 2^64 - p (two words), floor(2^64 / p)
    u32 x0, x1;               // low words of x and x + 1
};

__device__ __forceinline__ bool half_ok(u64 p, u32 kmax) {
    return p >= (1ull << 36) && p <= ((1ull << 62) / (u64)(kmax ? kmax : 1));
}

__device__ __forceinline__ Half64 make_half(const Prime& c) {
    Half64 H;
    H.p = c.p;
    H.x = (c.p - 1) >> 1;
    const u64 np = 0ull - c.p;
    H.np0 = (u32)np;
    H.np1 = (u32)(np >> 32);
    H.M = (u32)((~0ull) / c.p);
    H.x0 = (u32)H.x;
    H.x1 = (u32)(H.x + 1);
    return H;
}

// n! R (canonical) -> n! x, and back: x R^-1 by one Montgomery product with
// x, and x^-1 = -2 by one with -2 R^2.
__device__ __forceinline__ u64 half_enter(u64 r, const Prime& c, u64 x) { return mont_mul(r, x, c.p, c.pinv); }
__device__ __forceinline__ u64 half_leave(u64 r, const Prime& c) {
    const u64 two_r2 = mod_add(c.r2, c.r2, c.p);
    return mont_mul(r, c.p - two_r2, c.p, c.pinv);
}

__device__ __forceinline__ u64 half_step(u64 r, u32 k, const Half64& H) {
    const u64 t = r * (u64)k;
    const u32 qe = __umulhi((u32)(t >> 32), H.M);
    return t + (u64)qe * (((u64)H.np1 << 32) | H.np0);
}
__device__ __forceinline__ u64 half_canon(u64 r, const Half64& H) { return r >= H.p ? r - H.p : r; }

#define FS_HF_TEST(RL, X0, X1)                         \
    "setp.eq.or.u32 P, " RL ", " X0 ", P;\n\t"         \
    "setp.eq.or.u32 P, " RL ", " X1 ", P;\n\t"
#define FS_HF_STEP2(J)                                              \
    "add.u32 kk, %5, " #J ";\n\t"                                   \
    FS_HF_TEST("%0", "%9", "%10")                                   \
    FS_HF_TEST("%2", "%14", "%15")                                  \
    FS_LZ_MUL("%0", "%1", "%6", "%7", "%8", "TA", "RA", "aL", "aH", "qA") \
    FS_LZ_MUL("%2", "%3", "%11", "%12", "%13", "TB", "RB", "bL", "bH", "qB")

// Eight half-offset steps on two residues; the flag as lazy_walk8x2's.
__device__ __forceinline__ u32 half_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Half64& A,
                                            const Half64& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, aL, aH, qA, bL, bH, qB;\n\t"
        ".reg .u64 TA, RA, TB, RB;\n\t"
        ".reg .pred P;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_HF_STEP2(0) FS_HF_STEP2(1) FS_HF_STEP2(2) FS_HF_STEP2(3)
        FS_HF_STEP2(4) FS_HF_STEP2(5) FS_HF_STEP2(6) FS_HF_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "r"(A.M), "r"(A.x0), "r"(A.x1), "r"(B.np0), "r"(B.np1), "r"(B.M),
          "r"(B.x0), "r"(B.x1));
    return flag;
}

// ------------- iterate: half-offset 64-bit steps, quotient on the FP32 pipe --
//
// The half-offset lazy 64-bit step takes its quotient estimate with an
// IMAD.HI on the integer multiply pipe, which bounds the walk.  This step
// takes it on the FP32 pipe instead and keeps the multiplies that form
// t = r k and r' = t + q (2^64 - p).  Let s = bitlen(f) - 4 for a floor
// f <= p with s >= 35, z = floor(t / 2^s) and m = floor(2^e / p) with
// e = bitlen(p) + 23 (so m has 24 bits and m 2^(s-e) is 2^s/p rounded down
// to 24 bits).  The estimate floor(z m 2^(s-e)) comes from two exact
// instructions:
//   1. z = (t's high word) >> (s - 32).  Read as a float, the bit pattern of
//      an integer z < 2^23 is the subnormal z 2^-149 (exponent field 0).
//   2. fma rounding down, by the normal float m 2^(s-e), gives
//      z m 2^(s-e-149).  That lies below 2^-126, on the subnormal grid, so
//      its bit pattern is the integer floor(z m 2^(s-e)).
// The two float operations have no .ftz, so subnormal inputs and results are
// kept.  (An earlier form built the normal float 2^-63 + z 2^-86 with a
// funnel shift and subtracted 2^-63 exactly; it gives the same estimate with
// one instruction more per step: 9 % slower on the walk block.)
// The estimate never exceeds t/p.  It falls short of it by less than
// 1 + 2^s/p + (t/p) 2^-23, which is below 1 + 1/8 + 1/16 when
// r < (19/16) p and 19 k_max <= 2^23.  So r stays below (19/16) p < x + p,
// and the exact test is r in {x, x + 1}, as in the half-offset lazy step.
// Validity over a launch (checked by the host, walk_for_range), with f the
// thread's least candidate: p >= 2^38, p k_max <= 2^62, 19 k_max <= 2^23,
// and 19 p_max k_max < 2^(bitlen(p_min) + 23), which keeps z < 2^23.
struct HalfF {
    u64 p, x;
    u32 np0, np1;             // 2^64 - p
    float g;                  // m 2^(s - e): 2^s/p rounded down to 24 bits
    u32 sh;                   // s - 32: the shift that takes z from t's high word
    u32 x0, x1;               // low words of x and x + 1
};

// f <= p: the floor that sets s (the least candidate of the thread, whose
// launch-wide validity the host has shown, or p itself).
__device__ __forceinline__ HalfF make_halff(const Prime& c, u64 f) {
    HalfF H;
    H.p = c.p;
    H.x = (c.p - 1) >> 1;
    const u64 np = 0ull - c.p;
    H.np0 = (u32)np;
    H.np1 = (u32)(np >> 32);
    const int bl = bitlen64(c.p), s = bitlen64(f) - 4, e = bl + 23;
    // m = floor(2^e / p) in [2^23, 2^24)
    const u32 m = e <= 64 ? (u32)(((~0ull) / c.p) >> (64 - e)) : recip_pow2(c.p, e);
    // m 2^(s - e) as a float: exponent field s - e + 150 (normal), mantissa m - 2^23
    H.g = __uint_as_float(((u32)(s - e + 149) << 23) + m);
    H.sh = (u32)(s - 32);
    H.x0 = (u32)H.x;
    H.x1 = (u32)(H.x + 1);
    return H;
}

// floor(z m 2^(s-e)) from t's high word, as the PTX block computes it.
__device__ __forceinline__ u32 halff_quot(u32 th, const HalfF& H) {
    u32 q;
    asm("{\n\t"
        ".reg .b32 z;\n\t"
        ".reg .f32 f;\n\t"
        "shr.u32 z, %1, %2;\n\t"
        "mov.b32 f, z;\n\t"
        "fma.rm.f32 f, f, %3, 0f00000000;\n\t"
        "mov.b32 %0, f;\n\t"
        "}"
        : "=r"(q)
        : "r"(th), "r"(H.sh), "f"(H.g));
    return q;
}

__device__ __forceinline__ u64 halff_step(u64 r, u32 k, const HalfF& H) {
    const u64 t = r * (u64)k;
    const u32 q = halff_quot((u32)(t >> 32), H);
    return t + (u64)q * (((u64)H.np1 << 32) | H.np0);
}
__device__ __forceinline__ u64 halff_canon(u64 r, const HalfF& H) { return r >= H.p ? r - H.p : r; }

#define FS_HFF_MUL(RL, RH, NP0, NP1, G, SH, T, TL, TH, Q, Z, F, KK)      \
    "mul.wide.u32 " T ", " RL ", " KK ";\n\t"                                \
    "mov.b64 {" TL ", " TH "}, " T ";\n\t"                                   \
    "mad.lo.u32 " TH ", " RH ", " KK ", " TH ";\n\t"                         \
    "shr.u32 " Z ", " TH ", " SH ";\n\t"                                    \
    "mov.b32 " F ", " Z ";\n\t"                                          \
    "fma.rm.f32 " F ", " F ", " G ", 0f00000000;\n\t"                   \
    "mov.b32 " Q ", " F ";\n\t"                                          \
    "mad.lo.cc.u32 " RL ", " Q ", " NP0 ", " TL ";\n\t"                  \
    "madc.hi.u32 " TH ", " Q ", " NP0 ", " TH ";\n\t"                    \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " TH ";\n\t"
// The multipliers k1 .. k1 + 7 come in as operands %18-%25: computed outside
// the asm, they are shared by the blocks of a thread's two pairs.
#define FS_HFF_STEP2(KK)                                                                 \
    FS_HF_TEST("%0", "%9", "%10")                                                        \
    FS_HF_TEST("%2", "%15", "%16")                                                       \
    FS_HFF_MUL("%0", "%1", "%6", "%7", "%8", "%11", "TA", "aL", "aH", "qA", "zA", "fA", KK)   \
    FS_HFF_MUL("%2", "%3", "%12", "%13", "%14", "%17", "TB", "bL", "bH", "qB", "zB", "fB", KK)

// Eight float-quotient half-offset steps on two residues; the flag as
// lazy_walk8x2's.
__device__ __forceinline__ u32 halff_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const HalfF& A,
                                             const HalfF& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 aL, aH, qA, zA, bL, bH, qB, zB;\n\t"
        ".reg .f32 fA, fB;\n\t"
        ".reg .u64 TA, TB;\n\t"
        ".reg .pred P;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_HFF_STEP2("%18") FS_HFF_STEP2("%19") FS_HFF_STEP2("%20") FS_HFF_STEP2("%21")
        FS_HFF_STEP2("%22") FS_HFF_STEP2("%23") FS_HFF_STEP2("%24") FS_HFF_STEP2("%25")
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "f"(A.g), "r"(A.x0), "r"(A.x1), "r"(A.sh),
          "r"(B.np0), "r"(B.np1), "f"(B.g), "r"(B.x0), "r"(B.x1), "r"(B.sh),
          "r"(k1), "r"(k1 + 1), "r"(k1 + 2), "r"(k1 + 3), "r"(k1 + 4), "r"(k1 + 5), "r"(k1 + 6), "r"(k1 + 7));
    return flag;
}

// ------- iterate: half-offset steps, float quotient with a k_max-aware window --
//
// The float quotient of halff_walk8x2 with the window chosen from the
// multipliers as well: for each candidate, T = ceil(23 p k_max / 16) bounds
// t = r k while r < (23/16) p, s = bitlen(T) - 24 keeps z = floor(t / 2^s)
// below 2^24, and g = m 2^(s-e) (m = floor(2^e / p), e = bitlen(p) + 23)
// turns z into the estimate q = floor(z g) with one round-down FMA on the
// subnormal grid (an integer below 2^24 read as a float is z 2^-149: exponent
// field 0 or 1, both with spacing 2^-149).  Then q <= t/p and t/p - q <
// 1 + 2^s/p + (t/p) 2^-23 < 1 + (46/16) k_max 2^-23, so for 46 k_max < 7 2^23
// the residue stays below (23/16) p < x + p from a canonical start, and the
// hit test is the half-offset one, r in {x, x + 1}.  Three forms:
//   HG    t < 2^64, s >= 32: z = (t's high word) >> (s - 32) (the
//         halff_walk8x2 block with this window);
//   HGL   t < 2^64, s <= 32: z = the funnel shift of t's two words by s;
//   HG96  p < 2^63, t up to 96 bits, s >= 32: z = the funnel shift of t's
//         upper two words by s - 32, r' = t + q (2^64 - p) modulo 2^64.
// The host picks one for a whole launch (walk_for_range) when every
// candidate's s falls on its side of 32.
constexpr u32 kHalfGMaxK = 1276526;   // 46 k_max < 7 2^23 with a margin for the rounding of T

__device__ __forceinline__ int halfg_window(u64 p, u32 kmax) {
    const unsigned __int128 T = ((unsigned __int128)23 * p * kmax + 15) / 16;
    const u64 th = (u64)(T >> 64), tl = (u64)T;
    return (th ? 128 - __clzll(th) : 64 - __clzll(tl)) - 24;
}

// form: 0 HG (sh = s - 32), 1 HGL (sh = s), 2 HG96 (sh = s - 32)
__device__ __forceinline__ HalfF make_halfg(const Prime& c, u32 kmax, int form) {
    HalfF H;
    H.p = c.p;
    H.x = (c.p - 1) >> 1;
    const u64 np = 0ull - c.p;
    H.np0 = (u32)np;
    H.np1 = (u32)(np >> 32);
    const int bl = bitlen64(c.p), e = bl + 23, s = halfg_window(c.p, kmax);
    const u32 m = e <= 64 ? (u32)(((~0ull) / c.p) >> (64 - e)) : recip_pow2(c.p, e);
    H.g = __uint_as_float(((u32)(s - e + 149) << 23) + m);
    H.sh = (u32)(form == 1 ? s : s - 32);
    H.x0 = (u32)H.x;
    H.x1 = (u32)(H.x + 1);
    return H;
}

// floor(z g) for a window z < 2^24.
__device__ __forceinline__ u32 halfg_quot(u32 z, const HalfF& H) {
    u32 q;
    asm("{\n\t"
        ".reg .f32 f;\n\t"
        "mov.b32 f, %1;\n\t"
        "fma.rm.f32 f, f, %2, 0f00000000;\n\t"
        "mov.b32 %0, f;\n\t"
        "}"
        : "=r"(q)
        : "r"(z), "f"(H.g));
    return q;
}

__device__ __forceinline__ u64 halfgl_step(u64 r, u32 k, const HalfF& H) {
    const u64 t = r * (u64)k;
    const u32 q = halfg_quot((u32)(t >> H.sh), H);
    return t + (u64)q * (((u64)H.np1 << 32) | H.np0);
}

__device__ __forceinline__ u64 halfg96_step(u64 r, u32 k, const HalfF& H) {
    const unsigned __int128 t = (unsigned __int128)r * k;
    const u32 q = halfg_quot((u32)(t >> (H.sh + 32)), H);
    return (u64)t + (u64)q * (((u64)H.np1 << 32) | H.np0);
}

#define FS_HGL_MUL(RL, RH, NP0, NP1, G, SH, T, TL, TH, Z, Q, F)      \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                          \
    "mov.b64 {" TL ", " TH "}, " T ";\n\t"                         \
    "mad.lo.u32 " TH ", " RH ", kk, " TH ";\n\t"                   \
    "shf.r.clamp.b32 " Z ", " TL ", " TH ", " SH ";\n\t"           \
    "mov.b32 " F ", " Z ";\n\t"                                    \
    "fma.rm.f32 " F ", " F ", " G ", 0f00000000;\n\t"              \
    "mov.b32 " Q ", " F ";\n\t"                                    \
    "mad.lo.cc.u32 " RL ", " Q ", " NP0 ", " TL ";\n\t"            \
    "madc.hi.u32 " TH ", " Q ", " NP0 ", " TH ";\n\t"              \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " TH ";\n\t"
#define FS_HGL_STEP2(J)                                                                  \
    "add.u32 kk, %5, " #J ";\n\t"                                                        \
    FS_HF_TEST("%0", "%10", "%11")                                                       \
    FS_HF_TEST("%2", "%16", "%17")                                                       \
    FS_HGL_MUL("%0", "%1", "%6", "%7", "%8", "%9", "TA", "aL", "aH", "az", "aq", "fa")   \
    FS_HGL_MUL("%2", "%3", "%12", "%13", "%14", "%15", "TB", "bL", "bH", "bz", "bq", "fb")

// Eight HGL steps on two residues; the flag as lazy_walk8x2's.
__device__ __forceinline__ u32 halfgl_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const HalfF& A,
                                              const HalfF& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, aL, aH, az, aq, bL, bH, bz, bq;\n\t"
        ".reg .f32 fa, fb;\n\t"
        ".reg .u64 TA, TB;\n\t"
        ".reg .pred P;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_HGL_STEP2(0) FS_HGL_STEP2(1) FS_HGL_STEP2(2) FS_HGL_STEP2(3)
        FS_HGL_STEP2(4) FS_HGL_STEP2(5) FS_HGL_STEP2(6) FS_HGL_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "f"(A.g), "r"(A.sh), "r"(A.x0), "r"(A.x1),
          "r"(B.np0), "r"(B.np1), "f"(B.g), "r"(B.sh), "r"(B.x0), "r"(B.x1));
    return flag;
}

// The 96-bit multiply of half96_walk8x2 (mad.wide with 64-bit addends) with
// the float quotient.
#define FS_HG96_MUL(RL, RH, NP0, NP1, G, SH, T, U, R, CC, T0, C, T1, T2, Z, Q, F)  \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                                        \
    "mov.b64 {" T0 ", " C "}, " T ";\n\t"                                        \
    "mov.b64 " CC ", {" C ", zr};\n\t"                                           \
    "mad.wide.u32 " U ", " RH ", kk, " CC ";\n\t"                                \
    "mov.b64 {" T1 ", " T2 "}, " U ";\n\t"                                       \
    "shf.r.clamp.b32 " Z ", " T1 ", " T2 ", " SH ";\n\t"                         \
    "mov.b32 " F ", " Z ";\n\t"                                                  \
    "fma.rm.f32 " F ", " F ", " G ", 0f00000000;\n\t"                            \
    "mov.b32 " Q ", " F ";\n\t"                                                  \
    "mov.b64 " T ", {" T0 ", " T1 "};\n\t"                                       \
    "mad.wide.u32 " R ", " Q ", " NP0 ", " T ";\n\t"                             \
    "mov.b64 {" RL ", " RH "}, " R ";\n\t"                                       \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " RH ";\n\t"
#define FS_HG96_STEP2(J)                                                                       \
    "add.u32 kk, %5, " #J ";\n\t"                                                              \
    FS_HF_TEST("%0", "%10", "%11")                                                             \
    FS_HF_TEST("%2", "%16", "%17")                                                             \
    FS_HG96_MUL("%0", "%1", "%6", "%7", "%8", "%9", "TA", "UA", "RA", "CA", "a0", "ac", "a1", "a2", "az", "aq", "fa") \
    FS_HG96_MUL("%2", "%3", "%12", "%13", "%14", "%15", "TB", "UB", "RB", "CB", "b0", "bc", "b1", "b2", "bz", "bq", "fb")

// Eight HG96 steps on two residues; the flag as lazy_walk8x2's.
__device__ __forceinline__ u32 halfg96_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const HalfF& A,
                                               const HalfF& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, zr, a0, ac, a1, a2, az, aq, b0, bc, b1, b2, bz, bq;\n\t"
        ".reg .f32 fa, fb;\n\t"
        ".reg .u64 TA, UA, RA, CA, TB, UB, RB, CB;\n\t"
        ".reg .pred P;\n\t"
        "mov.u32 zr, 0;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_HG96_STEP2(0) FS_HG96_STEP2(1) FS_HG96_STEP2(2) FS_HG96_STEP2(3)
        FS_HG96_STEP2(4) FS_HG96_STEP2(5) FS_HG96_STEP2(6) FS_HG96_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "f"(A.g), "r"(A.sh), "r"(A.x0), "r"(A.x1),
          "r"(B.np0), "r"(B.np1), "f"(B.g), "r"(B.sh), "r"(B.x0), "r"(B.x1));
    return flag;
}

// ------------------------- iterate: lazy 96-bit steps, half-offset form --
//
// The half-offset form for the lazy 96-bit step.  With the window z = t >> s
// taken one bit lower than the lazy 96-bit step takes it (s = bitlen(p) +
// bitlen(k_max) - 29), the quotient falls short by d < 2^s/p + z/2^32.  If
// r < (1 + e) p then z < (1 + e) 2^29, so for k_max < 2^26 d < 1/4 +
// (1 + e)/8, whose fixed point is e = 3/7: r stays below (10/7) p < x + p,
// and the exact test is r in {x, x + 1}.  Needs s >= 32 (bitlen(p) +
// bitlen(k_max) >= 61), which every p k_max above 2^60 meets.
struct Half96 {
    u64 p, x;
    u32 np0, np1, M, sh;      // 2^64 - p, floor(2^(32+s) / p), s - 32
    u32 x0, x1;               // low words of x and x + 1
};

__device__ __forceinline__ bool half96_ok(u64 p, u32 kmax) {
    return p > (1ull << 33) && (p >> 63) == 0 && kmax != 0 && bitlen32(kmax) <= 26 &&
           bitlen64(p) + bitlen32(kmax) >= 61;
}

__device__ __forceinline__ Half96 make_half96(const Prime& c, u32 kmax) {
    Half96 H;
    H.p = c.p;
    H.x = (c.p - 1) >> 1;
    const u64 np = 0ull - c.p;
    H.np0 = (u32)np;
    H.np1 = (u32)(np >> 32);
    const int s = bitlen64(c.p) + bitlen32(kmax) - 29;
    H.sh = (u32)(s - 32);
    H.M = recip_pow2(c.p, 32 + s);
    H.x0 = (u32)H.x;
    H.x1 = (u32)(H.x + 1);
    return H;
}

__device__ __forceinline__ u64 half96_step(u64 r, u32 k, const Half96& H) {
    const u64 lo = r * (u64)k, hi = __umul64hi(r, (u64)k);
    const u32 q = __umulhi(top_bits(lo, hi, H.sh), H.M);
    return lo + (u64)q * (((u64)H.np1 << 32) | H.np0);
}
__device__ __forceinline__ u64 half96_canon(u64 r, const Half96& H) { return r >= H.p ? r - H.p : r; }

// The lazy 96-bit multiply with mad.wide and 64-bit addends: for the
// half-offset 96-bit step this form measures 2 % faster than the carry-pair
// form that FS_L96_MUL uses.
#define FS_H96_MUL(RL, RH, NP0, NP1, MM, SH, T, U, R, CC, T0, C, T1, T2, Z, Q)  \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                                        \
    "mov.b64 {" T0 ", " C "}, " T ";\n\t"                                        \
    "mov.b64 " CC ", {" C ", zr};\n\t"                                           \
    "mad.wide.u32 " U ", " RH ", kk, " CC ";\n\t"                                \
    "mov.b64 {" T1 ", " T2 "}, " U ";\n\t"                                       \
    "shf.r.clamp.b32 " Z ", " T1 ", " T2 ", " SH ";\n\t"                         \
    "mul.hi.u32 " Q ", " Z ", " MM ";\n\t"                                       \
    "mov.b64 " T ", {" T0 ", " T1 "};\n\t"                                       \
    "mad.wide.u32 " R ", " Q ", " NP0 ", " T ";\n\t"                             \
    "mov.b64 {" RL ", " RH "}, " R ";\n\t"                                       \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " RH ";\n\t"
#define FS_H96_STEP2(J)                                                                        \
    "add.u32 kk, %5, " #J ";\n\t"                                                              \
    FS_HF_TEST("%0", "%10", "%11")                                                             \
    FS_HF_TEST("%2", "%16", "%17")                                                             \
    FS_H96_MUL("%0", "%1", "%6", "%7", "%8", "%9", "TA", "UA", "RA", "CA", "a0", "ac", "a1", "a2", "az", "aq") \
    FS_H96_MUL("%2", "%3", "%12", "%13", "%14", "%15", "TB", "UB", "RB", "CB", "b0", "bc", "b1", "b2", "bz", "bq")

__device__ __forceinline__ u32 half96_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Half96& A,
                                              const Half96& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, zr, a0, ac, a1, a2, az, aq, b0, bc, b1, b2, bz, bq;\n\t"
        ".reg .u64 TA, UA, RA, CA, TB, UB, RB, CB;\n\t"
        ".reg .pred P;\n\t"
        "mov.u32 zr, 0;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_H96_STEP2(0) FS_H96_STEP2(1) FS_H96_STEP2(2) FS_H96_STEP2(3)
        FS_H96_STEP2(4) FS_H96_STEP2(5) FS_H96_STEP2(6) FS_H96_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "r"(A.M), "r"(A.sh), "r"(A.x0), "r"(A.x1),
          "r"(B.np0), "r"(B.np1), "r"(B.M), "r"(B.sh), "r"(B.x0), "r"(B.x1));
    return flag;
}

// -------------------------- iterate: 32-bit steps, half-offset form (p < 2^31) --
//
// For p < 2^31 the residue fits one word: t = r k is a single 32 x 32-bit
// product, and r' = t - q p < 2^32 needs only the low word, one IMAD.  The
// quotient takes the 32-bit window z = t >> s, s = max(0, bitlen(p) +
// bitlen(k_max) - 29), M = floor(2^(32+s) / p): with r < (1 + e) p,
// z < (1 + e) 2^29 and d < 2^(kb-28) + (1 + e)/8 (no first term when s = 0),
// fixed point e = 3/7 for k_max < 2^26.  Half-offset form as above: hits are
// r in {x, x + 1}.  The high word of the residue stays zero.
struct Half32 {
    u64 p, x;
    u32 np, M, sh;            // 2^32 - p, floor(2^(32+s) / p), s
    u32 x0, x1;               // x and x + 1
};

__device__ __forceinline__ bool half32_ok(u64 p, u32 kmax) {
    return p > 2 && p < (1ull << 31) && kmax != 0 && bitlen32(kmax) <= 26;
}

__device__ __forceinline__ Half32 make_half32(const Prime& c, u32 kmax) {
    Half32 H;
    H.p = c.p;
    H.x = (c.p - 1) >> 1;
    H.np = (u32)(0ull - c.p);
    const int s0 = bitlen64(c.p) + bitlen32(kmax) - 29;
    const int s = s0 > 0 ? s0 : 0;
    H.sh = (u32)s;
    H.M = (u32)((1ull << (32 + s)) / c.p);
    H.x0 = (u32)H.x;
    H.x1 = (u32)(H.x + 1);
    return H;
}

__device__ __forceinline__ u64 half32_step(u64 r, u32 k, const Half32& H) {
    const u64 t = (u64)(u32)r * (u64)k;
    const u32 q = __umulhi((u32)(t >> H.sh), H.M);
    return (u64)(u32)((u32)t + q * H.np);
}
__device__ __forceinline__ u64 half32_canon(u64 r, const Half32& H) { return r >= H.p ? r - H.p : r; }

#define FS_H32_MUL(RL, NP, MM, SH, T, T0, T1, Z, Q)                 \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                          \
    "mov.b64 {" T0 ", " T1 "}, " T ";\n\t"                         \
    "shf.r.clamp.b32 " Z ", " T0 ", " T1 ", " SH ";\n\t"           \
    "mul.hi.u32 " Q ", " Z ", " MM ";\n\t"                         \
    "mad.lo.u32 " RL ", " Q ", " NP ", " T0 ";\n\t"
#define FS_H32_STEP2(J)                                             \
    "add.u32 kk, %5, " #J ";\n\t"                                   \
    FS_HF_TEST("%0", "%9", "%10")                                   \
    FS_HF_TEST("%2", "%14", "%15")                                  \
    FS_H32_MUL("%0", "%6", "%7", "%8", "TA", "a0", "a1", "az", "aq") \
    FS_H32_MUL("%2", "%11", "%12", "%13", "TB", "b0", "b1", "bz", "bq")

// Eight 32-bit half-offset steps on two residues (high words untouched, zero).
__device__ __forceinline__ u32 half32_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Half32& A,
                                              const Half32& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, a0, a1, az, aq, b0, b1, bz, bq;\n\t"
        ".reg .u64 TA, TB;\n\t"
        ".reg .pred P;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_H32_STEP2(0) FS_H32_STEP2(1) FS_H32_STEP2(2) FS_H32_STEP2(3)
        FS_H32_STEP2(4) FS_H32_STEP2(5) FS_H32_STEP2(6) FS_H32_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np), "r"(A.M), "r"(A.sh), "r"(A.x0), "r"(A.x1), "r"(B.np), "r"(B.M), "r"(B.sh),
          "r"(B.x0), "r"(B.x1));
    return flag;
}

// ----------- iterate: lazy 64-bit steps, shifted window, half-offset form --
//
// 2^31 <= p < 2^36, where the half-offset 64-bit step's window z = t >> 32 is
// too coarse (2^32/p up to 2) and the 32-bit step's residue does not fit a
// word: the quotient window is z = t >> s, s = max(0, bitlen(p) +
// bitlen(k_max) - 29) <= 32, M = floor(2^(32+s) / p), with the same bound as
// the 96-bit half-offset step (window fixed point 10/7 p) for k_max < 2^25.
// The step is the half-offset 64-bit step with one funnel shift more.
__device__ __forceinline__ bool halfmid_ok(u64 p, u32 kmax) {
    return p >= (1ull << 31) && p < (1ull << 36) && kmax != 0 && bitlen32(kmax) <= 25;
}

__device__ __forceinline__ Half96 make_halfmid(const Prime& c, u32 kmax) {
    Half96 H;
    H.p = c.p;
    H.x = (c.p - 1) >> 1;
    const u64 np = 0ull - c.p;
    H.np0 = (u32)np;
    H.np1 = (u32)(np >> 32);
    const int s0 = bitlen64(c.p) + bitlen32(kmax) - 29;
    const int s = s0 > 0 ? s0 : 0;
    H.sh = (u32)s;
    // s reaches 32 (p >= 2^35 with k_max >= 2^24), where 1 << (32 + s) would
    // overflow: floor((2^(32+s) - 1) / p) is the same quotient for odd p > 1
    H.M = (u32)((~0ull >> (32 - s)) / c.p);
    H.x0 = (u32)H.x;
    H.x1 = (u32)(H.x + 1);
    return H;
}

__device__ __forceinline__ u64 halfmid_step(u64 r, u32 k, const Half96& H) {
    const u64 t = r * (u64)k;
    const u32 q = __umulhi((u32)(t >> H.sh), H.M);
    return t + (u64)q * (((u64)H.np1 << 32) | H.np0);
}

#define FS_HM_MUL(RL, RH, NP0, NP1, MM, SH, T, R, TL, TH, Z, Q)   \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                          \
    "mov.b64 {" TL ", " TH "}, " T ";\n\t"                         \
    "mad.lo.u32 " TH ", " RH ", kk, " TH ";\n\t"                   \
    "shf.r.clamp.b32 " Z ", " TL ", " TH ", " SH ";\n\t"           \
    "mul.hi.u32 " Q ", " Z ", " MM ";\n\t"                         \
    "mad.lo.cc.u32 " RL ", " Q ", " NP0 ", " TL ";\n\t"          \
    "madc.hi.u32 " TH ", " Q ", " NP0 ", " TH ";\n\t"            \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " TH ";\n\t"
#define FS_HM_STEP2(J)                                                                   \
    "add.u32 kk, %5, " #J ";\n\t"                                                        \
    FS_HF_TEST("%0", "%10", "%11")                                                       \
    FS_HF_TEST("%2", "%16", "%17")                                                       \
    FS_HM_MUL("%0", "%1", "%6", "%7", "%8", "%9", "TA", "RA", "aL", "aH", "az", "aq")     \
    FS_HM_MUL("%2", "%3", "%12", "%13", "%14", "%15", "TB", "RB", "bL", "bH", "bz", "bq")

__device__ __forceinline__ u32 halfmid_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Half96& A,
                                               const Half96& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, aL, aH, az, aq, bL, bH, bz, bq;\n\t"
        ".reg .u64 TA, RA, TB, RB;\n\t"
        ".reg .pred P;\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_HM_STEP2(0) FS_HM_STEP2(1) FS_HM_STEP2(2) FS_HM_STEP2(3)
        FS_HM_STEP2(4) FS_HM_STEP2(5) FS_HM_STEP2(6) FS_HM_STEP2(7)
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.np0), "r"(A.np1), "r"(A.M), "r"(A.sh), "r"(A.x0), "r"(A.x1),
          "r"(B.np0), "r"(B.np1), "r"(B.M), "r"(B.sh), "r"(B.x0), "r"(B.x1));
    return flag;
}

// ------------------- iterate: 96-bit steps for p >= 2^63, half-offset form --
//
// For p >= 2^63 a residue of the lazy window needs 65 bits.  Inside one
// eight-step PTX block the 65th bit is kept in a register (t gains W k 2^64
// from it, one mad.lo) and the window fold of the canonical step is skipped;
// the residue is folded once, at the end of the block, so every residue
// that leaves the block is canonical.  With the window z = t >> s, s =
// 64 + bitlen(k_max) - 29, the lazy residue stays below (10/7) p for k_max <
// 2^26 (the bound of the other 96-bit half-offset step), and in half-offset
// form (x = (p - 1)/2) a hit is r = x or x + 1 with the 65th bit clear.
struct Canon96H {
    u64 p, x;
    u32 p0, p1, M, sh;        // p (two words), floor(2^(32+s) / p), s - 32
    u32 x0, x1;               // low words of x and x + 1
};

__device__ __forceinline__ bool canon96h_ok(u64 p, u32 kmax) {
    return (p >> 63) != 0 && kmax != 0 && bitlen32(kmax) <= 26;
}

__device__ __forceinline__ Canon96H make_canon96h(const Prime& c, u32 kmax) {
    Canon96H C;
    C.p = c.p;
    C.x = (c.p - 1) >> 1;
    C.p0 = (u32)c.p;
    C.p1 = (u32)(c.p >> 32);
    const int s = 64 + bitlen32(kmax) - 29;
    C.sh = (u32)(s - 32);
    C.M = recip_pow2(c.p, 32 + s);
    C.x0 = (u32)C.x;
    C.x1 = (u32)(C.x + 1);
    return C;
}

// One step with the fold (canonical in and out): the replay and tail steps.
__device__ __forceinline__ u64 canon96h_step(u64 r, u32 k, const Canon96H& C) {
    const u64 lo = r * (u64)k, hi = __umul64hi(r, (u64)k);
    const u32 q = __umulhi(top_bits(lo, hi, C.sh), C.M);
    const u64 qlo = (u64)q * C.p, qhi = __umul64hi((u64)q, C.p);
    const u64 rl = lo - qlo;
    const u64 r2 = hi - qhi - (lo < qlo ? 1ull : 0ull);
    return (r2 || rl >= C.p) ? rl - C.p : rl;
}

#define FS_C96H_MUL(RL, RH, W, P0, P1, MM, SH, T, U, A, B, CC, T0, C, T1, T2, Z, Q, X0, X1, Y1, Y2) \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                                        \
    "mov.b64 {" T0 ", " C "}, " T ";\n\t"                                        \
    "mov.b64 " CC ", {" C ", zr};\n\t"                                           \
    "mad.wide.u32 " U ", " RH ", kk, " CC ";\n\t"                                \
    "mov.b64 {" T1 ", " T2 "}, " U ";\n\t"                                       \
    "mad.lo.u32 " T2 ", " W ", kk, " T2 ";\n\t"                                  \
    "shf.r.clamp.b32 " Z ", " T1 ", " T2 ", " SH ";\n\t"                         \
    "mul.hi.u32 " Q ", " Z ", " MM ";\n\t"                                       \
    "mul.wide.u32 " A ", " Q ", " P0 ";\n\t"                                     \
    "mov.b64 {" X0 ", " X1 "}, " A ";\n\t"                                       \
    "mov.b64 " CC ", {" X1 ", zr};\n\t"                                          \
    "mad.wide.u32 " B ", " Q ", " P1 ", " CC ";\n\t"                             \
    "mov.b64 {" Y1 ", " Y2 "}, " B ";\n\t"                                       \
    "sub.cc.u32 " RL ", " T0 ", " X0 ";\n\t"                                     \
    "subc.cc.u32 " RH ", " T1 ", " Y1 ";\n\t"                                    \
    "subc.u32 " W ", " T2 ", " Y2 ";\n\t"
#define FS_C96H_STEP2(J)                                                                                  \
    "add.u32 kk, %5, " #J ";\n\t"                                                                         \
    FS_HF_TEST("%0", "%10", "%11")                                                                        \
    FS_HF_TEST("%2", "%16", "%17")                                                                        \
    FS_C96H_MUL("%0", "%1", "aw", "%6", "%7", "%8", "%9", "TA", "UA", "AA", "BA", "CA", "a0", "ac", "a1", "a2", \
                "az", "aq", "ax0", "ax1", "ay1", "ay2")                                                   \
    FS_C96H_MUL("%2", "%3", "bw", "%12", "%13", "%14", "%15", "TB", "UB", "AB", "BB", "CB", "b0", "bc", "b1",   \
                "b2", "bz", "bq", "bx0", "bx1", "by1", "by2")
// fold a 65-bit residue below 2p back into [0, p)
#define FS_C96H_FOLD(RL, RH, W, R64, PP, P0, P1, G)          \
    "mov.b64 " R64 ", {" RL ", " RH "};\n\t"                  \
    "setp.ge.u64 " G ", " R64 ", " PP ";\n\t"                 \
    "setp.ne.or.u32 " G ", " W ", 0, " G ";\n\t"              \
    "@" G " sub.cc.u32 " RL ", " RL ", " P0 ";\n\t"           \
    "@" G " subc.u32 " RH ", " RH ", " P1 ";\n\t"

__device__ __forceinline__ u32 canon96h_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Canon96H& A,
                                                const Canon96H& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, zr, a0, ac, a1, a2, az, aq, ax0, ax1, ay1, ay2, aw;\n\t"
        ".reg .u32 b0, bc, b1, b2, bz, bq, bx0, bx1, by1, by2, bw;\n\t"
        ".reg .u64 TA, UA, AA, BA, CA, RA, PA, TB, UB, AB, BB, CB, RB, PB;\n\t"
        ".reg .pred P, GA, GB;\n\t"
        "mov.u32 zr, 0;\n\t"
        "mov.u32 aw, 0;\n\t"
        "mov.u32 bw, 0;\n\t"
        "mov.b64 PA, {%6, %7};\n\t"
        "mov.b64 PB, {%12, %13};\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_C96H_STEP2(0) FS_C96H_STEP2(1) FS_C96H_STEP2(2) FS_C96H_STEP2(3)
        FS_C96H_STEP2(4) FS_C96H_STEP2(5) FS_C96H_STEP2(6) FS_C96H_STEP2(7)
        FS_C96H_FOLD("%0", "%1", "aw", "RA", "PA", "%6", "%7", "GA")
        FS_C96H_FOLD("%2", "%3", "bw", "RB", "PB", "%12", "%13", "GB")
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.p0), "r"(A.p1), "r"(A.M), "r"(A.sh), "r"(A.x0), "r"(A.x1),
          "r"(B.p0), "r"(B.p1), "r"(B.M), "r"(B.sh), "r"(B.x0), "r"(B.x1));
    return flag;
}

// ----- iterate: 96-bit steps for p >= 2^63, half-offset form, float quotient --
//
// canon96h_walk8x2 with its quotient taken as in make_halfg instead of by
// IMAD.HI: for each candidate, T = ceil(23 p k_max / 16) and the window
// shift s = bitlen(T) - 24 (40 to 64 for p >= 2^63), z = floor(t / 2^s) <
// 2^24 read as the float z 2^-149, and q = floor(z g) from one round-down FMA
// by g = m 2^(s-e), m = floor(2^e / p), e = bitlen(p) + 23 = 87.  The estimate
// never exceeds t/p and falls short of it by less than 1 + (46/16) k_max
// 2^-23, so for 46 k_max < 7 2^23 a residue below (23/16) p stays below it:
// 65 bits inside the block (the 65th in a register, as in canon96h_walk8x2),
// folded to [0, p) at the end of the block.  The hit test is the half-offset
// one on canonical residues, r in {x, x + 1}; (23/16) p < x + p keeps the
// lifted values out of reach.
struct Canon96G {
    u64 p, x;
    u32 p0, p1;               // p (two words)
    float g;                  // m 2^(s - e)
    u32 sh;                   // s - 32
    u32 x0, x1;               // low words of x and x + 1
};

__device__ __forceinline__ bool canon96g_ok(u64 p, u32 kmax) {
    return (p >> 63) != 0 && kmax != 0 && kmax <= kHalfGMaxK;
}

__device__ __forceinline__ Canon96G make_canon96g(const Prime& c, u32 kmax) {
    Canon96G C;
    C.p = c.p;
    C.x = (c.p - 1) >> 1;
    C.p0 = (u32)c.p;
    C.p1 = (u32)(c.p >> 32);
    const int e = 64 + 23, s = halfg_window(c.p, kmax);
    C.g = __uint_as_float(((u32)(s - e + 149) << 23) + recip_pow2(c.p, e));
    C.sh = (u32)(s - 32);
    C.x0 = (u32)C.x;
    C.x1 = (u32)(C.x + 1);
    return C;
}

// floor(z g) for a window z < 2^24 (the subnormal construction of halfg_quot).
__device__ __forceinline__ u32 fquot(u32 z, float g) {
    u32 q;
    asm("{\n\t"
        ".reg .f32 f;\n\t"
        "mov.b32 f, %1;\n\t"
        "fma.rm.f32 f, f, %2, 0f00000000;\n\t"
        "mov.b32 %0, f;\n\t"
        "}"
        : "=r"(q)
        : "r"(z), "f"(g));
    return q;
}

// One step with the fold (canonical in and out): the replay and tail steps.
__device__ __forceinline__ u64 canon96g_step(u64 r, u32 k, const Canon96G& C) {
    const u64 lo = r * (u64)k, hi = __umul64hi(r, (u64)k);
    const u32 q = fquot(top_bits(lo, hi, C.sh), C.g);
    const u64 qlo = (u64)q * C.p, qhi = __umul64hi((u64)q, C.p);
    const u64 rl = lo - qlo;
    const u64 r2 = hi - qhi - (lo < qlo ? 1ull : 0ull);
    return (r2 || rl >= C.p) ? rl - C.p : rl;
}

#define FS_C96G_MUL(RL, RH, W, P0, P1, G, SH, T, U, A, B, CC, T0, C, T1, T2, Z, Q, F, X0, X1, Y1, Y2) \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                                        \
    "mov.b64 {" T0 ", " C "}, " T ";\n\t"                                        \
    "mov.b64 " CC ", {" C ", zr};\n\t"                                           \
    "mad.wide.u32 " U ", " RH ", kk, " CC ";\n\t"                                \
    "mov.b64 {" T1 ", " T2 "}, " U ";\n\t"                                       \
    "mad.lo.u32 " T2 ", " W ", kk, " T2 ";\n\t"                                  \
    "shf.r.clamp.b32 " Z ", " T1 ", " T2 ", " SH ";\n\t"                         \
    "mov.b32 " F ", " Z ";\n\t"                                                  \
    "fma.rm.f32 " F ", " F ", " G ", 0f00000000;\n\t"                            \
    "mov.b32 " Q ", " F ";\n\t"                                                  \
    "mul.wide.u32 " A ", " Q ", " P0 ";\n\t"                                     \
    "mov.b64 {" X0 ", " X1 "}, " A ";\n\t"                                       \
    "mov.b64 " CC ", {" X1 ", zr};\n\t"                                          \
    "mad.wide.u32 " B ", " Q ", " P1 ", " CC ";\n\t"                             \
    "mov.b64 {" Y1 ", " Y2 "}, " B ";\n\t"                                       \
    "sub.cc.u32 " RL ", " T0 ", " X0 ";\n\t"                                     \
    "subc.cc.u32 " RH ", " T1 ", " Y1 ";\n\t"                                    \
    "subc.u32 " W ", " T2 ", " Y2 ";\n\t"
#define FS_C96G_STEP2(J)                                                                                  \
    "add.u32 kk, %5, " #J ";\n\t"                                                                         \
    FS_HF_TEST("%0", "%10", "%11")                                                                        \
    FS_HF_TEST("%2", "%16", "%17")                                                                        \
    FS_C96G_MUL("%0", "%1", "aw", "%6", "%7", "%8", "%9", "TA", "UA", "AA", "BA", "CA", "a0", "ac", "a1", "a2", \
                "az", "aq", "af", "ax0", "ax1", "ay1", "ay2")                                             \
    FS_C96G_MUL("%2", "%3", "bw", "%12", "%13", "%14", "%15", "TB", "UB", "AB", "BB", "CB", "b0", "bc", "b1",   \
                "b2", "bz", "bq", "bf", "bx0", "bx1", "by1", "by2")

__device__ __forceinline__ u32 canon96g_walk8x2(u32& al, u32& ah, u32& bl, u32& bh, u32 k1, const Canon96G& A,
                                                const Canon96G& B) {
    u32 flag;
    asm("{\n\t"
        ".reg .u32 kk, zr, a0, ac, a1, a2, az, aq, ax0, ax1, ay1, ay2, aw;\n\t"
        ".reg .u32 b0, bc, b1, b2, bz, bq, bx0, bx1, by1, by2, bw;\n\t"
        ".reg .f32 af, bf;\n\t"
        ".reg .u64 TA, UA, AA, BA, CA, RA, PA, TB, UB, AB, BB, CB, RB, PB;\n\t"
        ".reg .pred P, GA, GB;\n\t"
        "mov.u32 zr, 0;\n\t"
        "mov.u32 aw, 0;\n\t"
        "mov.u32 bw, 0;\n\t"
        "mov.b64 PA, {%6, %7};\n\t"
        "mov.b64 PB, {%12, %13};\n\t"
        "setp.ne.u32 P, %5, %5;\n\t"
        FS_C96G_STEP2(0) FS_C96G_STEP2(1) FS_C96G_STEP2(2) FS_C96G_STEP2(3)
        FS_C96G_STEP2(4) FS_C96G_STEP2(5) FS_C96G_STEP2(6) FS_C96G_STEP2(7)
        FS_C96H_FOLD("%0", "%1", "aw", "RA", "PA", "%6", "%7", "GA")
        FS_C96H_FOLD("%2", "%3", "bw", "RB", "PB", "%12", "%13", "GB")
        "selp.u32 %4, 1, 0, P;\n\t"
        "}"
        : "+r"(al), "+r"(ah), "+r"(bl), "+r"(bh), "=r"(flag)
        : "r"(k1), "r"(A.p0), "r"(A.p1), "f"(A.g), "r"(A.sh), "r"(A.x0), "r"(A.x1),
          "r"(B.p0), "r"(B.p1), "f"(B.g), "r"(B.sh), "r"(B.x0), "r"(B.x1));
    return flag;
}

}  // namespace fs
