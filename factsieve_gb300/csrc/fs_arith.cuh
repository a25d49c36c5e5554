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
    u64 lo = a * b;
    u64 hi = mulhi64(a, b);
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
#define FS_LZ_MUL(RL, RH, NP0, NP1, MM, T, R, TL, TH, Q)          \
    "mul.wide.u32 " T ", " RL ", kk;\n\t"                          \
    "mov.b64 {" TL ", " TH "}, " T ";\n\t"                         \
    "mad.lo.u32 " TH ", " RH ", kk, " TH ";\n\t"                   \
    "mul.hi.u32 " Q ", " TH ", " MM ";\n\t"                        \
    "mov.b64 " T ", {" TL ", " TH "};\n\t"                         \
    "mad.wide.u32 " R ", " Q ", " NP0 ", " T ";\n\t"               \
    "mov.b64 {" RL ", " RH "}, " R ";\n\t"                         \
    "mad.lo.u32 " RH ", " Q ", " NP1 ", " RH ";\n\t"
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

}  // namespace fs
