// fs_arith.cuh -- exact 64-bit modular arithmetic for the FactSieve kernels.
//
// Residues live in Montgomery form with R = 2^64, the representation the
// reference's kernels use and checksum (kernels/iterate.cl:36-49): a value x
// is held as x*R mod p, always fully reduced into [0, p).  Three products
// are used:
//
//   mont_mul(a, b)     a*b/R mod p for a < p, b < 2^64.  Setup and the PRP test.
//   mul_small_t64(s,k) s*k mod p for a 32-bit k by a Barrett step, valid when
//                      p > 2^33 and p*k < 2^64.  The iterate hot loop: the
//                      multiplier k = n+1 is a plain integer, so multiplying a
//                      Montgomery-form residue by it keeps the form and needs
//                      no Montgomery image of n at all.
//   mont_mul with kR   generic iterate step for every other (p, n) (the
//                      reference's own step: multiply by the Montgomery image
//                      of n+1, which advances by R each step).
//
// Every routine returns the canonical residue, so any mix of them yields the
// same bits as the reference.
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

// ------------------------------------------------- iterate: Barrett step --

// Constants of the 32-bit-multiplier Barrett step for p in (2^33, 2^64/kmax).
//   mu = floor(2^96 / p)  (< 2^63),  np = 2^64 - p.
struct Barrett {
    u64 mu, np;
};

// floor(2^96 / p) for odd p > 2^33: A = floor((2^64-1)/p) = floor(2^64/p),
// rem = 2^64 - A p in [1, p), then 32 steps of binary long division of
// rem * 2^32 by p supply the low 32 quotient bits.
__device__ __forceinline__ Barrett make_barrett(u64 p) {
    Barrett b;
    u64 A = (~0ull) / p;
    u64 rem = 0ull - A * p;                // 2^64 - A p (mod 2^64), in [1, p)
    u32 lowq = 0;
    for (int i = 0; i < 32; ++i) {
        u64 top = rem >> 63;
        rem <<= 1;
        lowq <<= 1;
        if (top || rem >= p) {
            rem -= p;
            lowq |= 1;
        }
    }
    b.mu = (A << 32) | lowq;
    b.np = 0ull - p;
    return b;
}

// s*k mod p for s < p, k < 2^32, p > 2^33 and p*k < 2^64 (so t = s*k fits a
// u64).  z = floor(t/2^32); qe = floor(z*mu/2^64) is floor(t/p) or one less
// (the truncations cost < 2^32/p + 2^-32 < 1), so r = t - qe*p is in [0, 2p)
// and one conditional subtraction makes it canonical.
__device__ __forceinline__ u64 mul_small_t64(u64 s, u32 k, u64 p, const Barrett& br) {
    u64 t = s * (u64)k;
    u32 z = (u32)(t >> 32);
    u64 hz = __umulhi(z, (u32)br.mu);                      // floor(z*mu_lo / 2^32)
    u64 qe = ((u64)z * (br.mu >> 32) + hz) >> 32;          // floor(z*mu / 2^64)
    u64 r = t + qe * br.np;                                // t - qe*p (mod 2^64)
    return r >= p ? r - p : r;
}

}  // namespace fs
