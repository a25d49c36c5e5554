/*
 * oracle.c -- CPU restatement of the FactSieve search path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference legs may load it; the shipped library and CLI never
 * link it.
 *
 * It restates, step by step and in plain C with OpenMP over candidate primes,
 * what the reference (mfl0p/FactSieve v1.6) computes:
 *
 *   candidate generation   kernels/getsegprimes.cl:170-239 (wheel, 7..113 masks,
 *                          strong_prp_two at :79-108), cl_sieve.cpp:360-419
 *                          (findWheelOffset)
 *   power table            cl_sieve.cpp:773-838 (getPower + compression)
 *   starting residue       kernels/setup.cl:49-103
 *   residue iteration      kernels/iterate.cl:54-80
 *   checksum / validation  kernels/check.cl:50-109
 *   host post-processing   cl_sieve.cpp:439-554 (sort, CPU verify, 2-PRP filter,
 *                          checksum += n + c), verifyprime.c:105-173
 *
 * Arithmetic: 64-bit Montgomery with R = 2^64 exactly as the reference
 * (iterate.cl:36-49); the 128-bit products use unsigned __int128.
 *
 * Pinning: the end-to-end entry oracle_run() reproduces the reference's own
 * self-test goldens (cl_sieve.cpp:1283-1364); see tests/test_oracle.py.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------- */
/* Montgomery arithmetic, R = 2^64 (iterate.cl:19-49, verifyprime.c:18-55)   */
/* ------------------------------------------------------------------------- */

/* p^-1 mod 2^64 by Newton iteration until it stops changing
 * (getsegprimes.cl:73-77). */
uint64_t oracle_invert(uint64_t p)
{
    uint64_t x = 1, last = 0;
    while (x != last) {
        last = x;
        x = x * (2 - p * x);
    }
    return x;
}

/* (a*b - m*p) / 2^64 with m = (a*b mod 2^64) * p^-1, folded into [0, p)
 * (iterate.cl:36-42).  Requires a*b < p*2^64. */
uint64_t oracle_mmul(uint64_t a, uint64_t b, uint64_t p, uint64_t q)
{
    u128 ab = (u128)a * b;
    uint64_t lo = (uint64_t)ab, hi = (uint64_t)(ab >> 64);
    uint64_t m = lo * q;
    uint64_t mp = (uint64_t)(((u128)m * p) >> 64);
    uint64_t r = hi - mp;
    return hi < mp ? r + p : r;
}

/* a + b mod p for a, b < p (iterate.cl:44-49). */
uint64_t oracle_madd(uint64_t a, uint64_t b, uint64_t p)
{
    uint64_t sub = (a >= p - b) ? p : 0;
    return a + b - sub;
}

/* Per-prime constants of the reference's 64-byte record
 * (getsegprimes.cl:214-228): q, r2 = R^2 mod p, one = R mod p, two, nmo. */
typedef struct {
    uint64_t p, q, r2, one, two, nmo;
} oconst;

static oconst make_const(uint64_t p)
{
    oconst c;
    c.p = p;
    c.q = oracle_invert(p);
    c.one = (0 - p) % p;             /* 2^64 mod p */
    c.nmo = p - c.one;
    c.two = oracle_madd(c.one, c.one, p);
    uint64_t r = oracle_madd(c.two, c.two, p);   /* 4R */
    for (int i = 0; i < 5; ++i)                   /* (4R)^(2^5) / R^31 = 2^64 R */
        r = oracle_mmul(r, r, p, c.q);
    c.r2 = r;
    return c;
}

/* Base-2 strong probable-prime test with a left-to-right ladder whose
 * doublings are modular additions (getsegprimes.cl:79-108). */
static int sprp2(const oconst *c)
{
    const uint64_t n = c->p;
    int t = __builtin_ctzll(n - 1);
    uint64_t d = n >> t;                   /* (n-1)/2^t, top bits of n */
    /* d == 1 only for n = 2^t + 1.  The reference shifts by 64 there, which
     * OpenCL masks to a shift by 0 (a 2^(2^64+1) ladder); for every such n
     * below 2^64 with no factor <= 113 (t = 8, 16, 32, 40, 48, 56) both
     * readings give the same verdict, so the plain ladder is used. */
    uint64_t bit = d > 1 ? 0x8000000000000000ull >> (__builtin_clzll(d) + 1) : 0;
    uint64_t a = c->two;
    for (; bit; bit >>= 1) {
        a = oracle_mmul(a, a, n, c->q);
        if (d & bit)
            a = oracle_madd(a, a, n);
    }
    if (a == c->one || a == c->nmo)
        return 1;
    for (int s = 1; s < t; ++s) {
        a = oracle_mmul(a, a, n, c->q);
        if (a == c->nmo)
            return 1;
    }
    return 0;
}

int oracle_sprp2(uint64_t n)
{
    if (n < 3 || !(n & 1))
        return 0;
    oconst c = make_const(n);
    return sprp2(&c);
}

/* ------------------------------------------------------------------------- */
/* Candidate generation (getsegprimes.cl, cl_sieve.cpp:360-419)              */
/* ------------------------------------------------------------------------- */

/* Gaps of the mod-30 wheel in units of 2, repeated so an index never wraps
 * inside one 60-integer block (getsegprimes.cl:112). */
static const int wheel_half_gap[24] = {2, 1, 2, 1, 2, 3, 1, 3, 2, 1, 2, 1,
                                       2, 3, 1, 3, 2, 1, 2, 1, 2, 3, 1, 3};

static const uint32_t small_q[27] = {7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59,
                                     61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};

/* Mask for an odd block start P with P % q == r: bit i set iff q | P + 2i.
 * This is the content of the reference's constant tables p7..p113
 * (getsegprimes.cl:116-168), generated instead of spelled out. */
uint32_t oracle_small_mask(uint32_t q, uint32_t r)
{
    uint32_t m = 0;
    for (uint32_t i = 0; i < 32; ++i)
        if ((r + 2 * i) % q == 0)
            m |= 1u << i;
    return m;
}

static uint32_t mask_tab[27][113];
static int mask_ready = 0;

static void build_masks(void)
{
    if (mask_ready)
        return;
#pragma omp critical(oracle_masks)
    {
        if (!mask_ready) {
            for (int j = 0; j < 27; ++j)
                for (uint32_t r = 0; r < small_q[j]; ++r)
                    mask_tab[j][r] = oracle_small_mask(small_q[j], r);
            __sync_synchronize();
            mask_ready = 1;
        }
    }
}

/* Smallest N >= start with gcd(N, 30) = 1 and its index in the gap table
 * (cl_sieve.cpp:360-419).  The reference walks a mod-6 wheel forward to N,
 * then further forward to the next multiple of 5 to anchor the mod-30 phase,
 * then back to N; the result is the same as this direct search. */
void oracle_find_wheel_offset(uint64_t *start, int32_t *index)
{
    static const int gap[8] = {4, 2, 4, 2, 4, 6, 2, 6};
    /* residues mod 30 coprime to 30, in wheel order starting after 1:
     * gap[i] leads from res[i] to res[i+1]; res = 7,11,13,17,19,23,29,1 */
    static const int res[8] = {7, 11, 13, 17, 19, 23, 29, 1};
    uint64_t n = *start;
    while (n % 2 == 0 || n % 3 == 0 || n % 5 == 0)
        ++n;
    int r = (int)(n % 30), idx = -1;
    for (int i = 0; i < 8; ++i)
        if (res[i] == r)
            idx = i;
    (void)gap;
    *start = n;
    *index = idx;
}

/* Reference getsegprimes semantics over [low, high): every N coprime to 30,
 * with no prime factor in 7..113, that is a base-2 strong probable prime.
 * Candidates are appended in increasing order (the reference's order is
 * set by atomics and does not matter).  Walks 60-integer blocks and the
 * wheel exactly as the kernel does (getsegprimes.cl:184-210), including the
 * wrap guards near 2^64 (CKOVERFLOW, :185-209).  Returns the number found
 * (may exceed cap; only cap entries are written). */
uint64_t oracle_candidates(uint64_t low, uint64_t high, uint64_t *out, uint64_t cap)
{
    build_masks();
    if (low >= high)
        return 0;
    uint64_t start = low;
    int32_t widx;
    oracle_find_wheel_offset(&start, &widx);
    if (start < low)     /* wrapped past 2^64: nothing left */
        return 0;
    uint64_t nblk = (high - start) / 60 + 1;
    uint64_t found = 0;
    for (uint64_t g = 0; g < nblk; ++g) {
        uint64_t P = start + g * 60;
        if (P < start)
            break;
        uint64_t end = P + 60;
        if (end > high || end < P)
            end = high;
        if (P >= end)
            break;
        uint32_t sieve = 0;
        for (int j = 0; j < 27; ++j)
            sieve |= mask_tab[j][P % small_q[j]];
        int idx = widx;
        while (P < end) {
            if ((sieve & 1) == 0) {
                oconst c = make_const(P);
                if (sprp2(&c)) {
                    if (found < cap)
                        out[found] = P;
                    ++found;
                }
            }
            int inc = wheel_half_gap[idx++];
            uint64_t nP = P + 2 * (uint64_t)inc;
            sieve >>= inc;
            if (nP < P)
                break;
            P = nP;
        }
    }
    return found;
}

/* The same set by its definition, for cross-checking the walk above. */
uint64_t oracle_candidates_naive(uint64_t low, uint64_t high, uint64_t *out, uint64_t cap)
{
    uint64_t found = 0;
    for (uint64_t n = low; n < high && n >= low; ++n) {
        if (n % 2 == 0 || n % 3 == 0 || n % 5 == 0)
            continue;
        int skip = 0;
        for (int j = 0; j < 27 && !skip; ++j)
            if (n % small_q[j] == 0)
                skip = 1;
        if (skip || !oracle_sprp2(n))
            continue;
        if (found < cap)
            out[found] = n;
        ++found;
        if (n == UINT64_MAX)
            break;
    }
    return found;
}

/* ------------------------------------------------------------------------- */
/* Power table (cl_sieve.cpp:773-838)                                         */
/* ------------------------------------------------------------------------- */

/* Primes in [2, n] by a plain sieve of Eratosthenes; stands in for
 * primesieve_generate_primes(2, nmin) at cl_sieve.cpp:797. */
static uint32_t *primes_upto(uint32_t n, size_t *count)
{
    uint8_t *comp = (uint8_t *)calloc((size_t)n + 1, 1);
    size_t cnt = 0;
    for (uint64_t i = 2; i <= n; ++i) {
        if (comp[i])
            continue;
        ++cnt;
        for (uint64_t j = i * i; j <= n; j += i)
            comp[j] = 1;
    }
    uint32_t *pr = (uint32_t *)malloc(cnt * sizeof(uint32_t) + 4);
    size_t k = 0;
    for (uint64_t i = 2; i <= n; ++i)
        if (!comp[i])
            pr[k++] = (uint32_t)i;
    free(comp);
    *count = cnt;
    return pr;
}

/* Legendre exponent of q in n! and the bit just below its top bit, with the
 * reference's convention that the mark stays 0x80000000 for exponent 1
 * (cl_sieve.cpp:773-788). */
static void legendre(uint32_t q, uint32_t n, uint32_t *e_out, uint32_t *bit_out)
{
    uint32_t e = 0;
    uint64_t qk = q;
    while (qk <= n) {
        e += (uint32_t)(n / qk);
        qk *= q;
    }
    uint32_t bit = 0x80000000u;
    if (e > 1)
        bit >>= (__builtin_clz(e) + 1);
    *e_out = e;
    *bit_out = bit;
}

/* Compressed table: entry 0 is the prime 2; later entries multiply runs of
 * consecutive primes that share an exponent while the product stays below
 * 2^64-1 (cl_sieve.cpp:818-835).  Returns the number of entries (may exceed
 * cap; only cap entries are written). */
uint32_t oracle_power_table(uint32_t nmin, uint64_t *tprime, uint32_t *texp, uint32_t *tbit, uint32_t cap)
{
    size_t np;
    uint32_t *pr = primes_upto(nmin, &np);
    uint32_t m = 0;
    size_t i = 0;
    while (i < np) {
        uint32_t e, b;
        legendre(pr[i], nmin, &e, &b);
        uint64_t prod = pr[i];
        ++i;
        if (m > 0) {     /* entry 0 (the prime 2) is never merged */
            while (i < np) {
                uint32_t e2, b2;
                legendre(pr[i], nmin, &e2, &b2);
                if (e2 != e)
                    break;
                u128 pp = (u128)prod * pr[i];
                if (pp >= (u128)UINT64_MAX)
                    break;
                prod = (uint64_t)pp;
                ++i;
            }
        }
        if (m < cap) {
            tprime[m] = prod;
            texp[m] = e;
            tbit[m] = b;
        }
        ++m;
    }
    free(pr);
    return m;
}

/* ------------------------------------------------------------------------- */
/* setup / iterate / check for one candidate                                  */
/* ------------------------------------------------------------------------- */

/* nmin! * R mod p from the table (setup.cl:56-102). */
static uint64_t setup_one(const oconst *c, const uint64_t *tprime, const uint32_t *texp,
                          const uint32_t *tbit, uint32_t tlen)
{
    const uint64_t p = c->p, q = c->q;
    uint64_t a = c->two;
    uint32_t bit = tbit[0];
    for (; bit; bit >>= 1) {      /* 2^e by squaring and modular doubling */
        a = oracle_mmul(a, a, p, q);
        if (texp[0] & bit)
            a = oracle_madd(a, a, p);
    }
    uint64_t s6 = a;
    for (uint32_t i = 1; i < tlen; ++i) {
        uint64_t base = oracle_mmul(tprime[i], c->r2, p, q);
        uint64_t pw = base;
        if (texp[i] != 1) {
            for (uint32_t b = tbit[i]; b; b >>= 1) {
                pw = oracle_mmul(pw, pw, p, q);
                if (texp[i] & b)
                    pw = oracle_mmul(pw, base, p, q);
            }
        }
        s6 = oracle_mmul(s6, pw, p, q);
    }
    return s6;
}

uint64_t oracle_setup(uint64_t p, const uint64_t *tprime, const uint32_t *texp, const uint32_t *tbit,
                      uint32_t tlen)
{
    oconst c = make_const(p);
    return setup_one(&c, tprime, texp, tbit, tlen);
}

/* Reference factor record (cl_sieve.h:3-6): 16 bytes with padding. */
typedef struct {
    uint64_t p;
    int32_t nc;
    int32_t pad;
} ofactor;

/* setup + iterate + check over a candidate list.
 *   raw_sum     += sum over candidates of (s6 + s7)          (check.cl:64, 88-98)
 *   *nvalidfail  = number of candidates failing the nmax round trip (check.cl:67-78)
 *   factors      = every (p, +-n) hit, unsorted             (iterate.cl:69-73)
 * s6_out/s7_out, when not NULL, receive the final residues per candidate.
 * Returns the number of hits (may exceed fcap). */
uint64_t oracle_sieve_list(const uint64_t *cand, uint64_t ncand, uint32_t nmin, uint32_t nmax,
                           const uint64_t *tprime, const uint32_t *texp, const uint32_t *tbit,
                           uint32_t tlen, uint64_t *raw_sum, uint64_t *nvalidfail,
                           ofactor *factors, uint64_t fcap, uint64_t *s6_out, uint64_t *s7_out)
{
    uint64_t sum = 0, nhit = 0, bad = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : sum, bad)
    for (int64_t i = 0; i < (int64_t)ncand; ++i) {
        oconst c = make_const(cand[i]);
        const uint64_t p = c.p, q = c.q;
        uint64_t s6 = setup_one(&c, tprime, texp, tbit, tlen);
        uint64_t s7 = oracle_mmul(nmin, c.r2, p, q);
        for (uint32_t n = nmin; n < nmax; ++n) {
            s7 = oracle_madd(s7, c.one, p);
            if (s6 == c.one || s6 == c.nmo) {
                uint64_t k;
#pragma omp atomic capture
                k = nhit++;
                if (k < fcap) {
                    factors[k].p = p;
                    factors[k].nc = (s6 == c.one) ? -(int32_t)n : (int32_t)n;
                    factors[k].pad = 0;
                }
            }
            s6 = oracle_mmul(s6, s7, p, q);
        }
        sum += s6 + s7;
        uint32_t back = (uint32_t)oracle_mmul(s7, 1, p, q);
        if (p <= nmax && nmax % p == back)
            back = nmax;
        if (back != nmax)
            ++bad;
        if (s6_out)
            s6_out[i] = s6;
        if (s7_out)
            s7_out[i] = s7;
    }
    *raw_sum += sum;
    *nvalidfail += bad;
    return nhit;
}

/* ------------------------------------------------------------------------- */
/* Host post-processing (cl_sieve.cpp:422-554, verifyprime.c:105-173)         */
/* ------------------------------------------------------------------------- */

/* Slow check that p | n! + c, from 34! (verifyprime.c:146-173). */
int oracle_verify(uint64_t p, uint32_t n, int32_t c)
{
    const u128 f34 = ((u128)0xde1bc4d19efcac82ull << 64) | 0x445da75b00000000ull;
    uint64_t r = (uint64_t)(f34 % p);
    if (p < 0xFFFFFFFFull) {
        for (uint64_t i = 35; i <= n; ++i)
            r = (r * i) % p;
    } else {
        for (uint64_t i = 35; i <= n; ++i)
            r = (uint64_t)(((u128)r * i) % p);
    }
    if (c == -1)
        return r == 1;
    if (c == 1)
        return r == p - 1;
    return 0;
}

/* Deterministic Miller-Rabin with the seven bases valid below 2^64
 * (verifyprime.c:62-141). */
int oracle_is_prime(uint64_t p)
{
    static const uint32_t bases[7] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
    if (p % 2 == 0)
        return 0;
    oconst c = make_const(p);
    int t = __builtin_ctzll(p - 1);
    uint64_t d = p >> t;
    uint64_t top = d > 1 ? 0x8000000000000000ull >> (__builtin_clzll(d) + 1) : 0;
    for (int i = 0; i < 7; ++i) {
        uint64_t b = bases[i];
        if (b >= p) {
            b %= p;
            if (b == 0)
                continue;
        }
        uint64_t mb = oracle_mmul(b, c.r2, p, c.q);
        uint64_t a = mb;
        for (uint64_t bit = top; bit; bit >>= 1) {
            a = oracle_mmul(a, a, p, c.q);
            if (d & bit)
                a = oracle_mmul(a, mb, p, c.q);
        }
        int ok = (a == c.one || a == c.nmo);
        for (int s = 1; s < t && !ok; ++s) {
            a = oracle_mmul(a, a, p, c.q);
            if (a == c.nmo)
                ok = 1;
        }
        if (!ok)
            return 0;
    }
    return 1;
}

static int cmp_factor(const void *x, const void *y)
{
    const ofactor *a = (const ofactor *)x, *b = (const ofactor *)y;
    if (a->p != b->p)
        return a->p < b->p ? -1 : 1;
    int32_t na = a->nc < 0 ? -a->nc : a->nc, nb = b->nc < 0 ? -b->nc : b->nc;
    if (na != nb)
        return na < nb ? -1 : 1;
    return (a->nc > b->nc) - (a->nc < b->nc);
}

/* Sort by (p, |n|), verify each hit on the CPU, drop hits whose p is not
 * prime, and fold the kept ones into the checksum as n + c (cl_sieve.cpp:
 * 485-550).  Kept factors are compacted to the front of f.  Returns the
 * number kept, or -1 if a hit fails verification. */
int64_t oracle_postprocess(ofactor *f, uint64_t n, uint64_t *checksum, uint64_t *ndiscarded)
{
    qsort(f, n, sizeof(ofactor), cmp_factor);
    int fail = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : fail)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        uint32_t fn = (uint32_t)(f[i].nc < 0 ? -f[i].nc : f[i].nc);
        int32_t fc = f[i].nc < 0 ? -1 : 1;
        if (!oracle_verify(f[i].p, fn, fc))
            fail = 1;
    }
    if (fail)
        return -1;
    uint64_t kept = 0, last_good = 0, disc = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t fp = f[i].p;
        uint32_t fn = (uint32_t)(f[i].nc < 0 ? -f[i].nc : f[i].nc);
        int32_t fc = f[i].nc < 0 ? -1 : 1;
        if (fp == last_good || oracle_is_prime(fp)) {
            last_good = fp;
            *checksum += (uint32_t)(fn + (uint32_t)fc);
            f[kept++] = f[i];
        } else {
            ++disc;
        }
    }
    if (ndiscarded)
        *ndiscarded = disc;
    return (int64_t)kept;
}

/* ------------------------------------------------------------------------- */
/* End to end (cl_sieve.cpp:918-1270 without the device plumbing)            */
/* ------------------------------------------------------------------------- */

typedef struct {
    uint64_t primecount;   /* number of candidates (pseudoprimes included) */
    uint64_t checksum;     /* final checksum as printed by the reference */
    uint64_t factorcount;  /* kept factors */
    uint64_t raw_sum;      /* sum of (s6 + s7) alone */
    uint64_t nhits;        /* hits before the 2-PRP filter */
    uint64_t ndiscarded;   /* hits dropped because p was not prime */
    uint64_t nvalidfail;   /* nmax round-trip failures (must be 0) */
    int64_t status;        /* 0 ok, -1 verify failure, -2 factor buffer overflow, -3 alloc */
} oresult;

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Whole search over p in [pmin, pmax), n in [nmin, nmax).  The p-range is
 * walked in segments of seg_width (any width gives the same result; the
 * reference sizes them by GPU timing).  Kept factors are written to
 * factors[0..factorcount) sorted by (p, |n|). */
int oracle_run(uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax, uint64_t seg_width,
               ofactor *factors, uint64_t fcap, oresult *res)
{
    memset(res, 0, sizeof(*res));
    uint32_t tcap = nmin / 2 + 64;
    uint64_t *tp = (uint64_t *)malloc(tcap * sizeof(uint64_t));
    uint32_t *te = (uint32_t *)malloc(tcap * sizeof(uint32_t));
    uint32_t *tb = (uint32_t *)malloc(tcap * sizeof(uint32_t));
    uint32_t tlen = oracle_power_table(nmin, tp, te, tb, tcap);
    if (seg_width == 0)
        seg_width = 10000000;
    uint64_t ccap = seg_width / 4 + 1024;
    uint64_t *cand = (uint64_t *)malloc(ccap * sizeof(uint64_t));
    if (!tp || !te || !tb || !cand || tlen > tcap) {
        res->status = -3;
        free(tp); free(te); free(tb); free(cand);
        return -3;
    }
    uint64_t nhit = 0;
    for (uint64_t lo = pmin; lo < pmax;) {
        uint64_t hi = lo + seg_width;
        if (hi > pmax || hi < lo)
            hi = pmax;
        uint64_t nc = oracle_candidates(lo, hi, cand, ccap);
        res->primecount += nc;
        uint64_t room = nhit < fcap ? fcap - nhit : 0;
        uint64_t h = oracle_sieve_list(cand, nc, nmin, nmax, tp, te, tb, tlen, &res->raw_sum,
                                       &res->nvalidfail, factors + (nhit < fcap ? nhit : fcap),
                                       room, NULL, NULL);
        nhit += h;
        if (hi == pmax)
            break;
        lo = hi;
    }
    free(tp); free(te); free(tb); free(cand);
    res->nhits = nhit;
    if (nhit > fcap) {
        res->status = -2;
        return -2;
    }
    res->checksum = res->raw_sum;
    int64_t kept = oracle_postprocess(factors, nhit, &res->checksum, &res->ndiscarded);
    if (kept < 0) {
        res->status = -1;
        return -1;
    }
    res->factorcount = (uint64_t)kept;
    return 0;
}
