// fs_host.cpp -- host-side tables and CPU checks of the FactSieve path.
#include "fs_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

namespace fs {

typedef unsigned __int128 u128;

std::vector<uint32_t> primes_upto(uint32_t n) {
    std::vector<uint32_t> out;
    if (n < 2) return out;
    out.push_back(2);
    if (n < 3) return out;
    // odd-only segmented sieve; base primes up to sqrt(n)
    const uint32_t root = (uint32_t)std::sqrt((double)n) + 2;
    std::vector<uint8_t> small(root + 1, 0);
    std::vector<uint32_t> base;
    for (uint32_t i = 3; i <= root; i += 2) {
        if (small[i]) continue;
        base.push_back(i);
        for (uint64_t j = (uint64_t)i * i; j <= root; j += 2 * i) small[j] = 1;
    }
    out.reserve((size_t)(n / std::max(std::log((double)n) - 1.1, 1.0)) + 16);   // pi(n) < n / (ln n - 1.1)
    const uint64_t SEG = 1u << 19;  // odd numbers per segment
    std::vector<uint8_t> seg(SEG);
    for (uint64_t lo = 3; lo <= n; lo += 2 * SEG) {
        uint64_t hi = std::min<uint64_t>((uint64_t)n + 1, lo + 2 * SEG);  // [lo, hi)
        std::fill(seg.begin(), seg.end(), 0);
        for (uint32_t q : base) {
            uint64_t q2 = (uint64_t)q * q;
            if (q2 >= hi) break;
            uint64_t s = std::max<uint64_t>(q2, ((lo + q - 1) / q) * q);
            if ((s & 1) == 0) s += q;
            for (uint64_t j = s; j < hi; j += 2 * q) seg[(j - lo) >> 1] = 1;
        }
        for (uint64_t j = lo; j < hi; j += 2)
            if (!seg[(j - lo) >> 1]) out.push_back((uint32_t)j);
    }
    return out;
}

// The primes up to n from one list kept for the process (grown when a larger
// n comes): the setup plan of every search, batch job and served job starts
// from it, and sieving again each time was a third of a plan's host time.
// Above n = 2^27 (7.4 million primes, 30 MB) nothing is kept.
std::vector<uint32_t> primes_upto_cached(uint32_t n) {
    constexpr uint32_t kKeepUpto = 1u << 27;
    if (n > kKeepUpto) return primes_upto(n);
    static std::mutex mu;
    static std::vector<uint32_t> list;
    static uint32_t upto = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (n > upto) {
        list = primes_upto(n);
        upto = n;
    }
    return std::vector<uint32_t>(list.begin(), std::upper_bound(list.begin(), list.end(), n));
}

uint32_t legendre(uint32_t q, uint32_t n) {
    uint32_t e = 0;
    for (uint64_t qk = q; qk <= n; qk *= q) e += (uint32_t)(n / qk);
    return e;
}

RefTable reference_table(uint32_t n) {
    RefTable t;
    const std::vector<uint32_t> pr = primes_upto_cached(n);
    size_t i = 0;
    while (i < pr.size()) {
        uint32_t e = legendre(pr[i], n);
        uint64_t prod = pr[i++];
        if (!t.prime.empty()) {  // entry 0 (the prime 2) stays alone
            while (i < pr.size() && legendre(pr[i], n) == e) {
                u128 pp = (u128)prod * pr[i];
                if (pp >= (u128)UINT64_MAX) break;
                prod = (uint64_t)pp;
                ++i;
            }
        }
        uint32_t bit = 0x80000000u;
        if (e > 1) bit >>= (__builtin_clz(e) + 1);
        t.prime.push_back(prod);
        t.exp.push_back(e);
        t.bit.push_back(bit);
    }
    return t;
}

// Pack the odd primes of one layer (ascending) into 64-bit words, best fit
// decreasing: each word starts from the largest prime left and takes the
// largest prime that still fits until none does.  Most words are three large
// primes (about 60 bits) and the holes fill with small ones; against packing
// the ascending list in order this saves 9.7 % of the words (and of the
// setup's products) for n = 1e5, 5.7 % for 5e5 and 3.7 % for 1e6.  The
// remaining primes are found through a union-find over the sorted list whose
// links point from a taken slot to the next one below it.
static void pack_layer(const std::vector<uint32_t>& v, std::vector<uint64_t>& words) {
    const uint32_t m = (uint32_t)v.size();
    if (m == 0) return;
    std::vector<uint32_t> below(m + 1);   // slot i + 1 holds v[i]; 0: none left
    for (uint32_t i = 0; i <= m; ++i) below[i] = i;
    // slots holding primes <= x, for the common cases without a search: x at
    // least the largest prime (a word's second and third prime, as a rule)
    // and x below 4096 (the small prime that fills a word's hole)
    constexpr uint32_t kSmall = 4096;
    std::vector<uint32_t> upto(kSmall);
    for (uint32_t x = 0, i = 0; x < kSmall; ++x) {
        while (i < m && v[i] <= x) ++i;
        upto[x] = i;
    }
    const uint64_t vmax = v[m - 1];
    auto find = [&below](uint32_t x) {
        while (below[x] != x) {
            below[x] = below[below[x]];
            x = below[x];
        }
        return x;
    };
    // the largest slot left: slots go mostly from the top, so a cursor that
    // only moves down finds it without the union-find
    uint32_t hi = m;
    auto top_left = [&below, &hi]() {
        while (hi != 0 && below[hi] != hi) --hi;
        return hi;
    };
    // the largest slot left whose prime fits beside w (one 64-bit division
    // only when even the largest prime does not)
    auto largest_fit = [&](uint64_t w) -> uint32_t {
        if ((u128)w * vmax <= (u128)UINT64_MAX) return top_left();
        const uint64_t x = UINT64_MAX / w;
        if (x < kSmall) return find(upto[x]);
        return find((uint32_t)(std::upper_bound(v.begin(), v.end(), x) - v.begin()));
    };
    for (uint32_t top = top_left(); top != 0; top = top_left()) {
        uint64_t w = v[top - 1];
        below[top] = top - 1;
        for (;;) {
            const uint32_t s = largest_fit(w);
            if (s == 0) break;
            w *= v[s - 1];
            below[s] = s - 1;
        }
        words.push_back(w);
    }
}

SetupPlan build_plan(uint32_t n, uint32_t chunks) {
    SetupPlan plan;
    plan.n = n;
    const std::vector<uint32_t> pr = primes_upto_cached(n);
    plan.nprimes = pr.size();
    const uint32_t e2 = n >= 2 ? legendre(2, n) : 0;
    // odd primes and their exponents
    std::vector<uint32_t> q, e;
    q.reserve(pr.size());
    e.reserve(pr.size());
    for (uint32_t x : pr)
        if (x != 2) {
            q.push_back(x);
            e.push_back(legendre(x, n));
        }
    if (chunks < 1) chunks = 1;
    std::vector<size_t> cut(chunks + 1, q.size());
    cut[0] = 0;
    if (chunks > 1) {
        // balance chunks by bit mass sum(log2 q * popcount(e))
        std::vector<double> mass(q.size());
        double total = 0;
        for (size_t i = 0; i < q.size(); ++i) {
            mass[i] = std::log2((double)q[i]) * __builtin_popcount(e[i]);
            total += mass[i];
        }
        double acc = 0;
        uint32_t c = 1;
        for (size_t i = 0; i < q.size() && c < chunks; ++i) {
            acc += mass[i];
            if (acc >= total * c / chunks) cut[c++] = i + 1;
        }
        for (; c < chunks; ++c) cut[c] = q.size();
    }
    for (uint32_t c = 0; c < chunks; ++c) {
        PlanChunk ch;
        ch.layer_begin = (uint32_t)plan.layers.size();
        ch.deficit = 0;
        uint32_t emax = (c == 0) ? e2 : 0;
        for (size_t i = cut[c]; i < cut[c + 1]; ++i) emax = std::max(emax, e[i]);
        int nbits = emax ? 32 - __builtin_clz(emax) : 0;
        // each layer's primes, ascending: one pass over the chunk's primes
        std::vector<std::vector<uint32_t>> lq(nbits);
        for (size_t i = cut[c]; i < cut[c + 1]; ++i)
            for (uint32_t x = e[i]; x; x &= x - 1) lq[__builtin_ctz(x)].push_back(q[i]);
        for (int b = nbits - 1; b >= 0; --b) {
            PlanLayer L;
            L.begin = (uint32_t)plan.words.size();
            L.dbl = (c == 0 && ((e2 >> b) & 1)) ? 1u : 0u;
            L.pad = 0;
            pack_layer(lq[b], plan.words);
            L.end = (uint32_t)plan.words.size();
            // Horner: the first layer of a chunk starts from 1 (no squaring)
            if (b != nbits - 1) ch.deficit *= 2;
            ch.deficit += (uint64_t)(L.end - L.begin);
            plan.layers.push_back(L);
        }
        ch.layer_end = (uint32_t)plan.layers.size();
        plan.deficit += ch.deficit;
        plan.chunks.push_back(ch);
    }
    return plan;
}

// ------------------------------------------------------------ CPU checks --

static uint64_t mmul(uint64_t a, uint64_t b, uint64_t p, uint64_t pinv) {
    u128 ab = (u128)a * b;
    uint64_t lo = (uint64_t)ab, hi = (uint64_t)(ab >> 64);
    uint64_t mp = (uint64_t)(((u128)(lo * pinv) * p) >> 64);
    return hi >= mp ? hi - mp : hi - mp + p;
}

bool is_prime_u64(uint64_t p) {
    if (p < 2) return false;
    if (p % 2 == 0) return p == 2;
    if (p < 9) return true;   // 3, 5, 7
    static const uint64_t bases[7] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
    uint64_t pinv = p;
    for (int i = 0; i < 5; ++i) pinv *= 2 - p * pinv;
    const uint64_t one = (uint64_t)((((u128)1) << 64) % p);
    const uint64_t r2 = (uint64_t)(((u128)one * one) % p);
    const uint64_t pm1 = p - one;
    int t = __builtin_ctzll(p - 1);
    uint64_t d = (p - 1) >> t;
    for (uint64_t b : bases) {
        uint64_t a0 = b % p;
        if (a0 == 0) continue;
        uint64_t mb = mmul(a0, r2, p, pinv);
        uint64_t a = one;
        for (int bit = 63 - __builtin_clzll(d); bit >= 0; --bit) {
            a = mmul(a, a, p, pinv);
            if ((d >> bit) & 1) a = mmul(a, mb, p, pinv);
        }
        if (a == one || a == pm1) continue;
        bool ok = false;
        for (int s = 1; s < t; ++s) {
            a = mmul(a, a, p, pinv);
            if (a == pm1) {
                ok = true;
                break;
            }
        }
        if (!ok) return false;
    }
    return true;
}

bool verify_factor(uint64_t p, uint32_t n, int32_t c) {
    if (p < 3 || (p & 1) == 0 || (c != 1 && c != -1)) return false;
    // n! mod p by the plain running product (independent of the GPU's
    // table-driven setup).  Small p: 64-bit remainders.  Large p: Montgomery
    // products with the multiplier's image advanced by R each step.
    if (p <= 0xFFFFFFFFull) {
        uint64_t r = 1;
        for (uint64_t i = 2; i <= n && r; ++i) r = (r * (i % p)) % p;
        return c == -1 ? r == 1 : r == p - 1;
    }
    uint64_t pinv = p;
    for (int i = 0; i < 5; ++i) pinv *= 2 - p * pinv;
    const uint64_t one = (uint64_t)((((u128)1) << 64) % p);
    uint64_t r = one, k = one;                  // r = 1!*R, k = 1*R
    for (uint64_t i = 2; i <= n && r; ++i) {
        k = (k >= p - one) ? k + one - p : k + one;   // i*R mod p
        r = mmul(r, k, p, pinv);
    }
    return c == -1 ? r == one : r == p - one;
}

}  // namespace fs
