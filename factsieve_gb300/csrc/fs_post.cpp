// fs_post.cpp -- getResults' CPU half (cl_sieve.cpp:484-550) behind the C ABI.
#include <omp.h>

#include <algorithm>
#include <atomic>

#include "../../include/factsieve.h"
#include "fs_host.h"

extern "C" int fs_postprocess(fs_factor* f, uint64_t n, int threads, uint64_t* kept, uint64_t* checksum_add,
                              uint64_t* discarded) {
    if (!f && n) return FS_E_ARG;
    // (p, |n|) order as factorcompare (cl_sieve.cpp:422-436); equal keys are
    // ordered by sign so the result does not depend on the GPU's hit order
    std::sort(f, f + n, [](const fs_factor& a, const fs_factor& b) {
        if (a.p != b.p) return a.p < b.p;
        int32_t na = a.nc < 0 ? -a.nc : a.nc, nb = b.nc < 0 ? -b.nc : b.nc;
        if (na != nb) return na < nb;
        return a.nc < b.nc;
    });
    std::atomic<int> bad{0};
    const int nt = threads > 0 ? threads : 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        uint32_t fn = (uint32_t)(f[i].nc < 0 ? -f[i].nc : f[i].nc);
        int32_t fc = f[i].nc < 0 ? -1 : 1;
        if (!fs::verify_factor(f[i].p, fn, fc)) bad = 1;
    }
    if (bad) return FS_E_VERIFY;
    uint64_t k = 0, disc = 0, cs = 0, last_good = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t fp = f[i].p;
        uint32_t fn = (uint32_t)(f[i].nc < 0 ? -f[i].nc : f[i].nc);
        int32_t fc = f[i].nc < 0 ? -1 : 1;
        // the GPU keeps base-2 strong probable primes; only prime p are factors
        if (fp == last_good || fs::is_prime_u64(fp)) {
            last_good = fp;
            cs += (uint32_t)(fn + (uint32_t)fc);
            f[k++] = f[i];
        } else {
            ++disc;
        }
    }
    if (kept) *kept = k;
    if (checksum_add) *checksum_add = cs;
    if (discarded) *discarded = disc;
    return FS_OK;
}
