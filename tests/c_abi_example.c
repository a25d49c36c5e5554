/* A plain C caller of libfactsieve.so's host-side entry points (no GPU
 * needed): parse the reference's argument forms, check primality and
 * factors, post-process a few hit records the way getResults does, and
 * report the walk step a segment would run.  Built and run by
 * tests/test_host.py::test_c_caller; prints one "key value" line per check. */
#include <stdint.h>
#include <stdio.h>

#include "factsieve.h"

int main(void) {
    uint64_t pmin = 0, pmax = 0;
    uint32_t nmin = 0;
    printf("version %d\n", fs_version());
    const int rp = fs_parse_uint64(&pmin, "1e12", 127, UINT64_MAX - 1);
    const int rP = fs_parse_uint64(&pmax, "1001e9", 128, UINT64_MAX);
    const int rn = fs_parse_uint(&nmin, "1e5", 127, 0x7FFFFFFEu);
    printf("parse_p %d %llu\n", rp, (unsigned long long)pmin);
    printf("parse_P %d %llu\n", rP, (unsigned long long)pmax);
    printf("parse_n %d %u\n", rn, nmin);
    printf("bad_arg %d\n", fs_parse_uint64(&pmin, "2x", 127, UINT64_MAX));
    printf("is_prime %d %d\n", fs_is_prime(1000000007ull), fs_is_prime(1000000007ull * 3));
    /* 149 | 25! - 1 and 1000047465737 | 169725! + 1 (a config 2 factor) */
    printf("verify %d %d %d\n", fs_verify_factor(149, 25, -1), fs_verify_factor(149, 25, 1),
           fs_verify_factor(1000047465737ull, 169725, 1));
    /* two true hits, one duplicate p, one hit whose p is composite (discarded) */
    fs_factor f[4] = {{1000047465737ull, 169725, 0}, {149, -25, 0}, {149, 24, 0}, {0, 0, 0}};
    uint64_t kept = 0, cs = 0, disc = 0;
    int rc = fs_postprocess(f, 2, 2, &kept, &cs, &disc);
    printf("postprocess %d %llu %llu %llu %llu\n", rc, (unsigned long long)kept, (unsigned long long)cs,
           (unsigned long long)disc, (unsigned long long)f[0].p);
    printf("capacity %llu\n", (unsigned long long)fs_candidate_capacity(1000000000000ull, 1000100000000ull));
    printf("walk_step %d %d\n", fs_walk_step(1000000000000ull, 1001000000000ull, 200000),
           fs_walk_step(1000000ull, 2000000ull, 2000));
    printf("strerror %s\n", fs_strerror(FS_E_OVERFLOW));
    return 0;
}
