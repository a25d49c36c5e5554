// fs_putil.cpp -- numeric command-line arguments with size suffixes.
//
// Same accepted syntax and results as the reference's parser (putil.c:18-116):
// a C integer literal (decimal, 0x hex, 0 octal) optionally followed by
//   K M G T P   x 1000^1..5          e<d> / E<d>   x 10^d
//   k m g t p   x 2^(10..50)         b<d> / B<d>   x 2^d
// Returns 0 on success, -1 if the text does not parse, -2 if the value falls
// outside [lo, hi] (checked before and after scaling, without overflow).
#include "../../include/factsieve.h"

#include <cerrno>
#include <cstdlib>

extern "C" int fs_parse_uint64(uint64_t* result, const char* str, uint64_t lo, uint64_t hi) {
    if (!result || !str) return -1;
    char* tail = nullptr;
    errno = 0;
    uint64_t v = strtoull(str, &tail, 0);
    if (errno != 0 || v > hi) return -2;
    const char c = *tail;
    auto scale_dec = [&](unsigned times) -> int {
        for (unsigned i = 0; i < times && v; ++i) {
            if (v > hi / 10) return -2;
            v *= 10;
        }
        return 0;
    };
    auto scale_bin = [&](unsigned bits) -> int {
        for (unsigned i = 0; i < bits && v; ++i) {
            if (v > (hi >> 1)) return -2;
            v <<= 1;
        }
        return 0;
    };
    int rc = 0;
    switch (c) {
        case '\0':
            break;
        case 'K': case 'M': case 'G': case 'T': case 'P': {
            if (tail[1] != '\0') return -1;
            const unsigned k = c == 'K' ? 1 : c == 'M' ? 2 : c == 'G' ? 3 : c == 'T' ? 4 : 5;
            rc = scale_dec(3 * k);
            break;
        }
        case 'k': case 'm': case 'g': case 't': case 'p': {
            if (tail[1] != '\0') return -1;
            const unsigned k = c == 'k' ? 1 : c == 'm' ? 2 : c == 'g' ? 3 : c == 't' ? 4 : 5;
            rc = scale_bin(10 * k);
            break;
        }
        case 'e': case 'E': case 'b': case 'B': {
            char* end = nullptr;
            errno = 0;
            unsigned long d = strtoul(tail + 1, &end, 0);
            if (errno != 0) return -2;
            if (*end != '\0') return -1;
            rc = (c == 'e' || c == 'E') ? scale_dec((unsigned)d) : scale_bin((unsigned)d);
            break;
        }
        default:
            return -1;
    }
    if (rc) return rc;
    if (v < lo) return -2;
    *result = v;
    return 0;
}

extern "C" int fs_parse_uint(uint32_t* result, const char* str, uint32_t lo, uint32_t hi) {
    uint64_t v = 0;
    int rc = fs_parse_uint64(&v, str, lo, hi);
    if (rc == 0) *result = (uint32_t)v;
    return rc;
}
