// fs_host.h -- host-side pieces of the FactSieve path (C++, no CUDA).
#pragma once
#include <stdint.h>
#include <vector>

namespace fs {

// Primes in [2, n] by a segmented odd-only sieve of Eratosthenes.  Stands in
// for primesieve_generate_primes(2, nmin) (cl_sieve.cpp:797); the library's
// source is not part of the reference tree.
std::vector<uint32_t> primes_upto(uint32_t n);
std::vector<uint32_t> primes_upto_cached(uint32_t n);

// Legendre exponent of prime q in n!.
uint32_t legendre(uint32_t q, uint32_t n);

// Reference power table for n! (cl_sieve.cpp:773-838): entry 0 is the prime
// 2; later entries are products of runs of consecutive primes with equal
// exponent, kept while the product is below 2^64-1.  bit is the ladder mark
// (the bit below the exponent's top bit; 0x80000000 for exponent 1).
struct RefTable {
    std::vector<uint64_t> prime;
    std::vector<uint32_t> exp, bit;
};
RefTable reference_table(uint32_t n);

// Bit-layered setup plan for n!, the form the GPU setup consumes.
//
// n! = 2^e2 * prod_{odd q <= n} q^e_q.  Writing every exponent in binary,
// n! = prod_b L_b^(2^b) with L_b the product of the odd primes whose
// exponent has bit b set, so Horner over the bits costs one squaring per bit
// plus one multiplication per word of L_b (primes packed into u64 words,
// product < 2^64), and the 2^e2 factor becomes one modular doubling on each
// layer whose bit is set in e2.  Multiplying a Montgomery residue by a raw
// word w with a Montgomery product yields x*w*R^-1, so each word leaves a
// factor R^-1 ("deficit"); squarings double the deficit.  The device
// multiplies once by R^(D+1) at the end, D = total deficit.
//
// The odd primes are split into `chunks` contiguous groups with their own
// layers so several threads can build one prime's residue; partial results
// multiply together (their deficits add).
struct PlanLayer {
    uint32_t begin, end;   // word range [begin, end)
    uint32_t dbl;          // 1: double (multiply by 2) after the squaring
    uint32_t pad;
};
struct PlanChunk {
    uint32_t layer_begin, layer_end;
    uint64_t deficit;
};
struct SetupPlan {
    uint32_t n = 0;
    std::vector<uint64_t> words;
    std::vector<PlanLayer> layers;
    std::vector<PlanChunk> chunks;
    uint64_t deficit = 0;          // sum over chunks
    uint64_t nprimes = 0;          // primes <= n
};
SetupPlan build_plan(uint32_t n, uint32_t chunks);

// CPU arithmetic for the factor post-processing (cl_sieve.cpp:439-554).
bool is_prime_u64(uint64_t p);                        // 7-base deterministic Miller-Rabin
bool verify_factor(uint64_t p, uint32_t n, int32_t c); // p | n! + c by the slow product

}  // namespace fs
