// fs_launch.h -- kernel argument blocks and launch wrappers (host <-> device).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_kernels.cuh"

namespace fs {

// SETUP_PLAN_PM: SETUP_PLAN for a launch whose candidates all lie in
// (2^63, 2^63 + 2^30), with the folding product of that form (four
// candidates per thread, 96-bit walks only).
enum { SETUP_LOAD = 0, SETUP_PLAN = 1, SETUP_PARTIALS = 2, SETUP_PLAN_PM = 3 };
// Walk step used for every candidate of a launch (WALK_ANY: per candidate).
enum { WALK_ANY = 0, WALK_T64 = 1, WALK_L96 = 2, WALK_C96 = 3, WALK_H64 = 4, WALK_H96 = 5, WALK_H32 = 6, WALK_HM = 7,
       WALK_C96H = 8, WALK_HF = 9, WALK_HG = 10, WALK_HGL = 11, WALK_HG96 = 12,
       WALK_C96G = 13 };

// Candidate generator over the odd numbers o0 + 2 j < high.
struct GenArgs {
    u64 o0;          // first odd number >= low
    u64 high;        // exclusive
    u64 nwords;      // ceil((high - o0) / 64): words of 32 odd numbers
    u32 r0[29];      // o0 mod q for the 29 sieving primes 3..113
    u32 cap;         // capacity of cand[]
    u64* cand;       // out: candidates (unordered)
    Counters* ctr;   // ctr->ncand counts every candidate found, even past cap
};

struct PlanChunkDev {
    u32 layer_begin, layer_end;
    u64 deficit;
};

struct SieveArgs {
    const u64* cand;      // candidates
    const u32* ncand;     // device count (read by the kernel)
    u32 cap;              // capacity of cand[] / residue[]
    u64* residue;         // starting residues (SETUP_LOAD), updated residues (non-final)
    u32* walked;          // per candidate, the n its residue stands at (read with SETUP_LOAD, written by
                          // non-final launches); nullptr: no earlier launch, residues start at nstart
    u64* partials;        // SETUP_PARTIALS: nchunks x cap partial products
    u32 nchunks;
    const PlanChunkDev* chunks;
    PlanDev plan;         // words/layers; layer range and total deficit for SETUP_PLAN
    u32 nstart, nend;     // walk n over [nstart, nend)
    u32 nmax;             // final n (s7 = nmax * R) on the final chunk
    u32 count_candidates; // final chunk adds ncand to the candidate total
    Factor* hits;
    u32 hitcap;
    Counters* ctr;
};

struct TableCheckArgs {
    const u64* cand;
    const u32* ncand;
    u32 n0;
    const u64* words;
    const Layer* layers;
    const PlanChunkDev* chunks;
    u32 nchunks;
    u64 deficit;
    u64* scratch;     // one u64 per block
    u32* done;        // block completion counter (reset by the last block)
    u64* result;      // [direct, table]
    Counters* ctr;
};

// One job of a batch: its candidates, n-range and setup-plan layers.
struct BatchJob {
    const u64* cand;
    u32 cap;
    u32 nstart, nend;            // walk [nstart, nend); the walk must reach nend (= the job's nmax)
    u32 layer_begin, layer_end;  // its plan's layers in the shared layer table
    u32 walk;                    // WALK_* step valid for the job's whole p-range
    u64 deficit;
};

struct BatchArgs {
    const BatchJob* jobs;
    u32 njobs;
    Counters* ctr;               // per job: ncand (from the generator), raw_sum, flags
    Counters* gctr;              // batch-wide: nhits, overflow flags
    u32* tile_counter;           // zeroed before each run
    const u64* words;
    const Layer* layers;
    Factor* hits;                // pad = job index
    u32 hitcap;
    u32 tile_candidates;         // candidates per tile: a multiple of kTileCandidates
};

// Candidates per tile of the batch and serving kernels (four per thread).
constexpr u32 kTileCandidates = 4 * 256;

// Serving round: one chunk = a block of one job's candidates in one phase;
// the kernel cuts chunks into tiles of kTileCandidates.
enum : u32 { SERVE_SETUP = 1u, SERVE_FINAL = 2u };
struct ServeChunk {
    const u64* cand;
    u64* residue;
    u32* walked;                 // per candidate, the n its residue stands at between rounds
    Counters* ctr;               // the job's counters (raw_sum, flags)
    const u64* words;            // the job's setup plan
    const Layer* layers;
    u64 deficit;
    u32 layer_begin, layer_end;
    u32 first, count;            // candidates [first, first + count)
    u32 nstart, nend;            // walk [nstart, nend)
    u32 nmax;                    // the job's nmax: a final chunk's walks must have reached it
    u32 flags;                   // SERVE_SETUP: start from the plan; SERVE_FINAL: checksum, no store
    u32 tag;                     // job slot, stored in hit records
    u32 tile_end;                // inclusive prefix of tiles over the round's chunks
    u32 walk;                    // WALK_* step valid for the job's whole p-range and this chunk's n
};

constexpr int kServeMaxChunks = 4096;

struct ServeArgs {
    const ServeChunk* chunks;
    u32 nchunks;
    u32* tile_counter;
    Counters* gctr;              // round-wide hit count and overflow flag
    Factor* hits;
    u32 hitcap;
};

cudaError_t launch_serve_round(const ServeArgs& a, int grid, cudaStream_t s, int ppt);
cudaError_t serve_occupancy(int* blocks_per_sm, int ppt);
cudaError_t launch_gen(const GenArgs& a, int grid, cudaStream_t s);
cudaError_t launch_batch(const BatchArgs& a, int grid, cudaStream_t s);
cudaError_t batch_occupancy(int* blocks_per_sm);
int batch_max_jobs();
// The fused sieve kernel: variant 3 (two candidates per thread) or 5 (four), the walk
// step, and blocks of `threads` = 256 or 128 threads.
cudaError_t launch_sieve(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s, int variant,
                         int walk, int threads = 256);
cudaError_t launch_sieve_pair(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s, int walk,
                              int threads);
cudaError_t launch_sieve_quad(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s, int walk,
                              int threads);
cudaError_t sieve_pair_occupancy(int* blocks_per_sm, int threads);
cudaError_t sieve_quad_occupancy(int* blocks_per_sm, int threads);
// The walk step valid for every p in [plo, phi) with multipliers up to kmax.
int walk_for_range(uint64_t plo, uint64_t phi, uint32_t kmax);
// 1 when every odd p in [plo, phi) has the form 2^63 + d with 0 < d < 2^30
// (the setup's folding product applies), else 0.
int pm_setup_for_range(uint64_t plo, uint64_t phi);
cudaError_t launch_setup_partial(const SieveArgs& a, int grid_x, int nchunks, cudaStream_t s);
cudaError_t launch_table_check(const TableCheckArgs& a, int grid, cudaStream_t s);
cudaError_t launch_imad_bench(u32 iters, u32 kind, u32 seed, u32* sink, int grid, cudaStream_t s);
double bench_units_per_thread_iter(u32 kind);
cudaError_t sieve_occupancy(int* blocks_per_sm, int variant, int threads = 256);
int sieve_threads();
int gen_threads();

}  // namespace fs
