// fs_internal.h -- the library context shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/factsieve.h"
#include "fs_host.h"
#include "fs_launch.h"

namespace fs_internal {

struct PlanGPU {
    uint32_t n = 0, nchunks = 0;
    u64* d_words = nullptr;
    fs::Layer* d_layers = nullptr;
    fs::PlanChunkDev* d_chunks = nullptr;
    uint64_t deficit = 0, nwords = 0;
    uint32_t nlayers = 0;
    std::vector<fs::PlanChunkDev> chunks;
};

}  // namespace fs_internal

namespace fs_serve { struct Server; }

struct fs_ctx {
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    int sm_count = 0, clock_khz = 0;
    uint64_t total_mem = 0;
    int sieve_occ[7] = {1, 1, 1, 1, 1, 1, 1};      // resident 256-thread sieve blocks per SM, by build
    int sieve_occ128[7] = {2, 2, 2, 2, 2, 2, 2};   // and 128-thread ones
    fs_tuning tuning{};
    std::string err;
    // search state
    bool active = false, table_checked = false;
    uint64_t pmin = 0, pmax = 0;
    uint32_t nmin = 0, nmax = 0;
    fs::Counters* d_ctr = nullptr;
    u64* d_cand = nullptr;
    uint64_t cand_cap = 0;
    u64* d_residue = nullptr;
    uint64_t residue_cap = 0;
    u64* d_partials = nullptr;
    uint64_t partials_cap = 0;
    fs::Factor* d_hits = nullptr;
    uint32_t hit_cap = 0;
    u64* d_chk_scratch = nullptr;
    u32* d_chk_done = nullptr;
    u64* d_chk_result = nullptr;
    fs::PlanChunkDev* d_chk_chunk = nullptr;
    int chk_grid = 0;
    u32* d_sink = nullptr;
    std::map<std::pair<uint32_t, uint32_t>, fs_internal::PlanGPU> plans;
    // batch
    struct Batch {
        bool ready = false;
        uint32_t njobs = 0;
        std::vector<uint32_t> order;        // device slot k runs caller job order[k]
        std::vector<uint64_t> cap;          // candidate capacity per slot
        u64* d_cand = nullptr;
        u64* d_words = nullptr;
        fs::Layer* d_layers = nullptr;
        fs::BatchJob* d_jobs = nullptr;
        fs::Counters* d_ctr = nullptr;      // per slot
        fs::Counters* d_gctr = nullptr;     // batch-wide
        u32* d_tile = nullptr;
        fs::Factor* d_hits = nullptr;
        uint32_t hitcap = 0;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
    } batch;
    uint64_t batch_launches = 0;
    double batch_ms = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> batch_ev;
    // statistics
    bool timing = false;
    uint64_t launches = 0, sieve_launches = 0, gen_launches = 0;
    double sieve_ms = 0, gen_ms = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> sieve_ev, gen_ev, ev_pool;
    fs_serve::Server* server = nullptr;
};

#define CK(ctx, call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);   \
            return e_ == cudaErrorMemoryAllocation ? FS_E_NOMEM : FS_E_CUDA;   \
        }                                                                      \
    } while (0)


namespace fs_internal {
int bind(fs_ctx* c);
int run_gen(fs_ctx* c, uint64_t low, uint64_t high, u64* d_cand, uint32_t cap, fs::Counters* d_ctr);
}  // namespace fs_internal
