// fs_noalloc.cu -- a segment search that allocates no device memory.
//
// fs_segment_noalloc() runs the same kernels as fs_search_segment()
// (candidate generation, then setup/iterate/check fused) for callers that
// cannot call cudaMalloc: code that runs while a CUDA stream is being
// captured, memory-budgeted services whose device memory is owned by a pool
// they must not bypass, and embedders that hand this library preallocated
// buffers only.  The caller passes every input and output as device memory it
// already owns; the only scratch -- the candidate list that connects the two
// kernels -- lives in the fixed array below, sized at compile time.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/factsieve.h"
#include "fs_launch.h"

namespace {

constexpr uint32_t kMaxCand = FS_NOALLOC_MAX_CANDIDATES;
constexpr u32 kQ[29] = {3,  5,  7,  11, 13, 17, 19, 23, 29,  31,  37,  41,  43,  47, 53,
                        59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};

// Candidate scratch shared by every call on a device (8 MiB per device that
// loads the library, held until the process exits).
static __device__ __align__(256) unsigned long long g_noalloc_cand[kMaxCand];

struct DeviceState {
    bool ready = false;
    u64* cand = nullptr;   // device address of g_noalloc_cand on this device
    int sm_count = 0;
    int occ3 = 1;          // resident blocks per SM of the two-candidate build
    int occ5 = 1;          // and of the four-candidate build
};

constexpr int kMaxDevices = 64;
std::mutex g_mu;
DeviceState g_dev[kMaxDevices];

// Once per device, with that device current: resolve the array's device
// address (the host-side symbol is only a stand-in) and the launch geometry.
int device_state(DeviceState** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FS_E_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceState& s = g_dev[dev];
    if (!s.ready) {
        void* ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_cand) != cudaSuccess || !ptr) return FS_E_CUDA;
        int sms = 0, occ3 = 0, occ5 = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FS_E_CUDA;
        if (fs::sieve_occupancy(&occ3, 3) != cudaSuccess || occ3 < 1) occ3 = 1;
        if (fs::sieve_occupancy(&occ5, 5) != cudaSuccess || occ5 < 1) occ5 = 1;
        s.cand = (u64*)ptr;
        s.sm_count = sms;
        s.occ3 = occ3;
        s.occ5 = occ5;
        s.ready = true;
    }
    *out = &s;
    return FS_OK;
}

}  // namespace

extern "C" int fs_segment_noalloc(uint64_t low, uint64_t high, uint32_t nmin, uint32_t nmax,
                                  const uint64_t* d_words, const uint32_t* d_layers4, uint32_t nlayers,
                                  uint64_t deficit, fs_factor* d_hits, uint32_t hitcap, fs_counters* d_ctr,
                                  void* stream) {
    if (!d_ctr || (hitcap && !d_hits) || (nlayers && (!d_words || !d_layers4))) return FS_E_ARG;
    // the range checks of a search (setupSearch, cl_sieve.cpp:561-589): n from 1, p not below nmin
    if (nmin == 0 || nmin > nmax || nmax > 0x7FFFFFFFu || low < 3 || low < nmin) return FS_E_ARG;
    if (high <= low) return FS_OK;
    if (fs_candidate_capacity(low, high) > kMaxCand) return FS_E_LIMIT;
    DeviceState* ds = nullptr;
    int rc = device_state(&ds);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    fs::Counters* ctr = (fs::Counters*)d_ctr;
    // the candidate count must start at zero; the array itself is overwritten
    if (cudaMemsetAsync(&ctr->ncand, 0, sizeof(u32), s) != cudaSuccess) return FS_E_CUDA;

    const uint64_t o0 = low | 1ull;
    if (o0 < high) {
        fs::GenArgs g = {};
        g.o0 = o0;
        g.high = high;
        g.nwords = (high - o0 + 63) / 64;
        for (int j = 0; j < 29; ++j) g.r0[j] = (u32)(o0 % kQ[j]);
        g.cap = kMaxCand;
        g.cand = ds->cand;
        g.ctr = ctr;
        const uint64_t blocks = (g.nwords + fs::gen_threads() - 1) / fs::gen_threads();
        const uint64_t maxb = (uint64_t)ds->sm_count * 8;
        if (fs::launch_gen(g, (int)(blocks < maxb ? (blocks ? blocks : 1) : maxb), s) != cudaSuccess)
            return FS_E_CUDA;
    }
    fs::SieveArgs a = {};
    a.cand = ds->cand;
    a.ncand = &ctr->ncand;
    a.cap = kMaxCand;
    a.plan.words = (const u64*)d_words;
    a.plan.layers = (const fs::Layer*)d_layers4;
    a.plan.layer_begin = 0;
    a.plan.layer_end = nlayers;
    a.plan.deficit = deficit;
    a.nchunks = 1;
    a.nstart = nmin;
    a.nend = nmax;
    a.nmax = nmax;
    a.count_candidates = 1;
    a.hits = (fs::Factor*)d_hits;
    a.hitcap = hitcap;
    a.ctr = ctr;
    // The launch fs_search_segment would make for this segment: the walk step
    // proven for the whole p-range with the four-candidate build (four times
    // its resident blocks per SM, so the last wave is short), folded setup
    // products just above 2^63, or each candidate's own step with the
    // two-candidate build when no one step covers the range.
    const int walk = fs::walk_for_range(low, high, nmax);
    const int kv = walk == fs::WALK_ANY ? 3 : 5;
    int smode = fs::SETUP_PLAN;
    if (kv == 5 && (walk == fs::WALK_C96H || walk == fs::WALK_C96G || walk == fs::WALK_C96) &&
        fs::pm_setup_for_range(low, high))
        smode = fs::SETUP_PLAN_PM;
    const int grid = ds->sm_count * (kv == 5 ? 4 * ds->occ5 : ds->occ3);
    if (fs::launch_sieve(a, smode, true, grid, s, kv, walk) != cudaSuccess) return FS_E_CUDA;
    return FS_OK;
}
