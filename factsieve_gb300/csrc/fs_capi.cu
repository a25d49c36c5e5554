// fs_capi.cu -- the C ABI of libfactsieve.so (declared in include/factsieve.h).
//
// Owns device memory, streams and the per-n setup plans, and sequences the
// kernels of one p-segment the way the reference's cl_sieve() loop does
// (cl_sieve.cpp:1107-1241): candidates -> (first segment) table check ->
// setup -> iterate -> check.  Nothing here calls exit(); every failure is a
// status code, and the text of the last CUDA error stays on the context.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/factsieve.h"
#include "fs_host.h"
#include "fs_internal.h"
#include "fs_launch.h"

static_assert(sizeof(fs_factor) == 16, "factor record is 16 bytes");
static_assert(sizeof(fs_factor) == sizeof(fs::Factor), "factor layouts agree");
static_assert(sizeof(fs_counters) == sizeof(fs::Counters), "counter layouts agree");

namespace {

constexpr u32 kQ[29] = {3,  5,  7,  11, 13, 17, 19, 23, 29,  31,  37,  41,  43,  47, 53,
                        59, 61, 67, 71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113};

using fs_internal::PlanGPU;

}  // namespace

namespace fs_internal {

int bind(fs_ctx* c) {
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) {
        c->err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return FS_E_CUDA;
    }
    return FS_OK;
}

}  // namespace fs_internal

namespace {

using fs_internal::bind;

// A pair of events around one launch when timing is on.
int ev_begin(fs_ctx* c, std::pair<cudaEvent_t, cudaEvent_t>* ev) {
    if (!c->timing) return FS_OK;
    if (!c->ev_pool.empty()) {
        *ev = c->ev_pool.back();
        c->ev_pool.pop_back();
    } else {
        CK(c, cudaEventCreate(&ev->first));
        CK(c, cudaEventCreate(&ev->second));
    }
    CK(c, cudaEventRecord(ev->first, c->stream));
    return FS_OK;
}

int ev_end(fs_ctx* c, std::pair<cudaEvent_t, cudaEvent_t>& ev, std::vector<std::pair<cudaEvent_t, cudaEvent_t>>& list) {
    if (!c->timing) return FS_OK;
    CK(c, cudaEventRecord(ev.second, c->stream));
    list.push_back(ev);
    return FS_OK;
}

int ev_drain(fs_ctx* c) {
    for (int k = 0; k < 3; ++k) {
        auto& list = k == 2 ? c->batch_ev : k ? c->gen_ev : c->sieve_ev;
        for (auto& ev : list) {
            CK(c, cudaEventSynchronize(ev.second));
            float ms = 0;
            CK(c, cudaEventElapsedTime(&ms, ev.first, ev.second));
            (k == 2 ? c->batch_ms : k ? c->gen_ms : c->sieve_ms) += ms;
            c->ev_pool.push_back(ev);
        }
        list.clear();
    }
    return FS_OK;
}

template <class T>
int grow(fs_ctx* c, T** ptr, uint64_t* have, uint64_t need) {
    if (*have >= need && *ptr) return FS_OK;
    if (*ptr) {
        CK(c, cudaStreamSynchronize(c->stream));
        CK(c, cudaFree(*ptr));
        *ptr = nullptr;
        *have = 0;
    }
    CK(c, cudaMalloc((void**)ptr, need * sizeof(T)));
    *have = need;
    return FS_OK;
}

void free_plans(fs_ctx* c) {
    for (auto& kv : c->plans) {
        cudaFree(kv.second.d_words);
        cudaFree(kv.second.d_layers);
        cudaFree(kv.second.d_chunks);
    }
    c->plans.clear();
}

int get_plan(fs_ctx* c, uint32_t n, uint32_t chunks, PlanGPU** out) {
    auto key = std::make_pair(n, chunks);
    auto it = c->plans.find(key);
    if (it != c->plans.end()) {
        *out = &it->second;
        return FS_OK;
    }
    fs::SetupPlan hp = fs::build_plan(n, chunks);
    PlanGPU g;
    g.n = n;
    g.nchunks = chunks;
    g.deficit = hp.deficit;
    g.nwords = hp.words.size();
    g.nlayers = (uint32_t)hp.layers.size();
    for (auto& ch : hp.chunks) g.chunks.push_back({ch.layer_begin, ch.layer_end, ch.deficit});
    // +2 words of padding keep the paired 16-byte loads inside the buffer
    size_t wbytes = (hp.words.size() + 2) * sizeof(u64);
    CK(c, cudaMalloc((void**)&g.d_words, wbytes));
    CK(c, cudaMalloc((void**)&g.d_layers, (hp.layers.size() + 1) * sizeof(fs::Layer)));
    CK(c, cudaMalloc((void**)&g.d_chunks, (g.chunks.size() + 1) * sizeof(fs::PlanChunkDev)));
    CK(c, cudaMemsetAsync(g.d_words, 0, wbytes, c->stream));
    if (!hp.words.empty())
        CK(c, cudaMemcpyAsync(g.d_words, hp.words.data(), hp.words.size() * sizeof(u64),
                              cudaMemcpyHostToDevice, c->stream));
    if (!hp.layers.empty())
        CK(c, cudaMemcpyAsync(g.d_layers, hp.layers.data(), hp.layers.size() * sizeof(fs::Layer),
                              cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(g.d_chunks, g.chunks.data(), g.chunks.size() * sizeof(fs::PlanChunkDev),
                          cudaMemcpyHostToDevice, c->stream));
    // the host vectors die here: wait for the copies
    CK(c, cudaStreamSynchronize(c->stream));
    auto ins = c->plans.emplace(key, std::move(g));
    *out = &ins.first->second;
    return FS_OK;
}

fs::SieveArgs base_args(PlanGPU* pl) {
    fs::SieveArgs a;
    memset(&a, 0, sizeof(a));
    if (pl) {
        a.plan.words = pl->d_words;
        a.plan.layers = pl->d_layers;
        a.plan.layer_begin = 0;
        a.plan.layer_end = pl->nlayers;
        a.plan.deficit = pl->deficit;
        a.chunks = pl->d_chunks;
        a.nchunks = pl->nchunks;
    }
    return a;
}

// Sieve kernel build (fs_tuning.sieve_variant): 3 two candidates per thread
// at 3 resident blocks per SM, 5 four candidates per thread at 2.  The
// default is 5, which the measurements favour on every segment whose
// candidates share one walk step (the usual case).
int variant(fs_ctx* c) { return c->tuning.sieve_variant == 3 ? 3 : 5; }

// The build a launch really runs: the four-candidate kernels exist for the
// launch-wide walks only; a mixed segment (WALK_ANY) runs variant 3.
int kernel_variant(int v, int walk) { return (v == 5 && walk == fs::WALK_ANY) ? 3 : v; }

// Threads per sieve block (fs_tuning.sieve_block_threads): 256 or 128.
int block_threads(fs_ctx* c) { return c->tuning.sieve_block_threads == 128 ? 128 : 256; }

// Default blocks per SM for a build: its resident occupancy at the block
// size, and for the four-candidate build four times that, so the candidates
// are dealt in smaller shares and the last wave is short.
int default_bpsm(fs_ctx* c, int kv) {
    const int occ = block_threads(c) == 128 ? c->sieve_occ128[kv] : c->sieve_occ[kv];
    return occ * (kv == 5 ? 4 : 1);
}

// The build for launches that walk each candidate with its own step.
int any_variant(fs_ctx* c) { return kernel_variant(variant(c), fs::WALK_ANY); }

int sieve_grid(fs_ctx* c, int kv) {
    const int bpsm = c->tuning.sieve_blocks_per_sm ? (int)c->tuning.sieve_blocks_per_sm : default_bpsm(c, kv);
    return std::max(1, c->sm_count * bpsm);
}

// How many threads should share one prime's setup: enough to fill the GPU
// when the candidates alone cannot, and only when the table is long.
uint32_t auto_chunks(fs_ctx* c, uint64_t est_cand, uint32_t n) {
    if (c->tuning.setup_chunks) return c->tuning.setup_chunks;
    const uint64_t slots = (uint64_t)c->sm_count * 2048;
    const double words = 0.03 * n;   // bit-layered table length, about 0.03 n words
    if (words < 8192 || est_cand * 2 >= slots) return 1;
    uint64_t k = slots / std::max<uint64_t>(est_cand, 1);
    k = std::min<uint64_t>(k, (uint64_t)(words / 2048));
    return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(k, 64));
}

}  // namespace

int fs_internal::run_gen(fs_ctx* c, uint64_t low, uint64_t high, u64* d_cand, uint32_t cap, fs::Counters* d_ctr) {
    if (high <= low) return FS_OK;
    uint64_t o0 = low | 1ull;
    if (o0 < low || o0 >= high) return FS_OK;
    fs::GenArgs g;
    memset(&g, 0, sizeof(g));
    g.o0 = o0;
    g.high = high;
    g.nwords = (high - o0 + 63) / 64;
    if (g.nwords >= (1ull << 31)) {
        c->err = "segment too wide for one candidate launch";
        return FS_E_ARG;
    }
    for (int j = 0; j < 29; ++j) g.r0[j] = (u32)(o0 % kQ[j]);
    g.cap = cap;
    g.cand = d_cand;
    g.ctr = d_ctr;
    const int threads = fs::gen_threads();
    uint64_t blocks = (g.nwords + threads - 1) / threads;
    uint64_t maxb = (uint64_t)c->sm_count * (c->tuning.gen_blocks_per_sm ? c->tuning.gen_blocks_per_sm : 8);
    std::pair<cudaEvent_t, cudaEvent_t> ev;
    int rc = ev_begin(c, &ev);
    if (rc) return rc;
    CK(c, fs::launch_gen(g, (int)std::max<uint64_t>(1, std::min(blocks, maxb)), c->stream));
    ++c->launches;
    ++c->gen_launches;
    return ev_end(c, ev, c->gen_ev);
}

namespace {

using fs_internal::run_gen;

// Per-block partial products, the completion counter and the result of the
// table check, allocated on first use.
int ensure_check_buffers(fs_ctx* c) {
    if (!c->d_chk_scratch) {
        c->chk_grid = c->sm_count * 4;
        CK(c, cudaMalloc((void**)&c->d_chk_scratch, c->chk_grid * sizeof(u64)));
        CK(c, cudaMalloc((void**)&c->d_chk_done, sizeof(u32)));
        CK(c, cudaMalloc((void**)&c->d_chk_result, 2 * sizeof(u64)));
        CK(c, cudaMalloc((void**)&c->d_chk_chunk, sizeof(fs::PlanChunkDev)));
        CK(c, cudaMemsetAsync(c->d_chk_done, 0, sizeof(u32), c->stream));
    }
    return FS_OK;
}

int run_table_check_raw(fs_ctx* c, const u64* d_cand, fs::Counters* d_ctr, uint32_t n, const u64* words,
                        const fs::Layer* layers, const fs::PlanChunkDev* chunks, uint32_t nchunks,
                        uint64_t deficit) {
    int rc = ensure_check_buffers(c);
    if (rc) return rc;
    fs::TableCheckArgs t;
    memset(&t, 0, sizeof(t));
    t.cand = d_cand;
    t.ncand = &d_ctr->ncand;
    t.n0 = n;
    t.words = words;
    t.layers = layers;
    t.chunks = chunks;
    t.nchunks = nchunks;
    t.deficit = deficit;
    t.scratch = c->d_chk_scratch;
    t.done = c->d_chk_done;
    t.result = c->d_chk_result;
    t.ctr = d_ctr;
    CK(c, cudaMemsetAsync(c->d_chk_result, 0, 2 * sizeof(u64), c->stream));
    CK(c, fs::launch_table_check(t, c->chk_grid, c->stream));
    ++c->launches;
    return FS_OK;
}

int run_table_check(fs_ctx* c, const u64* d_cand, fs::Counters* d_ctr, uint32_t n, PlanGPU* pl) {
    return run_table_check_raw(c, d_cand, d_ctr, n, pl->d_words, pl->d_layers, pl->d_chunks, pl->nchunks,
                               pl->deficit);
}

// setup + iterate + check of the candidates in d_cand over [nstart, nend),
// finishing with s7 = nmax R when final.  Splits the n-range into launches
// of at most tuning.max_steps_per_launch steps, and the table across
// threads when auto_chunks() says so.
int run_sieve(fs_ctx* c, const u64* d_cand, uint32_t cap, fs::Counters* d_ctr, uint32_t nstart,
              uint32_t nend, uint32_t nmax, bool count, uint64_t est_cand, fs::Factor* d_hits,
              uint32_t hitcap, uint64_t plo, uint64_t phi) {
    uint32_t chunks = auto_chunks(c, est_cand, nstart);
    PlanGPU* pl = nullptr;
    int rc = get_plan(c, nstart, chunks, &pl);
    if (rc) return rc;
    const uint32_t span = nend > nstart ? nend - nstart : 0;
    const uint32_t maxs = c->tuning.max_steps_per_launch;
    const bool split = maxs && span > maxs;
    if (split) {
        if ((rc = grow(c, &c->d_residue, &c->residue_cap, FS_WALK_STATE_WORDS(cap)))) return rc;
    }
    fs::SieveArgs a = base_args(pl);
    a.cand = d_cand;
    a.ncand = &d_ctr->ncand;
    a.cap = cap;
    a.hits = d_hits;
    a.hitcap = hitcap;
    a.ctr = d_ctr;
    a.nmax = nmax;
    int setup_mode = fs::SETUP_PLAN;
    if (chunks > 1) {
        if ((rc = grow(c, &c->d_partials, &c->partials_cap, (uint64_t)cap * chunks + 1))) return rc;
        a.partials = c->d_partials;
        int gx = std::max(1, sieve_grid(c, any_variant(c)) / (int)chunks);
        std::pair<cudaEvent_t, cudaEvent_t> ev;
        if ((rc = ev_begin(c, &ev))) return rc;
        CK(c, fs::launch_setup_partial(a, gx, (int)chunks, c->stream));
        if ((rc = ev_end(c, ev, c->sieve_ev))) return rc;
        ++c->launches;
        ++c->sieve_launches;
        setup_mode = fs::SETUP_PARTIALS;
    }
    uint32_t s = nstart;
    bool first = true;
    do {
        uint32_t e = split ? std::min<uint64_t>((uint64_t)s + maxs, nend) : nend;
        const int walk = fs::walk_for_range(plo, phi, e);
        const bool fin = (e == nend);
        a.nstart = s;
        a.nend = e;
        // split launches carry residues and the n each stands at (its tag) from one launch to the next
        a.residue = split ? c->d_residue : nullptr;
        a.walked = split ? (u32*)(c->d_residue + cap) : nullptr;
        a.count_candidates = (fin && count) ? 1u : 0u;
        std::pair<cudaEvent_t, cudaEvent_t> ev;
        if ((rc = ev_begin(c, &ev))) return rc;
        const int kv = kernel_variant(variant(c), walk);
        int smode = first ? setup_mode : fs::SETUP_LOAD;
        // p = 2^63 + d, d < 2^30 over the segment: the four-candidate kernels of
        // the 96-bit walks fold their setup products instead of Montgomery's
        if (smode == fs::SETUP_PLAN && kv == 5 &&
            (walk == fs::WALK_C96H || walk == fs::WALK_C96G || walk == fs::WALK_C96) &&
            fs::pm_setup_for_range(plo, phi))
            smode = fs::SETUP_PLAN_PM;
        CK(c, fs::launch_sieve(a, smode, fin, sieve_grid(c, kv), c->stream, kv, walk, block_threads(c)));
        if ((rc = ev_end(c, ev, c->sieve_ev))) return rc;
        ++c->launches;
        ++c->sieve_launches;
        first = false;
        s = e;
    } while (s < nend);
    return FS_OK;
}

uint64_t est_candidates(uint64_t low, uint64_t high) {
    if (high <= low) return 0;
    double w = (double)(high - low);
    double lx = std::log(std::max<double>((double)low, 3.0));
    return (uint64_t)(w / lx * 1.05) + 16;
}

}  // namespace

// =================================================================== ABI ===

extern "C" {

int fs_version(void) { return 10000; }

const char* fs_strerror(int code) {
    switch (code) {
        case FS_OK: return "ok";
        case FS_E_ARG: return "invalid argument";
        case FS_E_CUDA: return "CUDA error";
        case FS_E_OVERFLOW: return "candidate or factor buffer overflow";
        case FS_E_VALIDATION: return "gpu validation failure";
        case FS_E_TABLE: return "power table verification failed";
        case FS_E_NOMEM: return "out of memory";
        case FS_E_VERIFY: return "CPU factor verification failed";
        case FS_E_STATE: return "call out of order";
        case FS_E_LIMIT: return "request exceeds a fixed size limit";
        default: return "unknown error";
    }
}

const char* fs_last_error(fs_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

int fs_device_count(int* count) {
    if (!count) return FS_E_ARG;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        *count = 0;
        return FS_E_CUDA;
    }
    *count = n;
    return FS_OK;
}

int fs_create(int device, fs_ctx** out) {
    if (!out) return FS_E_ARG;
    *out = nullptr;
    fs_ctx* c = new fs_ctx();
    c->device = device;
    int rc = bind(c);
    if (rc) {
        delete c;
        return rc;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return FS_E_CUDA;
    }
    c->stream = c->own;
    c->sm_count = prop.multiProcessorCount;
    int clk = 0;
    cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
    c->clock_khz = clk;
    c->total_mem = prop.totalGlobalMem;
    for (int v : {3, 5}) {
        int occ = 0;
        if (fs::sieve_occupancy(&occ, v) == cudaSuccess && occ > 0) c->sieve_occ[v] = occ;
        occ = 0;
        if (fs::sieve_occupancy(&occ, v, 128) == cudaSuccess && occ > 0) c->sieve_occ128[v] = occ;
    }
    if (cudaMalloc((void**)&c->d_ctr, sizeof(fs::Counters)) != cudaSuccess ||
        cudaMalloc((void**)&c->d_sink, 4096 * sizeof(u32)) != cudaSuccess) {
        cudaStreamDestroy(c->own);
        delete c;
        return FS_E_NOMEM;
    }
    cudaMemset(c->d_ctr, 0, sizeof(fs::Counters));
    *out = c;
    return FS_OK;
}

int fs_destroy(fs_ctx* c) {
    if (!c) return FS_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_plans(c);
    cudaFree(c->d_ctr);
    cudaFree(c->d_cand);
    cudaFree(c->d_residue);
    cudaFree(c->d_partials);
    cudaFree(c->d_hits);
    cudaFree(c->d_chk_scratch);
    cudaFree(c->d_chk_done);
    cudaFree(c->d_chk_result);
    cudaFree(c->d_chk_chunk);
    cudaFree(c->d_sink);
    fs_batch_release(c);
    fs_serve_destroy(c);
    for (auto* l : {&c->sieve_ev, &c->gen_ev, &c->batch_ev, &c->ev_pool})
        for (auto& ev : *l) {
            cudaEventDestroy(ev.first);
            cudaEventDestroy(ev.second);
        }
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
    return FS_OK;
}

int fs_set_timing(fs_ctx* c, int enable) {
    if (!c) return FS_E_ARG;
    c->timing = enable != 0;
    return FS_OK;
}

int fs_get_stats(fs_ctx* c, fs_stats* out) {
    if (!c || !out) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    if ((rc = ev_drain(c))) return rc;
    out->launches = c->launches;
    out->sieve_launches = c->sieve_launches;
    out->gen_launches = c->gen_launches;
    out->sieve_ms = c->sieve_ms;
    out->gen_ms = c->gen_ms;
    out->batch_launches = c->batch_launches;
    out->batch_ms = c->batch_ms;
    return FS_OK;
}

int fs_reset_stats(fs_ctx* c) {
    if (!c) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    if ((rc = ev_drain(c))) return rc;
    c->launches = c->sieve_launches = c->gen_launches = c->batch_launches = 0;
    c->sieve_ms = c->gen_ms = c->batch_ms = 0;
    return FS_OK;
}

int fs_set_stream(fs_ctx* c, void* stream) {
    if (!c) return FS_E_ARG;
    c->stream = stream ? (cudaStream_t)stream : c->own;
    return FS_OK;
}

void* fs_get_stream(fs_ctx* c) { return c ? (void*)c->stream : nullptr; }

int fs_set_tuning(fs_ctx* c, const fs_tuning* t) {
    if (!c || !t) return FS_E_ARG;
    if ((t->sieve_variant && t->sieve_variant != 3 && t->sieve_variant != 5) ||
        (t->sieve_block_threads && t->sieve_block_threads != 128 && t->sieve_block_threads != 256) ||
        (t->batch_tile_candidates && t->batch_tile_candidates != 1024 && t->batch_tile_candidates != 2048 &&
         t->batch_tile_candidates != 4096)) {
        c->err = "unsupported tuning value";
        return FS_E_ARG;
    }
    c->tuning = *t;
    return FS_OK;
}

int fs_get_tuning(fs_ctx* c, fs_tuning* t) {
    if (!c || !t) return FS_E_ARG;
    *t = c->tuning;
    if (!t->sieve_variant) t->sieve_variant = (uint32_t)variant(c);
    if (!t->sieve_blocks_per_sm) t->sieve_blocks_per_sm = (uint32_t)default_bpsm(c, variant(c));
    if (!t->sieve_block_threads) t->sieve_block_threads = (uint32_t)block_threads(c);
    if (!t->batch_tile_candidates) t->batch_tile_candidates = fs::kTileCandidates;
    return FS_OK;
}

int fs_device_info(fs_ctx* c, int* sm_count, int* clock_khz, uint64_t* total_mem) {
    if (!c) return FS_E_ARG;
    if (sm_count) *sm_count = c->sm_count;
    if (clock_khz) *clock_khz = c->clock_khz;
    if (total_mem) *total_mem = c->total_mem;
    return FS_OK;
}

int fs_synchronize(fs_ctx* c) {
    if (!c) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    CK(c, cudaStreamSynchronize(c->stream));
    return FS_OK;
}

uint64_t fs_candidate_capacity(uint64_t low, uint64_t high) {
    if (high <= low) return 1024;
    const double w = (double)(high - low);
    // Brun-Titchmarsh in the Montgomery-Vaughan form: an interval of length
    // w > 1 holds at most 2w/ln w primes; base-2 strong pseudoprimes with no
    // factor <= 113 are far rarer than the 1024-slot margin.
    double bound = w > 2.0 ? 2.0 * w / std::log(w) : w + 1;
    double wheel = 8.0 * std::ceil(w / 30.0) + 16;   // numbers coprime to 30
    double cap = std::min(bound, wheel) * 1.02 + 1024;
    return (uint64_t)std::min(cap, 4.0e9);
}

int fs_search_begin(fs_ctx* c, uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax,
                    uint32_t result_cap) {
    if (!c) return FS_E_ARG;
    // setupSearch's checks (cl_sieve.cpp:561-589)
    if (pmin == 0 || pmax == 0 || nmin == 0 || nmax == 0 || nmin > nmax || pmin > pmax || pmin < nmin) {
        c->err = "invalid search range";
        return FS_E_ARG;
    }
    int rc = bind(c);
    if (rc) return rc;
    c->pmin = pmin;
    c->pmax = pmax;
    c->nmin = nmin;
    c->nmax = nmax;
    c->active = true;
    c->table_checked = false;
    // a search builds and uploads its own power table (cl_sieve.cpp:1159)
    CK(c, cudaStreamSynchronize(c->stream));
    free_plans(c);
    uint32_t cap = result_cap ? result_cap : (pmin < 0xFFFFFFFFull ? 30000000u : 1000000u);
    uint64_t have = c->hit_cap;
    if ((rc = grow(c, &c->d_hits, &have, cap))) return rc;
    c->hit_cap = cap;
    CK(c, cudaMemsetAsync(c->d_ctr, 0, sizeof(fs::Counters), c->stream));
    return FS_OK;
}

int fs_search_segment(fs_ctx* c, uint64_t low, uint64_t high) {
    if (!c) return FS_E_ARG;
    if (!c->active) return FS_E_STATE;
    int rc = bind(c);
    if (rc) return rc;
    if (high <= low) return FS_OK;
    uint64_t cap64 = fs_candidate_capacity(low, high);
    if (cap64 >= 0xFFFFFFF0ull) {
        c->err = "segment too wide";
        return FS_E_ARG;
    }
    const uint32_t cap = (uint32_t)cap64;
    if ((rc = grow(c, &c->d_cand, &c->cand_cap, cap64))) return rc;
    CK(c, cudaMemsetAsync(&c->d_ctr->ncand, 0, sizeof(u32), c->stream));
    if ((rc = run_gen(c, low, high, c->d_cand, cap, c->d_ctr))) return rc;
    if (!c->table_checked) {
        PlanGPU* pl = nullptr;
        if ((rc = get_plan(c, c->nmin, 1, &pl))) return rc;
        if ((rc = run_table_check(c, c->d_cand, c->d_ctr, c->nmin, pl))) return rc;
        c->table_checked = true;
    }
    return run_sieve(c, c->d_cand, cap, c->d_ctr, c->nmin, c->nmax, c->nmax, true,
                     est_candidates(low, high), c->d_hits, c->hit_cap, low, high);
}

int fs_search_range(fs_ctx* c, uint64_t low, uint64_t high, uint64_t seg_width) {
    if (!c) return FS_E_ARG;
    if (!seg_width) seg_width = 1000000000ull;
    for (uint64_t lo = low; lo < high;) {
        uint64_t hi = lo + seg_width;
        if (hi > high || hi < lo) hi = high;
        int rc = fs_search_segment(c, lo, hi);
        if (rc) return rc;
        lo = hi;
    }
    return FS_OK;
}

int fs_search_collect(fs_ctx* c, fs_factor* out, uint64_t cap, uint64_t* nfactors, uint64_t* raw_sum,
                      uint64_t* primecount, uint32_t* flags) {
    if (!c) return FS_E_ARG;
    if (!c->active) return FS_E_STATE;
    int rc = bind(c);
    if (rc) return rc;
    fs::Counters h;
    CK(c, cudaMemcpyAsync(&h, c->d_ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    uint64_t nh = std::min<uint64_t>(h.nhits, c->hit_cap);
    if (nfactors) *nfactors = h.nhits;
    if (raw_sum) *raw_sum = h.raw_sum;
    if (primecount) *primecount = h.primecount;
    if (flags) *flags = h.flags;
    uint64_t ncopy = std::min<uint64_t>(nh, out ? cap : 0);
    if (ncopy)
        CK(c, cudaMemcpy(out, c->d_hits, ncopy * sizeof(fs_factor), cudaMemcpyDeviceToHost));
    // clear sums, hits and flags for the next interval (clearresult.cl)
    CK(c, cudaMemsetAsync(c->d_ctr, 0, offsetof(fs::Counters, ncand), c->stream));
    CK(c, cudaMemsetAsync(&c->d_ctr->nhits, 0, 2 * sizeof(u32), c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (h.flags & FS_FLAG_TABLE) return FS_E_TABLE;
    if (h.flags & FS_FLAG_VALIDATION) return FS_E_VALIDATION;
    if (h.flags & (FS_FLAG_CAND_OVERFLOW | FS_FLAG_HIT_OVERFLOW)) return FS_E_OVERFLOW;
    if (h.nhits > c->hit_cap || (out && h.nhits > cap)) return FS_E_OVERFLOW;
    return FS_OK;
}

int fs_search_pending(fs_ctx* c, uint64_t* nfactors) {
    if (!c || !nfactors) return FS_E_ARG;
    if (!c->active) return FS_E_STATE;
    int rc = bind(c);
    if (rc) return rc;
    u32 n = 0;
    CK(c, cudaMemcpyAsync(&n, &c->d_ctr->nhits, sizeof(n), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    *nfactors = n;
    return FS_OK;
}

// ------------------------------------------------------------ stage-level --

int fs_getsegprimes(fs_ctx* c, uint64_t low, uint64_t high, uint64_t* d_cand, uint32_t cap,
                    fs_counters* d_ctr) {
    if (!c || !d_cand || !d_ctr) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    return run_gen(c, low, high, (u64*)d_cand, cap, (fs::Counters*)d_ctr);
}

int fs_setup(fs_ctx* c, const uint64_t* d_cand, uint32_t cap, fs_counters* d_ctr, uint32_t nstart,
             uint64_t* d_residue) {
    if (!c || !d_cand || !d_ctr || !d_residue) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    const uint32_t chunks = c->tuning.setup_chunks ? c->tuning.setup_chunks : 1;
    PlanGPU* pl = nullptr;
    if ((rc = get_plan(c, nstart, chunks, &pl))) return rc;
    fs::SieveArgs a = base_args(pl);
    a.cand = (const u64*)d_cand;
    a.ncand = &((fs::Counters*)d_ctr)->ncand;
    a.cap = cap;
    a.ctr = (fs::Counters*)d_ctr;
    a.residue = (u64*)d_residue;
    a.walked = (u32*)((u64*)d_residue + cap);
    a.nstart = a.nend = nstart;
    int mode = fs::SETUP_PLAN;
    if (chunks > 1) {
        if ((rc = grow(c, &c->d_partials, &c->partials_cap, (uint64_t)cap * chunks + 1))) return rc;
        a.partials = c->d_partials;
        CK(c, fs::launch_setup_partial(a, std::max(1, sieve_grid(c, any_variant(c)) / (int)chunks), (int)chunks, c->stream));
        mode = fs::SETUP_PARTIALS;
    }
    CK(c, fs::launch_sieve(a, mode, false, sieve_grid(c, any_variant(c)), c->stream, any_variant(c), fs::WALK_ANY,
                           block_threads(c)));
    return FS_OK;
}

int fs_iterate(fs_ctx* c, const uint64_t* d_cand, uint32_t cap, fs_counters* d_ctr, uint64_t* d_residue,
               uint32_t nstart, uint32_t nend, fs_factor* d_hits, uint32_t hitcap) {
    if (!c || !d_cand || !d_ctr || !d_residue || (!d_hits && hitcap)) return FS_E_ARG;
    if (nend > 0x7FFFFFFFu) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    fs::SieveArgs a = base_args(nullptr);
    a.cand = (const u64*)d_cand;
    a.ncand = &((fs::Counters*)d_ctr)->ncand;
    a.cap = cap;
    a.ctr = (fs::Counters*)d_ctr;
    a.residue = (u64*)d_residue;
    a.walked = (u32*)((u64*)d_residue + cap);
    a.hits = (fs::Factor*)d_hits;
    a.hitcap = hitcap;
    const uint32_t maxs = c->tuning.max_steps_per_launch;
    uint32_t s = nstart;
    do {
        uint32_t e = (maxs && nend - s > maxs) ? s + maxs : nend;
        a.nstart = s;
        a.nend = e;
        CK(c, fs::launch_sieve(a, fs::SETUP_LOAD, false, sieve_grid(c, any_variant(c)), c->stream, any_variant(c),
                               fs::WALK_ANY, block_threads(c)));
        s = e;
    } while (s < nend);
    return FS_OK;
}

int fs_check(fs_ctx* c, const uint64_t* d_cand, uint32_t cap, fs_counters* d_ctr, const uint64_t* d_residue,
             uint32_t nmax) {
    if (!c || !d_cand || !d_ctr || !d_residue) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    fs::SieveArgs a = base_args(nullptr);
    a.cand = (const u64*)d_cand;
    a.ncand = &((fs::Counters*)d_ctr)->ncand;
    a.cap = cap;
    a.ctr = (fs::Counters*)d_ctr;
    a.residue = (u64*)d_residue;
    a.walked = (u32*)((u64*)d_residue + cap);
    a.nstart = a.nend = nmax;
    a.nmax = nmax;
    a.count_candidates = 1;
    CK(c, fs::launch_sieve(a, fs::SETUP_LOAD, true, sieve_grid(c, any_variant(c)), c->stream, any_variant(c),
                           fs::WALK_ANY, block_threads(c)));
    return FS_OK;
}

int fs_table_check(fs_ctx* c, const uint64_t* d_cand, fs_counters* d_ctr, uint32_t nmin, uint64_t* out2) {
    if (!c || !d_cand || !d_ctr) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    const uint32_t chunks = c->tuning.setup_chunks ? c->tuning.setup_chunks : 1;
    PlanGPU* pl = nullptr;
    if ((rc = get_plan(c, nmin, chunks, &pl))) return rc;
    if ((rc = run_table_check(c, (const u64*)d_cand, (fs::Counters*)d_ctr, nmin, pl))) return rc;
    if (out2) {
        CK(c, cudaMemcpyAsync(out2, c->d_chk_result, 2 * sizeof(u64), cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
    }
    return FS_OK;
}

int fs_plan_check(fs_ctx* c, const uint64_t* d_cand, fs_counters* d_ctr, uint32_t nmin, const uint64_t* d_words,
                  const uint32_t* d_layers4, uint32_t nlayers, uint64_t deficit, uint64_t* out2) {
    if (!c || !d_cand || !d_ctr || (nlayers && (!d_words || !d_layers4))) return FS_E_ARG;
    int rc = bind(c);
    if (rc || (rc = ensure_check_buffers(c))) return rc;
    const fs::PlanChunkDev one{0, nlayers, deficit};
    CK(c, cudaMemcpyAsync(c->d_chk_chunk, &one, sizeof(one), cudaMemcpyHostToDevice, c->stream));
    if ((rc = run_table_check_raw(c, (const u64*)d_cand, (fs::Counters*)d_ctr, nmin, (const u64*)d_words,
                                  (const fs::Layer*)d_layers4, c->d_chk_chunk, 1, deficit)))
        return rc;
    if (out2) {
        CK(c, cudaMemcpyAsync(out2, c->d_chk_result, 2 * sizeof(u64), cudaMemcpyDeviceToHost, c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));   // `one` and out2 are host locals
    return FS_OK;
}

int fs_walk_step(uint64_t plo, uint64_t phi, uint32_t kmax) { return fs::walk_for_range(plo, phi, kmax); }
int fs_setup_form(uint64_t plo, uint64_t phi) { return fs::pm_setup_for_range(plo, phi); }

int fs_bench_int_pipe(fs_ctx* c, uint32_t kind, uint32_t iters, double* ops_per_sec, double* ms) {
    if (!c || kind > 19 || iters == 0 || iters > (1u << 24)) return FS_E_ARG;
    // kinds 16-19 walk multipliers up to 100001 + 8 iters, within their k_max bound
    if (kind >= 16 && 100001u + 8u * iters > 1276526u) return FS_E_ARG;
    int rc = bind(c);
    if (rc) return rc;
    const int grid = c->sm_count * 8;   // 8 x 256 threads = 2048 per SM
    cudaEvent_t e0, e1;
    CK(c, cudaEventCreate(&e0));
    CK(c, cudaEventCreate(&e1));
    CK(c, fs::launch_imad_bench(iters / 8 + 1, kind, 12345, c->d_sink, grid, c->stream));   // warm-up
    CK(c, cudaEventRecord(e0, c->stream));
    CK(c, fs::launch_imad_bench(iters, kind, 12345, c->d_sink, grid, c->stream));
    CK(c, cudaEventRecord(e1, c->stream));
    CK(c, cudaEventSynchronize(e1));
    float t = 0;
    CK(c, cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double ops = (double)grid * 256.0 * (double)iters * fs::bench_units_per_thread_iter(kind);
    if (ms) *ms = t;
    if (ops_per_sec) *ops_per_sec = t > 0 ? ops / (t * 1e-3) : 0;
    return FS_OK;
}

// ---------------------------------------------------------------- host ----

int fs_power_table(uint32_t n, uint64_t* prime, uint32_t* exp, uint32_t* bit, uint32_t cap, uint32_t* len) {
    fs::RefTable t = fs::reference_table(n);
    if (len) *len = (uint32_t)t.prime.size();
    if (t.prime.size() > cap) return FS_E_OVERFLOW;
    for (size_t i = 0; i < t.prime.size(); ++i) {
        if (prime) prime[i] = t.prime[i];
        if (exp) exp[i] = t.exp[i];
        if (bit) bit[i] = t.bit[i];
    }
    return FS_OK;
}

int fs_setup_plan(uint32_t n, uint32_t chunks, uint64_t* words, uint64_t wcap, uint64_t* nwords,
                  uint32_t* layers4, uint32_t lcap, uint32_t* nlayers, uint64_t* deficit) {
    fs::SetupPlan p = fs::build_plan(n, chunks ? chunks : 1);
    if (nwords) *nwords = p.words.size();
    if (nlayers) *nlayers = (uint32_t)p.layers.size();
    if (deficit) *deficit = p.deficit;
    if (p.words.size() > wcap || p.layers.size() > lcap) return (words || layers4) ? FS_E_OVERFLOW : FS_OK;
    if (words) std::copy(p.words.begin(), p.words.end(), words);
    if (layers4)
        for (size_t i = 0; i < p.layers.size(); ++i) {
            layers4[4 * i] = p.layers[i].begin;
            layers4[4 * i + 1] = p.layers[i].end;
            layers4[4 * i + 2] = p.layers[i].dbl;
            layers4[4 * i + 3] = 0;
        }
    return FS_OK;
}

int fs_setup_plan_chunks(uint32_t n, uint32_t chunks, uint32_t* bounds, uint64_t* deficits) {
    if (!bounds || !deficits) return FS_E_ARG;
    fs::SetupPlan p = fs::build_plan(n, chunks ? chunks : 1);
    for (size_t i = 0; i < p.chunks.size(); ++i) {
        bounds[i] = p.chunks[i].layer_begin;
        deficits[i] = p.chunks[i].deficit;
    }
    bounds[p.chunks.size()] = p.chunks.empty() ? 0 : p.chunks.back().layer_end;
    return FS_OK;
}

int fs_find_wheel_offset(uint64_t* start, int32_t* index) {
    if (!start || !index) return FS_E_ARG;
    // residues coprime to 30 in wheel order; the gap from res[i] to the next
    // one is the i-th entry of the mod-30 gap table {4,2,4,2,4,6,2,6}
    static const int res[8] = {7, 11, 13, 17, 19, 23, 29, 1};
    uint64_t n = *start;
    while (n % 2 == 0 || n % 3 == 0 || n % 5 == 0) ++n;
    int r = (int)(n % 30);
    for (int i = 0; i < 8; ++i)
        if (res[i] == r) *index = i;
    *start = n;
    return FS_OK;
}

int fs_is_prime(uint64_t p) { return fs::is_prime_u64(p) ? 1 : 0; }

int fs_verify_factor(uint64_t p, uint32_t n, int32_t c) { return fs::verify_factor(p, n, c) ? 1 : 0; }

}  // extern "C"

// ------------------------------------------------------------------ batch --

namespace {

// Work per candidate of a job in walk-step units: the walk (slower steps for
// larger p*k) plus the setup (about 0.036 n Montgomery products, each worth
// about 2.7 walk steps).
double job_cost(const fs_job& j) {
    const double w = (double)(j.nmax - j.nmin);
    const double pk = (double)j.pmax * (double)j.nmax;
    const double wf = pk <= 4.6e18 ? 1.0 : (j.pmax < (1ull << 63) ? 1.2 : 1.5);
    return w * wf + 0.036 * (double)j.nmin * 2.7 + 64.0;
}

void batch_free(fs_ctx* c) {
    auto& b = c->batch;
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    cudaFree(b.d_cand);
    cudaFree(b.d_words);
    cudaFree(b.d_layers);
    cudaFree(b.d_jobs);
    cudaFree(b.d_ctr);
    cudaFree(b.d_gctr);
    cudaFree(b.d_tile);
    cudaFree(b.d_hits);
    b = fs_ctx::Batch();
}

}  // namespace

extern "C" int fs_batch_release(fs_ctx* c) {
    if (!c) return FS_E_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    batch_free(c);
    return FS_OK;
}

extern "C" int fs_batch_prepare(fs_ctx* c, const fs_job* jobs, uint32_t njobs, uint32_t hitcap) {
    if (!c || !jobs || njobs == 0 || njobs > (uint32_t)fs::batch_max_jobs() || hitcap == 0) return FS_E_ARG;
    for (uint32_t i = 0; i < njobs; ++i) {
        const fs_job& j = jobs[i];
        if (j.nmin > j.nmax || j.nmax > 0x7FFFFFFFu || j.pmin > j.pmax || j.pmin < j.nmin || j.pmin < 3) {
            c->err = "invalid job " + std::to_string(i);
            return FS_E_ARG;
        }
        if (fs_candidate_capacity(j.pmin, j.pmax) >= 0xFFFFFFF0ull || (j.pmax - j.pmin) / 64 >= (1ull << 31)) {
            c->err = "job " + std::to_string(i) + " too wide";
            return FS_E_ARG;
        }
    }
    int rc = bind(c);
    if (rc) return rc;
    CK(c, cudaStreamSynchronize(c->stream));
    batch_free(c);
    auto& b = c->batch;
    b.njobs = njobs;
    b.order.resize(njobs);
    for (uint32_t i = 0; i < njobs; ++i) b.order[i] = i;
    std::stable_sort(b.order.begin(), b.order.end(),
                     [&](uint32_t x, uint32_t y) { return job_cost(jobs[x]) > job_cost(jobs[y]); });
    // plans: one per distinct nmin, concatenated
    std::map<uint32_t, std::pair<uint32_t, uint32_t>> layer_range;   // nmin -> [begin, end)
    std::map<uint32_t, uint64_t> deficit;
    std::vector<uint64_t> words;
    std::vector<fs::Layer> layers;
    for (uint32_t i = 0; i < njobs; ++i) {
        const uint32_t n = jobs[i].nmin;
        if (layer_range.count(n)) continue;
        fs::SetupPlan p = fs::build_plan(n, 1);
        const uint32_t woff = (uint32_t)words.size(), lb = (uint32_t)layers.size();
        words.insert(words.end(), p.words.begin(), p.words.end());
        if (words.size() & 1) words.push_back(0);   // keep every plan's paired loads 16-byte aligned
        for (const auto& L : p.layers) layers.push_back({L.begin + woff, L.end + woff, L.dbl, 0});
        layer_range[n] = {lb, (uint32_t)layers.size()};
        deficit[n] = p.deficit;
    }
    std::vector<fs::BatchJob> dj(njobs);
    b.cap.resize(njobs);
    uint64_t total = 0;
    std::vector<uint64_t> off(njobs);
    for (uint32_t k = 0; k < njobs; ++k) {
        const fs_job& j = jobs[b.order[k]];
        b.cap[k] = fs_candidate_capacity(j.pmin, j.pmax);
        off[k] = total;
        total += (b.cap[k] + 1) & ~1ull;
    }
    CK(c, cudaMalloc((void**)&b.d_cand, (total + 2) * sizeof(u64)));
    CK(c, cudaMalloc((void**)&b.d_words, (words.size() + 2) * sizeof(u64)));
    CK(c, cudaMalloc((void**)&b.d_layers, (layers.size() + 1) * sizeof(fs::Layer)));
    CK(c, cudaMalloc((void**)&b.d_jobs, njobs * sizeof(fs::BatchJob)));
    CK(c, cudaMalloc((void**)&b.d_ctr, njobs * sizeof(fs::Counters)));
    CK(c, cudaMalloc((void**)&b.d_gctr, sizeof(fs::Counters)));
    CK(c, cudaMalloc((void**)&b.d_tile, sizeof(u32)));
    CK(c, cudaMalloc((void**)&b.d_hits, (size_t)hitcap * sizeof(fs::Factor)));
    b.hitcap = hitcap;
    for (uint32_t k = 0; k < njobs; ++k) {
        const fs_job& j = jobs[b.order[k]];
        dj[k].cand = b.d_cand + off[k];
        dj[k].cap = (u32)b.cap[k];
        dj[k].nstart = j.nmin;
        dj[k].nend = j.nmax;
        dj[k].layer_begin = layer_range[j.nmin].first;
        dj[k].layer_end = layer_range[j.nmin].second;
        dj[k].walk = (u32)fs::walk_for_range(j.pmin, j.pmax, j.nmax);
        dj[k].deficit = deficit[j.nmin];
    }
    CK(c, cudaMemcpy(b.d_words, words.data(), words.size() * sizeof(u64), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(b.d_layers, layers.data(), layers.size() * sizeof(fs::Layer), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(b.d_jobs, dj.data(), njobs * sizeof(fs::BatchJob), cudaMemcpyHostToDevice));
    int occ = 0;
    if (fs::batch_occupancy(&occ) != cudaSuccess || occ < 1) occ = 1;

    // capture: clears, the candidate launches, the persistent sieve
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(b.d_ctr, 0, njobs * sizeof(fs::Counters), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.d_gctr, 0, sizeof(fs::Counters), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.d_tile, 0, sizeof(u32), c->stream);
    const bool timing = c->timing;
    const uint64_t l0 = c->launches, g0 = c->gen_launches;
    c->timing = false;   // no event records inside the capture
    int grc = FS_OK;
    for (uint32_t k = 0; k < njobs && e == cudaSuccess && grc == FS_OK; ++k) {
        const fs_job& j = jobs[b.order[k]];
        grc = run_gen(c, j.pmin, j.pmax, b.d_cand + off[k], (uint32_t)b.cap[k], b.d_ctr + k);
    }
    c->timing = timing;
    c->launches = l0;    // launches are counted when the graph replays
    c->gen_launches = g0;
    fs::BatchArgs a;
    memset(&a, 0, sizeof(a));
    a.jobs = b.d_jobs;
    a.njobs = njobs;
    a.ctr = b.d_ctr;
    a.gctr = b.d_gctr;
    a.tile_counter = b.d_tile;
    a.words = b.d_words;
    a.layers = b.d_layers;
    a.hits = b.d_hits;
    a.hitcap = hitcap;
    // tile size from the context's tuning (fs_autotune_batch measures it)
    a.tile_candidates = c->tuning.batch_tile_candidates ? c->tuning.batch_tile_candidates : fs::kTileCandidates;
    if (e == cudaSuccess && grc == FS_OK) e = fs::launch_batch(a, c->sm_count * occ, c->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (grc != FS_OK) {
        if (g) cudaGraphDestroy(g);
        return grc;
    }
    CK(c, e);
    CK(c, e2);
    b.graph = g;
    CK(c, cudaGraphInstantiate(&b.exec, g, 0));
    b.ready = true;
    return FS_OK;
}

extern "C" int fs_batch_launch(fs_ctx* c) {
    if (!c) return FS_E_ARG;
    if (!c->batch.ready) return FS_E_STATE;
    int rc = bind(c);
    if (rc) return rc;
    std::pair<cudaEvent_t, cudaEvent_t> ev;
    if ((rc = ev_begin(c, &ev))) return rc;
    CK(c, cudaGraphLaunch(c->batch.exec, c->stream));
    if ((rc = ev_end(c, ev, c->batch_ev))) return rc;
    c->launches += c->batch.njobs + 1;
    c->gen_launches += c->batch.njobs;
    ++c->batch_launches;
    return FS_OK;
}

extern "C" int fs_batch_collect(fs_ctx* c, fs_job_result* results, fs_factor* hits, uint64_t hitcap,
                                uint64_t* nhits) {
    if (!c) return FS_E_ARG;
    auto& b = c->batch;
    if (!b.ready) return FS_E_STATE;
    int rc = bind(c);
    if (rc) return rc;
    std::vector<fs::Counters> h(b.njobs);
    fs::Counters g;
    CK(c, cudaStreamSynchronize(c->stream));
    CK(c, cudaMemcpy(h.data(), b.d_ctr, b.njobs * sizeof(fs::Counters), cudaMemcpyDeviceToHost));
    CK(c, cudaMemcpy(&g, b.d_gctr, sizeof(g), cudaMemcpyDeviceToHost));
    const uint64_t stored = std::min<uint64_t>(g.nhits, b.hitcap);
    std::vector<fs::Factor> hv(stored);
    if (stored) CK(c, cudaMemcpy(hv.data(), b.d_hits, stored * sizeof(fs::Factor), cudaMemcpyDeviceToHost));
    uint32_t any = g.flags;
    std::vector<uint64_t> per(b.njobs, 0);
    for (auto& f : hv) {
        const uint32_t k = (uint32_t)f.pad;
        f.pad = (int)b.order[k];
        per[k]++;
    }
    for (uint32_t k = 0; k < b.njobs; ++k) {
        uint32_t fl = h[k].flags;
        if (h[k].ncand > b.cap[k]) fl |= FS_FLAG_CAND_OVERFLOW;
        any |= fl;
        if (results) {
            fs_job_result& r = results[b.order[k]];
            r.raw_sum = h[k].raw_sum;
            r.primecount = h[k].ncand;
            r.nhits = per[k];
            r.flags = fl;
            r.pad = 0;
        }
    }
    if (nhits) *nhits = g.nhits;
    if (hits) memcpy(hits, hv.data(), std::min<uint64_t>(stored, hitcap) * sizeof(fs_factor));
    if (any & FS_FLAG_TABLE) return FS_E_TABLE;
    if (any & FS_FLAG_VALIDATION) return FS_E_VALIDATION;
    if ((any & (FS_FLAG_CAND_OVERFLOW | FS_FLAG_HIT_OVERFLOW)) || g.nhits > b.hitcap || (hits && g.nhits > hitcap))
        return FS_E_OVERFLOW;
    return FS_OK;
}
