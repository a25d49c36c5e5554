// fs_serve.cu -- continuous-batching request loop over the sieve kernels.
//
// Requests (jobs: a p-range and an n-range) queue on the host.  Each round:
//   1. admit queued jobs while a slot is free and the device keeps
//      `mem_reserve` bytes free after the job's buffers (cudaMemGetInfo);
//      an admitted job gets its candidate and residue buffers, its setup plan
//      uploaded, and a candidate-generation launch;
//   2. give every working job an equal share of the round's work budget:
//      starting residues for the next block of its candidates, or the next
//      chunk of its walk over all its candidates (residues stay in its device
//      buffer between rounds), ending with the checksum step;
//   3. run the round as one persistent kernel over all those tiles, wait,
//      drain the hits (tagged by job slot), and retire finished jobs.
// Jobs that arrive while others are on the GPU join at the next round, so
// their work overlaps with the running ones'.  Every job's result is the
// same bits as a search of that job alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "../../include/factsieve.h"
#include "fs_host.h"
#include "fs_internal.h"
#include "fs_launch.h"

namespace fs_serve {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum State { QUEUED = 0, GENERATING, SETUP, WALK, DONE };

struct Job {
    int64_t id = 0;
    fs_job spec{};
    int slot = -1;
    State state = QUEUED;
    double t_submit = 0, t_admit = 0, t_done = 0;
    u64* d_cand = nullptr;
    u64* d_res = nullptr;      // cap residues, then cap u32 walked-n tags
    u64* d_words = nullptr;
    fs::Layer* d_layers = nullptr;
    uint32_t nlayers = 0;
    uint64_t nwords = 0, deficit = 0;
    uint64_t cap = 0;
    uint32_t ncand = 0;
    uint32_t setup_next = 0;   // starting residues done for candidates [0, setup_next)
    uint32_t walk_n = 0;       // residues hold walk_n! * R
    bool final_queued = false;
    int64_t gen_round = -1;    // its candidate launch completes with this round
    int64_t final_round = -1;  // its checksum step runs in this round
    uint64_t raw_sum = 0;
    uint32_t flags = 0;
    std::vector<fs_factor> hits;
};

struct Server {
    fs_serve_config cfg{};
    std::deque<std::unique_ptr<Job>> queue;
    std::vector<std::unique_ptr<Job>> active;   // indexed by slot (nullptr = free)
    std::vector<std::unique_ptr<Job>> done;
    fs::Counters* d_ctr = nullptr;               // one per slot
    // two rounds in flight at most: the one running and the one being drained
    fs::Counters* d_gctr[2] = {nullptr, nullptr};
    u32* d_tile_counter[2] = {nullptr, nullptr};
    fs::Factor* d_hits[2] = {nullptr, nullptr};
    fs::ServeChunk* d_chunks[2] = {nullptr, nullptr};
    fs::ServeChunk* h_chunks[2] = {nullptr, nullptr};   // pinned
    cudaEvent_t ev[2] = {nullptr, nullptr};
    // pinned staging for plan uploads of the jobs admitted behind round b
    uint8_t* stage[2] = {nullptr, nullptr};
    size_t stage_used[2] = {0, 0};
    int inflight = -1;                           // buffer of the round in flight
    int64_t inflight_id = -1;
    int64_t round_id = 0;                        // id of the next round
    uint32_t next_job = 0;                       // round-robin start slot
    int grid4 = 1, grid2 = 1;                    // persistent grids of the 4- and 2-per-thread forms
    uint64_t rounds = 0, served_steps = 0;
    double setup_units = 0;                      // setup work queued, in walk-step units
    // CUDA events around each round kernel, read when drained
    cudaEvent_t kev[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    bool kev_used[2] = {false, false};
    double kernel_ms = 0;
    std::map<uint32_t, fs::SetupPlan> plan_cache;
};

// Stream-ordered frees: they wait for the work already queued, not the host.
void free_job_buffers(Job& j, cudaStream_t st) {
    cudaFreeAsync(j.d_cand, st);
    cudaFreeAsync(j.d_res, st);
    cudaFreeAsync(j.d_words, st);
    cudaFreeAsync(j.d_layers, st);
    j.d_cand = j.d_res = j.d_words = nullptr;
    j.d_layers = nullptr;
}

const fs::SetupPlan& plan_for(Server& s, uint32_t n) {
    auto it = s.plan_cache.find(n);
    if (it != s.plan_cache.end()) return it->second;
    if (s.plan_cache.size() > 256) s.plan_cache.erase(s.plan_cache.begin());
    return s.plan_cache.emplace(n, fs::build_plan(n, 1)).first->second;
}

// Bytes a job needs on the device.
uint64_t job_bytes(const fs_job& j) {
    const uint64_t cap = fs_candidate_capacity(j.pmin, j.pmax);
    const uint64_t words = (uint64_t)(0.04 * j.nmin) + 64;
    return cap * 20 + words * 8 + 4096;
}

}  // namespace fs_serve

using fs_serve::Job;
using fs_serve::Server;

#define SK(ctx, call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            (ctx)->err = std::string(#call) + ": " + cudaGetErrorString(e_);   \
            return e_ == cudaErrorMemoryAllocation ? FS_E_NOMEM : FS_E_CUDA;   \
        }                                                                      \
    } while (0)

namespace {

constexpr size_t kStageBytes = 32u << 20;

// Admit one job behind the round using buffer b: stream-ordered buffers,
// plan upload through pinned staging, candidate launch.  1 admitted, 0 not now.
int admit(fs_ctx* c, Server& s, Job& j, int slot, int b, int* rc_out) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        *rc_out = FS_E_CUDA;
        return 0;
    }
    const uint64_t need = fs_serve::job_bytes(j.spec);
    if ((uint64_t)free_b < need + s.cfg.mem_reserve) return 0;
    const fs::SetupPlan& p = fs_serve::plan_for(s, j.spec.nmin);
    const size_t wbytes = p.words.size() * sizeof(u64), lbytes = p.layers.size() * sizeof(fs::Layer);
    const size_t need_stage = ((wbytes + 255) & ~size_t(255)) + ((lbytes + 255) & ~size_t(255));
    const bool staged = need_stage <= kStageBytes;
    if (staged && s.stage_used[b] + need_stage > kStageBytes) return 0;   // next round
    j.cap = fs_candidate_capacity(j.spec.pmin, j.spec.pmax);
    j.nlayers = (uint32_t)p.layers.size();
    j.nwords = p.words.size();
    j.deficit = p.deficit;
    auto fail = [&](int rc) {
        fs_serve::free_job_buffers(j, c->stream);
        *rc_out = rc;
        return 0;
    };
    if (cudaMallocAsync((void**)&j.d_cand, (j.cap + 2) * sizeof(u64), c->stream) != cudaSuccess ||
        cudaMallocAsync((void**)&j.d_res, (j.cap + 2 + (j.cap + 1) / 2) * sizeof(u64), c->stream) != cudaSuccess ||
        cudaMallocAsync((void**)&j.d_words, (j.nwords + 2) * sizeof(u64), c->stream) != cudaSuccess ||
        cudaMallocAsync((void**)&j.d_layers, (j.nlayers + 1) * sizeof(fs::Layer), c->stream) != cudaSuccess) {
        cudaGetLastError();
        fs_serve::free_job_buffers(j, c->stream);
        return 0;   // not enough memory after all: stay queued
    }
    if (staged) {
        // pinned staging keeps the copies asynchronous; the region is reused
        // only after this round's event has completed
        uint8_t* w = s.stage[b] + s.stage_used[b];
        uint8_t* l = w + ((wbytes + 255) & ~size_t(255));
        if (wbytes) memcpy(w, p.words.data(), wbytes);
        if (lbytes) memcpy(l, p.layers.data(), lbytes);
        s.stage_used[b] += need_stage;
        if (wbytes && cudaMemcpyAsync(j.d_words, w, wbytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            return fail(FS_E_CUDA);
        if (lbytes && cudaMemcpyAsync(j.d_layers, l, lbytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            return fail(FS_E_CUDA);
    } else {
        // a plan larger than the staging area: ordinary (synchronising) copies
        if (wbytes && cudaMemcpyAsync(j.d_words, p.words.data(), wbytes, cudaMemcpyHostToDevice, c->stream) !=
                          cudaSuccess)
            return fail(FS_E_CUDA);
        if (lbytes && cudaMemcpyAsync(j.d_layers, p.layers.data(), lbytes, cudaMemcpyHostToDevice, c->stream) !=
                          cudaSuccess)
            return fail(FS_E_CUDA);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(FS_E_CUDA);
    }
    j.slot = slot;
    if (cudaMemsetAsync(s.d_ctr + slot, 0, sizeof(fs::Counters), c->stream) != cudaSuccess) return fail(FS_E_CUDA);
    const int rc = fs_internal::run_gen(c, j.spec.pmin, j.spec.pmax, j.d_cand, (uint32_t)j.cap, s.d_ctr + slot);
    if (rc) return fail(rc);
    j.state = fs_serve::GENERATING;
    j.t_admit = fs_serve::now_s();
    j.walk_n = j.spec.nmin;
    return 1;
}

}  // namespace

extern "C" double fs_clock(void) { return fs_serve::now_s(); }

extern "C" int fs_serve_create(fs_ctx* c, const fs_serve_config* cfg) {
    if (!c || !cfg || cfg->max_active == 0 || cfg->max_active > 4096 || cfg->hitcap == 0) return FS_E_ARG;
    int rc = fs_internal::bind(c);
    if (rc) return rc;
    if (c->server) fs_serve_destroy(c);
    auto* s = new Server();
    s->cfg = *cfg;
    if (!s->cfg.round_budget) s->cfg.round_budget = 30000000000ull;
    s->active.resize(cfg->max_active);
    c->server = s;
    SK(c, cudaMalloc((void**)&s->d_ctr, cfg->max_active * sizeof(fs::Counters)));
    SK(c, cudaMemset(s->d_ctr, 0, cfg->max_active * sizeof(fs::Counters)));
    for (int b = 0; b < 2; ++b) {
        SK(c, cudaMalloc((void**)&s->d_gctr[b], sizeof(fs::Counters)));
        SK(c, cudaMalloc((void**)&s->d_tile_counter[b], sizeof(u32)));
        SK(c, cudaMalloc((void**)&s->d_hits[b], (size_t)cfg->hitcap * sizeof(fs::Factor)));
        SK(c, cudaMalloc((void**)&s->d_chunks[b], fs::kServeMaxChunks * sizeof(fs::ServeChunk)));
        SK(c, cudaMallocHost((void**)&s->h_chunks[b], fs::kServeMaxChunks * sizeof(fs::ServeChunk)));
        SK(c, cudaEventCreateWithFlags(&s->ev[b], cudaEventDisableTiming));
        SK(c, cudaEventCreate(&s->kev[b][0]));
        SK(c, cudaEventCreate(&s->kev[b][1]));
        SK(c, cudaMallocHost((void**)&s->stage[b], kStageBytes));
    }
    int occ = 0;
    if (fs::serve_occupancy(&occ, 4) != cudaSuccess || occ < 1) occ = 1;
    s->grid4 = c->sm_count * occ;
    occ = 0;
    if (fs::serve_occupancy(&occ, 2) != cudaSuccess || occ < 1) occ = 1;
    s->grid2 = c->sm_count * occ;
    return FS_OK;
}

extern "C" int fs_serve_destroy(fs_ctx* c) {
    if (!c || !c->server) return FS_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    Server* s = c->server;
    for (auto& j : s->active)
        if (j) fs_serve::free_job_buffers(*j, c->stream);
    cudaStreamSynchronize(c->stream);
    cudaFree(s->d_ctr);
    for (int b = 0; b < 2; ++b) {
        cudaFree(s->d_gctr[b]);
        cudaFree(s->d_tile_counter[b]);
        cudaFree(s->d_hits[b]);
        cudaFree(s->d_chunks[b]);
        if (s->h_chunks[b]) cudaFreeHost(s->h_chunks[b]);
        if (s->ev[b]) cudaEventDestroy(s->ev[b]);
        if (s->kev[b][0]) cudaEventDestroy(s->kev[b][0]);
        if (s->kev[b][1]) cudaEventDestroy(s->kev[b][1]);
        if (s->stage[b]) cudaFreeHost(s->stage[b]);
    }
    delete s;
    c->server = nullptr;
    return FS_OK;
}

extern "C" int fs_serve_submit(fs_ctx* c, const fs_job* job, int64_t id) {
    if (!c || !c->server || !job) return FS_E_ARG;
    const fs_job& j = *job;
    if (j.nmin > j.nmax || j.nmax > 0x7FFFFFFFu || j.pmin > j.pmax || j.pmin < j.nmin || j.pmin < 3 ||
        fs_candidate_capacity(j.pmin, j.pmax) >= 0xFFFFFFF0ull || (j.pmax - j.pmin) / 64 >= (1ull << 31))
        return FS_E_ARG;
    auto p = std::make_unique<Job>();
    p->id = id;
    p->spec = j;
    p->t_submit = fs_serve::now_s();
    c->server->queue.push_back(std::move(p));
    return FS_OK;
}

namespace {

// Drain round `rid` (buffer b), whose event has completed: hits, candidate
// counts of jobs whose generation finished with it, finished jobs.
int drain(fs_ctx* c, Server& s, int b, int64_t rid) {
    const uint32_t S = s.cfg.max_active;
    fs::Counters g;
    SK(c, cudaMemcpy(&g, s.d_gctr[b], sizeof(g), cudaMemcpyDeviceToHost));
    const uint32_t nh = std::min<uint32_t>(g.nhits, s.cfg.hitcap);
    if (nh) {
        std::vector<fs::Factor> hv(nh);
        SK(c, cudaMemcpy(hv.data(), s.d_hits[b], nh * sizeof(fs::Factor), cudaMemcpyDeviceToHost));
        for (const auto& f : hv) {
            Job* j = (f.pad >= 0 && (uint32_t)f.pad < S) ? s.active[f.pad].get() : nullptr;
            if (j) j->hits.push_back({f.p, f.nc, 0});
        }
    }
    if ((g.flags & FS_FLAG_HIT_OVERFLOW) || g.nhits > s.cfg.hitcap)
        for (auto& jp : s.active)
            if (jp) jp->flags |= FS_FLAG_HIT_OVERFLOW;
    // counters of slots the running round does not touch are final here
    std::vector<fs::Counters> ctr(S);
    SK(c, cudaMemcpy(ctr.data(), s.d_ctr, S * sizeof(fs::Counters), cudaMemcpyDeviceToHost));
    const double t = fs_serve::now_s();
    for (uint32_t slot = 0; slot < S; ++slot) {
        auto& jp = s.active[slot];
        if (!jp) continue;
        Job& j = *jp;
        if (j.state == fs_serve::GENERATING && j.gen_round >= 0 && j.gen_round <= rid) {
            j.ncand = ctr[slot].ncand;
            if (j.ncand > j.cap) {
                j.flags |= FS_FLAG_CAND_OVERFLOW;
                j.ncand = (uint32_t)j.cap;
            }
            j.state = j.ncand ? fs_serve::SETUP : fs_serve::DONE;
            j.setup_next = 0;
        } else if (j.final_queued && j.final_round <= rid) {
            j.state = fs_serve::DONE;
        }
        if (j.state == fs_serve::DONE) {
            j.raw_sum = ctr[slot].raw_sum;
            j.flags |= ctr[slot].flags;
            j.t_done = t;
            fs_serve::free_job_buffers(j, c->stream);
            s.done.push_back(std::move(jp));
        }
    }
    return FS_OK;
}

}  // namespace

// Walk chunks shorter than this spend too much of their time rebuilding the
// per-candidate constants; a job with less left finishes in one chunk.
constexpr uint64_t kMinWalkChunk = 2048;

// One pipeline step: queue the next round (its chunks follow from the host's
// bookkeeping alone), admit queued jobs behind it, then wait for the previous
// round and drain it.  One round stays in flight between calls.
extern "C" int fs_serve_round(fs_ctx* c, uint32_t* n_active, uint32_t* n_queued) {
    if (!c || !c->server) return FS_E_STATE;
    int rc = fs_internal::bind(c);
    if (rc) return rc;
    Server& s = *c->server;
    const uint32_t S = s.cfg.max_active;
    const int b = s.inflight == 0 ? 1 : 0;
    const int64_t R = s.round_id++;
    fs::ServeChunk* hc = s.h_chunks[b];
    // 1. the round's chunks: jobs in round-robin order until the budget is used
    uint32_t nch = 0;
    double budget = (double)s.cfg.round_budget;
    const uint32_t start = s.next_job;   // each job gets at most one chunk per round
    for (uint32_t k = 0; k < S && nch < (uint32_t)fs::kServeMaxChunks; ++k) {
        const uint32_t slot = (start + k) % S;
        auto& jp = s.active[slot];
        if (!jp || (jp->state != fs_serve::SETUP && jp->state != fs_serve::WALK) || jp->final_queued) continue;
        if (budget <= 0 && nch > 0) break;
        Job& j = *jp;
        fs::ServeChunk ch;
        memset(&ch, 0, sizeof(ch));
        ch.cand = j.d_cand;
        ch.residue = j.d_res;
        ch.walked = (u32*)(j.d_res + j.cap + 2);
        ch.nmax = j.spec.nmax;
        ch.ctr = s.d_ctr + j.slot;
        ch.words = j.d_words;
        ch.layers = j.d_layers;
        ch.deficit = j.deficit;
        ch.layer_begin = 0;
        ch.layer_end = j.nlayers;
        ch.tag = (u32)j.slot;
        const double per = 2.7 * (double)j.nwords + 64.0;   // setup cost per candidate, in walk-step units
        const double whole = (double)j.ncand * (per + (double)(j.spec.nmax - j.spec.nmin));
        if (j.state == fs_serve::SETUP && j.setup_next == 0 && whole <= std::max(budget, 0.0)) {
            // the whole job fits the round: starting residues, the walk and the
            // checksum in one chunk (one round instead of two or more)
            ch.first = 0;
            ch.count = j.ncand;
            ch.flags = fs::SERVE_SETUP | fs::SERVE_FINAL;
            ch.nstart = j.spec.nmin;
            ch.nend = j.spec.nmax;
            j.setup_next = j.ncand;
            j.walk_n = j.spec.nmax;
            j.state = fs_serve::WALK;
            j.final_queued = true;
            j.final_round = R;
            budget -= whole;
            s.setup_units += per * j.ncand;
            s.served_steps += (uint64_t)j.ncand * (uint64_t)(j.spec.nmax - j.spec.nmin);
        } else if (j.state == fs_serve::SETUP) {
            uint64_t cnt = (uint64_t)std::max(4096.0, std::max(budget, 0.0) / per);
            cnt = (cnt + fs::kTileCandidates - 1) / fs::kTileCandidates * fs::kTileCandidates;
            ch.first = j.setup_next;
            ch.count = (uint32_t)std::min<uint64_t>(cnt, j.ncand - j.setup_next);
            ch.flags = fs::SERVE_SETUP;
            ch.nstart = ch.nend = j.spec.nmin;
            if (j.spec.nmin == j.spec.nmax && j.setup_next + ch.count == j.ncand) {
                ch.flags |= fs::SERVE_FINAL;
                j.final_queued = true;
                j.final_round = R;
            }
            j.setup_next += ch.count;
            if (j.setup_next == j.ncand) j.state = fs_serve::WALK;
            budget -= per * ch.count;
            s.setup_units += per * ch.count;
        } else {
            const uint64_t left = j.spec.nmax - j.walk_n;
            uint64_t steps = (uint64_t)(std::max(budget, 0.0) / std::max<uint32_t>(j.ncand, 1));
            steps = std::max<uint64_t>(steps, kMinWalkChunk);
            steps = (steps + 7) / 8 * 8;
            if (steps >= left || left - steps < kMinWalkChunk / 2) steps = left;
            ch.first = 0;
            ch.count = j.ncand;
            ch.nstart = j.walk_n;
            ch.nend = j.walk_n + (uint32_t)steps;
            if (ch.nend == j.spec.nmax) {
                ch.flags = fs::SERVE_FINAL;
                j.final_queued = true;
                j.final_round = R;
            }
            s.served_steps += (uint64_t)j.ncand * steps;
            j.walk_n = ch.nend;
            budget -= (double)j.ncand * (double)steps;
        }
        ch.walk = (u32)fs::walk_for_range(j.spec.pmin, j.spec.pmax, ch.nend);
        hc[nch++] = ch;
        s.next_job = (slot + 1) % S;
    }
    // four candidates per thread, unless the round's tiles would not fill the
    // GPU: then two per thread, twice the blocks, a shorter round
    uint32_t tiles4 = 0;
    for (uint32_t k = 0; k < nch; ++k) tiles4 += (hc[k].count + fs::kTileCandidates - 1) / fs::kTileCandidates;
    const int ppt = tiles4 < (uint32_t)s.grid4 ? 2 : 4;
    const uint32_t per_tile = (uint32_t)ppt * fs::sieve_threads();
    uint32_t tiles = 0;
    for (uint32_t k = 0; k < nch; ++k) {
        tiles += (hc[k].count + per_tile - 1) / per_tile;
        hc[k].tile_end = tiles;
    }
    // 2. queue the round
    SK(c, cudaMemsetAsync(s.d_gctr[b], 0, sizeof(fs::Counters), c->stream));
    if (nch) {
        SK(c, cudaMemcpyAsync(s.d_chunks[b], hc, nch * sizeof(fs::ServeChunk), cudaMemcpyHostToDevice, c->stream));
        SK(c, cudaMemsetAsync(s.d_tile_counter[b], 0, sizeof(u32), c->stream));
        fs::ServeArgs a;
        memset(&a, 0, sizeof(a));
        a.chunks = s.d_chunks[b];
        a.nchunks = nch;
        a.tile_counter = s.d_tile_counter[b];
        a.gctr = s.d_gctr[b];
        a.hits = s.d_hits[b];
        a.hitcap = s.cfg.hitcap;
        SK(c, cudaEventRecord(s.kev[b][0], c->stream));
        SK(c, fs::launch_serve_round(a, std::min<int>(ppt == 2 ? s.grid2 : s.grid4, (int)tiles), c->stream, ppt));
        SK(c, cudaEventRecord(s.kev[b][1], c->stream));
        s.kev_used[b] = true;
        ++c->launches;
        ++c->sieve_launches;
    }
    // 3. admit queued jobs behind it, oldest first, while slots and memory allow
    s.stage_used[b] = 0;   // buffer b's staging: its previous round was drained last step
    for (uint32_t slot = 0; slot < S && !s.queue.empty(); ++slot) {
        if (s.active[slot]) continue;
        int arc = FS_OK;
        if (!admit(c, s, *s.queue.front(), (int)slot, b, &arc)) {
            if (arc) return arc;
            break;
        }
        s.queue.front()->gen_round = R;
        s.active[slot] = std::move(s.queue.front());
        s.queue.pop_front();
    }
    SK(c, cudaEventRecord(s.ev[b], c->stream));
    const int prev = s.inflight;
    const int64_t prev_id = s.inflight_id;
    s.inflight = b;
    s.inflight_id = R;
    ++s.rounds;
    // 4. wait for the previous round and drain it
    if (prev >= 0) {
        SK(c, cudaEventSynchronize(s.ev[prev]));
        if (s.kev_used[prev]) {
            float ms = 0;
            SK(c, cudaEventElapsedTime(&ms, s.kev[prev][0], s.kev[prev][1]));
            s.kernel_ms += ms;
            s.kev_used[prev] = false;
        }
        if ((rc = drain(c, s, prev, prev_id))) return rc;
    }
    uint32_t na = 0;
    for (auto& jp : s.active)
        if (jp) ++na;
    if (n_active) *n_active = na;
    if (n_queued) *n_queued = (uint32_t)s.queue.size();
    return FS_OK;
}

extern "C" int fs_serve_poll(fs_ctx* c, fs_served* out, uint32_t cap, uint32_t* n, fs_factor* hits,
                             uint64_t hitcap, uint64_t* nhits) {
    if (!c || !c->server || !n) return FS_E_ARG;
    Server& s = *c->server;
    uint32_t k = 0;
    uint64_t h = 0;
    size_t taken = 0;
    for (auto& jp : s.done) {
        if (k >= cap) break;
        const Job& j = *jp;
        if (hits && h + j.hits.size() > hitcap) break;
        fs_served& o = out[k++];
        o.id = j.id;
        o.raw_sum = j.raw_sum;
        o.primecount = j.ncand;
        o.nhits = j.hits.size();
        o.flags = j.flags;
        o.pad = 0;
        o.t_submit = j.t_submit;
        o.t_admit = j.t_admit;
        o.t_done = j.t_done;
        o.hit_offset = h;
        if (hits && !j.hits.empty()) memcpy(hits + h, j.hits.data(), j.hits.size() * sizeof(fs_factor));
        h += j.hits.size();
        ++taken;
    }
    s.done.erase(s.done.begin(), s.done.begin() + taken);
    *n = k;
    if (nhits) *nhits = h;
    return FS_OK;
}

extern "C" int fs_serve_stats(fs_ctx* c, uint64_t* rounds, uint64_t* served_steps, double* setup_units,
                              double* kernel_ms) {
    if (!c || !c->server) return FS_E_STATE;
    if (rounds) *rounds = c->server->rounds;
    if (served_steps) *served_steps = c->server->served_steps;
    if (setup_units) *setup_units = c->server->setup_units;
    if (kernel_ms) *kernel_ms = c->server->kernel_ms;
    return FS_OK;
}
