// fs_tune.cu -- measured launch sizing: the role of the reference's
// profileGPU (cl_sieve.cpp:617-718) and of its setup/iterate retuning
// (cl_sieve.cpp:1158-1227).
//
// The reference times one candidate-generator launch and scales a segment's
// p-range so the generator takes 1 ms, then times one setup and one iterate
// launch and scales their work to 10-50 ms of kernel time.  Here one fused
// launch does setup, walk and check for a whole segment, so the tuner times
// whole segment searches of a sample of the real workload (its first
// p-values, the real n-range), one per launch shape:
//   primes per thread        sieve_variant 3 (two) or 5 (four)
//   blocks per SM            sieve_blocks_per_sm: 1x, 2x, 4x the resident ones
//   threads per block        sieve_block_threads: 256 or 128
//   n-steps per launch       max_steps_per_launch: the whole n-range, all but
//                            the last 8 steps (the check in a launch of its
//                            own), or halves
// keeps the fastest (a shape must beat the one before by 0.5 % to replace it,
// so noise does not move the choice), applies it to the context, and sizes
// the segment so one launch takes about target_ms at the measured rate.
// Batches get the tile size of the persistent batch kernel the same way
// (fs_autotune_batch), timed on the job mix with narrowed p-ranges.
// Choices are cached in a text file keyed by GPU name, SM count and the
// workload's bucket (log2 of the n-width, of p and of nmin; for a batch, a
// hash of its job list).  Tuning changes speed only, never results.
#include <cuda_runtime.h>

#include <algorithm>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/factsieve.h"
#include "fs_host.h"
#include "fs_internal.h"
#include "fs_launch.h"

namespace {

constexpr uint64_t kMaxSegment = 4294900000ull;   // the reference's segment limit (cl_sieve.cpp:625-627)

std::string gpu_name(fs_ctx* c) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) return "gpu";
    std::string n(prop.name);
    for (char& ch : n)
        if (ch == ' ' || ch == '|' || ch == '\t') ch = '_';
    return n;
}

int lg(double x) { return (int)std::floor(std::log2(std::max(x, 1.0))); }

uint32_t steps_code(uint32_t steps, uint32_t W) {
    if (steps == 0 || steps >= W) return 0;
    if (W > 8 && steps == W - 8) return 1;
    if (steps == (W + 1) / 2) return 2;
    return steps > 2 ? steps : 0;
}

uint32_t steps_from_code(uint32_t code, uint32_t W) {
    if (code == 1) return W > 8 ? W - 8 : 0;
    if (code == 2) return (W + 1) / 2;
    return code;
}

std::string search_key(fs_ctx* c, uint64_t pmin, uint32_t nmin, uint32_t nmax) {
    char buf[256];
    snprintf(buf, sizeof buf, "search|%s|sm%d|W%d|P%d|N%d", gpu_name(c).c_str(), c->sm_count,
             lg((double)(nmax - nmin)), lg((double)pmin), lg((double)nmin));
    return buf;
}

// One cached choice: a text line "<key> <variant> <bpsm> <threads> <steps> <tile> <rate>",
// <steps> coded against the search's own n-width W (the bucket holds several):
// 0 one launch, 1 all but the last 8 steps, 2 halves (larger: that many steps).
struct Entry {
    uint32_t variant = 0, bpsm = 0, threads = 0, steps = 0, tile = 0;
    double rate = 0;
};

bool cache_get(const char* path, const std::string& key, Entry* e) {
    if (!path || !*path) return false;
    FILE* f = fopen(path, "r");
    if (!f) return false;
    char line[512], k[320];
    bool found = false;
    while (fgets(line, sizeof line, f)) {
        Entry x;
        if (sscanf(line, "%319s %u %u %u %u %u %lf", k, &x.variant, &x.bpsm, &x.threads, &x.steps, &x.tile,
                   &x.rate) == 7 &&
            key == k) {
            *e = x;
            found = true;
        }
    }
    fclose(f);
    return found;
}

// Rewrite the file with this key's line replaced (other keys kept), through a
// temporary file and a rename.
void cache_put(const char* path, const std::string& key, const Entry& e) {
    if (!path || !*path) return;
    std::vector<std::string> keep;
    if (FILE* f = fopen(path, "r")) {
        char line[512], k[320];
        while (fgets(line, sizeof line, f))
            if (sscanf(line, "%319s", k) == 1 && key != k) keep.emplace_back(line);
        fclose(f);
    }
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "w");
    if (!f) return;
    for (const auto& l : keep) fputs(l.c_str(), f);
    fprintf(f, "%s %u %u %u %u %u %.6e\n", key.c_str(), e.variant, e.bpsm, e.threads, e.steps, e.tile, e.rate);
    if (fclose(f) == 0) rename(tmp.c_str(), path);
}

// The context's statistics, kept across the tuner's own timed launches.
struct SavedStats {
    uint64_t launches, sieve_launches, gen_launches, batch_launches;
    double sieve_ms, gen_ms, batch_ms;
    bool timing;
};

SavedStats save_stats(fs_ctx* c) {
    fs_stats st;
    fs_get_stats(c, &st);   // drains pending events into the totals
    return {c->launches, c->sieve_launches, c->gen_launches, c->batch_launches,
            c->sieve_ms,  c->gen_ms,         c->batch_ms,     c->timing};
}

void restore_stats(fs_ctx* c, const SavedStats& s) {
    fs_stats st;
    fs_get_stats(c, &st);
    c->launches = s.launches;
    c->sieve_launches = s.sieve_launches;
    c->gen_launches = s.gen_launches;
    c->batch_launches = s.batch_launches;
    c->sieve_ms = s.sieve_ms;
    c->gen_ms = s.gen_ms;
    c->batch_ms = s.batch_ms;
    c->timing = s.timing;
}

// Work units of a search: candidates x n-steps (candidates when the n-range is empty).
double units(uint64_t cands, uint32_t nmin, uint32_t nmax) {
    return (double)cands * (double)std::max<uint32_t>(nmax - nmin, 1);
}

// One sample search with shape t: units per second of generator + sieve
// kernel time (CUDA events), or a status.  The rate is the steady-state one
// a long segment sees: a grid-stride launch of G threads over N thread-units
// (pairs or quads of candidates) takes ceil(N/G) rounds, so a sample's rate
// is scaled by ceil(x)/x, x = N/G, and a short sample does not favour the
// shapes whose grid it happens to fill.
int time_shape(fs_ctx* c, const fs_tuning& t, uint64_t lo, uint64_t hi, uint32_t nmin, uint32_t nmax,
               double* rate) {
    int rc = fs_set_tuning(c, &t);
    if (rc || (rc = fs_search_begin(c, lo, hi, nmin, nmax, 0))) return rc;
    c->timing = true;
    if ((rc = fs_reset_stats(c))) return rc;
    if ((rc = fs_search_segment(c, lo, hi))) return rc;
    fs_stats st;
    if ((rc = fs_get_stats(c, &st))) return rc;
    uint64_t nf = 0, raw = 0, pc = 0;
    uint32_t flags = 0;
    rc = fs_search_collect(c, nullptr, 0, &nf, &raw, &pc, &flags);
    if (rc && rc != FS_E_OVERFLOW) return rc;   // a sample may hold more hits than a zero-size buffer
    if (flags & (FS_FLAG_VALIDATION | FS_FLAG_TABLE | FS_FLAG_CAND_OVERFLOW)) return FS_E_VALIDATION;
    const double ms = st.sieve_ms + st.gen_ms;
    *rate = ms > 0 ? units(pc, nmin, nmax) / (ms * 1e-3) : 0.0;
    const bool quad = t.sieve_variant == 5 && fs::walk_for_range(lo, hi, nmax) != fs::WALK_ANY;
    const double ppt = quad ? 4.0 : 2.0;
    const double grid = (double)c->sm_count * t.sieve_blocks_per_sm * (t.sieve_block_threads ? t.sieve_block_threads : 256);
    const double x = std::ceil((double)pc / ppt) / std::max(grid, 1.0);
    if (x > 0) *rate *= std::ceil(x) / x;
    return FS_OK;
}

double est_cands(uint64_t lo, uint64_t hi) {
    if (hi <= lo) return 0;
    return (double)(hi - lo) / std::log(std::max<double>((double)lo, 3.0));
}

// Segment width whose launch takes about target_ms at `rate` units/s (or,
// with nothing measured, about 1.5e12 units at the planning rate).
uint64_t width_for(double rate, double target_ms, uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax) {
    const double lp = std::log(std::max<double>((double)pmin, 3.0));
    const double w1 = (double)std::max<uint32_t>(nmax - nmin, 1);
    double cands = rate > 0 ? rate / w1 * target_ms * 1e-3 : 1.5e12 / (w1 + 0.036 * nmin + 64.0);
    double w = std::min(std::max(cands * lp, 1e5), (double)kMaxSegment);
    uint64_t wi = (uint64_t)w;
    if (pmax - pmin < wi) wi = pmax - pmin;
    return std::max<uint64_t>(wi, 1);
}

void fill_result(fs_ctx* c, uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax, double target_ms,
                 double rate, fs_tune_result* out) {
    fs_get_tuning(c, &out->tuning);
    out->rate = rate;
    out->seg_width = width_for(rate, target_ms, pmin, pmax, nmin, nmax);
    out->seg_capacity = fs_candidate_capacity(pmin, pmin + out->seg_width);
    out->setup_words = (uint32_t)fs::build_plan(nmin, 1).words.size();
    const uint32_t w = nmax - nmin, ms = c->tuning.max_steps_per_launch;
    out->steps_per_launch = ms && ms < w ? ms : w;
}

}  // namespace

extern "C" int fs_autotune(fs_ctx* c, uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax, double target_ms,
                           const char* cache_path, fs_tune_result* out) {
    if (!c || !out) return FS_E_ARG;
    if (pmin == 0 || pmax == 0 || nmin == 0 || nmax == 0 || nmin > nmax || pmin > pmax || pmin < nmin ||
        nmax > 0x7FFFFFFFu) {
        c->err = "invalid search range";
        return FS_E_ARG;
    }
    int rc = fs_internal::bind(c);
    if (rc) return rc;
    if (!(target_ms > 0)) target_ms = 1000.0;
    memset(out, 0, sizeof(*out));
    const std::string key = search_key(c, pmin, nmin, nmax);
    Entry e;
    if (cache_get(cache_path, key, &e)) {
        fs_tuning t{};
        t.sieve_variant = e.variant;
        t.sieve_blocks_per_sm = e.bpsm;
        t.sieve_block_threads = e.threads;
        t.max_steps_per_launch = steps_from_code(e.steps, nmax - nmin);
        t.batch_tile_candidates = c->tuning.batch_tile_candidates;
        if ((rc = fs_set_tuning(c, &t))) return rc;
        fill_result(c, pmin, pmax, nmin, nmax, target_ms, e.rate, out);
        out->from_cache = 1;
        return FS_OK;
    }
    // the sample: the range's first p-values, at least about 2e11 units of
    // work (a tenth of a second on a GB300) and three passes of the largest
    // grid tried (so the last partial pass does not decide); the ten or so
    // samples together stay near a tenth of the whole run, and a run too
    // short for that keeps the defaults
    const uint32_t W = nmax - nmin;
    const double words = (double)fs::build_plan(nmin, 1).words.size();
    const double per_cand = (double)W + 2.7 * words + 64.0;   // walk steps + setup, in walk-step units
    const double pass = (double)c->sm_count * c->sieve_occ[5] * 4 * 256 * 4;
    const double want = std::max(2e11 / per_cand, 3 * pass);
    const double sample_cands = want <= est_cands(pmin, pmax) / 100 ? want : 0.0;
    const uint32_t batch_tile = c->tuning.batch_tile_candidates;
    if (sample_cands < 20000) {
        // too short a run to time: the defaults
        fs_tuning t{};
        t.batch_tile_candidates = batch_tile;
        if ((rc = fs_set_tuning(c, &t))) return rc;
        fill_result(c, pmin, pmax, nmin, nmax, target_ms, 0.0, out);
        return FS_OK;
    }
    const double lp = std::log(std::max<double>((double)pmin, 3.0));
    uint64_t ws = (uint64_t)std::min<double>(sample_cands * lp, (double)kMaxSegment);
    if (ws > pmax - pmin) ws = pmax - pmin;
    const uint64_t lo = pmin, hi = pmin + ws;
    const SavedStats saved = save_stats(c);
    std::vector<fs_tuning> shapes;
    const bool quad = fs::walk_for_range(lo, hi, nmax) != fs::WALK_ANY;
    for (int v : quad ? std::vector<int>{5, 3} : std::vector<int>{3}) {
        const int occ = c->sieve_occ[v];
        for (int m : v == 5 ? std::vector<int>{4, 2, 1} : std::vector<int>{1, 2, 4}) {
            fs_tuning t{};
            t.sieve_variant = (uint32_t)v;
            t.sieve_blocks_per_sm = (uint32_t)(occ * m);
            t.sieve_block_threads = 256;
            t.batch_tile_candidates = batch_tile;
            shapes.push_back(t);
        }
    }
    fs_tuning best{};
    double best_rate = -1;
    uint32_t tried = 0;
    auto consider = [&](const fs_tuning& t) -> int {
        double r = 0;
        const int trc = time_shape(c, t, lo, hi, nmin, nmax, &r);
        if (trc) return trc;
        ++tried;
        if (best_rate < 0 || r > best_rate * 1.005) {
            best = t;
            best_rate = r;
        }
        return FS_OK;
    };
    double warm = 0;
    rc = time_shape(c, shapes[0], lo, hi, nmin, nmax, &warm);   // first launches, plan upload: not counted
    for (size_t i = 0; !rc && i < shapes.size(); ++i) rc = consider(shapes[i]);
    if (!rc) {
        // the best shape with 128-thread blocks (same threads per SM)
        fs_tuning t = best;
        t.sieve_block_threads = 128;
        t.sieve_blocks_per_sm = 2 * best.sieve_blocks_per_sm;
        rc = consider(t);
    }
    if (!rc && W >= 4096) {
        // the n-range in two launches instead of one: all but the last eight
        // steps in a launch that stores residues and tags, and the final check
        // in a launch of its own (the walk loop of a kernel that also checks
        // runs 1-2 % slower for some steps and faster for others), or halves
        const fs_tuning base = best;
        for (uint32_t steps : {W - 8, (W + 1) / 2}) {
            fs_tuning t = base;
            t.max_steps_per_launch = steps;
            if ((rc = consider(t))) break;
        }
    }
    c->active = false;   // the sample searches are over; the caller begins its own
    restore_stats(c, saved);
    if (rc) {
        fs_tuning d{};
        fs_set_tuning(c, &d);
        return rc;
    }
    if ((rc = fs_set_tuning(c, &best))) return rc;
    fill_result(c, pmin, pmax, nmin, nmax, target_ms, best_rate, out);
    out->shapes_tried = tried;
    Entry ne;
    ne.variant = best.sieve_variant;
    ne.bpsm = best.sieve_blocks_per_sm;
    ne.threads = best.sieve_block_threads;
    ne.steps = steps_code(best.max_steps_per_launch, W);
    ne.rate = best_rate;
    cache_put(cache_path, key, ne);
    return FS_OK;
}

extern "C" int fs_autotune_batch(fs_ctx* c, const fs_job* jobs, uint32_t njobs, uint32_t scale_down,
                                 const char* cache_path, uint32_t* tile_out, double* ms_out) {
    if (!c || !jobs || njobs == 0) return FS_E_ARG;
    int rc = fs_internal::bind(c);
    if (rc) return rc;
    if (scale_down == 0) scale_down = 16;
    // key: the GPU and an FNV-1a hash of the job list
    uint64_t h = 1469598103934665603ull;
    const unsigned char* b = (const unsigned char*)jobs;
    for (size_t i = 0; i < njobs * sizeof(fs_job); ++i) h = (h ^ b[i]) * 1099511628211ull;
    char key[256];
    snprintf(key, sizeof key, "batch|%s|sm%d|J%u|S%u|H%016" PRIx64, gpu_name(c).c_str(), c->sm_count, njobs,
             scale_down, h);
    Entry e;
    fs_tuning t = c->tuning;
    if (cache_get(cache_path, key, &e)) {
        t.batch_tile_candidates = e.tile;
        if ((rc = fs_set_tuning(c, &t))) return rc;
        if (tile_out) *tile_out = e.tile;
        if (ms_out) *ms_out = 0;
        return FS_OK;
    }
    // the mix with every p-range narrowed scale_down times: the same n-ranges
    // and setup plans, fewer candidates per job
    std::vector<fs_job> sample(jobs, jobs + njobs);
    for (auto& j : sample) {
        const uint64_t w = std::max<uint64_t>((j.pmax - j.pmin) / scale_down, 10000);
        j.pmax = j.pmin + w < j.pmin ? ~0ull : j.pmin + w;   // no wrap past 2^64
    }
    const SavedStats saved = save_stats(c);
    uint32_t best_tile = fs::kTileCandidates;
    double best_ms = -1;
    for (int pass = 0; pass < 2 && !rc; ++pass) {   // pass 0 warms up (graph, plans), pass 1 is timed
        for (uint32_t tile : {1024u, 2048u, 4096u}) {
            t.batch_tile_candidates = tile;
            if ((rc = fs_set_tuning(c, &t))) break;
            if ((rc = fs_batch_prepare(c, sample.data(), njobs, 1u << 20))) break;
            c->timing = true;
            if ((rc = fs_reset_stats(c)) || (rc = fs_batch_launch(c))) break;
            rc = fs_batch_collect(c, nullptr, nullptr, 0, nullptr);
            if (rc && rc != FS_E_OVERFLOW) break;
            rc = FS_OK;
            fs_stats st;
            if ((rc = fs_get_stats(c, &st))) break;
            if (pass == 1 && (best_ms < 0 || st.batch_ms < best_ms * 0.995)) {
                best_ms = st.batch_ms;
                best_tile = tile;
            }
        }
    }
    fs_batch_release(c);
    restore_stats(c, saved);
    t.batch_tile_candidates = best_tile;
    if (rc) {
        t.batch_tile_candidates = 0;
        fs_set_tuning(c, &t);
        return rc;
    }
    if ((rc = fs_set_tuning(c, &t))) return rc;
    if (tile_out) *tile_out = best_tile;
    if (ms_out) *ms_out = best_ms;
    Entry ne;
    ne.tile = best_tile;
    ne.rate = best_ms;
    cache_put(cache_path, key, ne);
    return FS_OK;
}
