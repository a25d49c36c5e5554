/*
 * factsieve.h -- C ABI of the GB300 FactSieve sieve (libfactsieve.so).
 *
 * The library replaces the reference's device layer: the OpenCL shim
 * (simpleCL.h:67-117) plus the kernels getsegprimes, setup, iterate, check,
 * clearn, clearresult and the verify kernels of the kernels directory, and
 * carries the host pieces of the same path (power table, CPU factor
 * verification).  Every function returns a status code (FS_OK or FS_E_*)
 * and never exits the process; the reference printed and called exit() on
 * any error (simpleCL.c:347, cl_sieve.cpp:451-476).
 *
 * Threading: one fs_ctx per host thread; calls on one context are not
 * thread-safe.  Device buffers of a search belong to the context; host
 * arrays belong to the caller.  Functions taking d_* pointers want device
 * memory the caller owns (any allocator); they run asynchronously on the
 * context's stream.  That stream is created non-blocking: it does not wait
 * for work on the legacy default stream, so a caller that fills a d_* buffer
 * on another stream synchronizes first, or hands its stream to
 * fs_set_stream.
 */
#ifndef FACTSIEVE_H
#define FACTSIEVE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FS_OK 0
#define FS_E_ARG 1         /* bad argument (the reference's range checks, main.cpp:51-65, cl_sieve.cpp:561-589) */
#define FS_E_CUDA 2        /* a CUDA call failed; fs_last_error() has the text */
#define FS_E_OVERFLOW 3    /* candidate or factor buffer full (cl_sieve.cpp:451-455, 473-476) */
#define FS_E_VALIDATION 4  /* nmax round trip failed (check.cl:67-78, cl_sieve.cpp:463-467) */
#define FS_E_TABLE 5       /* power table disagrees with the direct product (verify*.cl, cl_sieve.cpp:903-907) */
#define FS_E_NOMEM 6       /* device or host allocation failed */
#define FS_E_VERIFY 7      /* a hit failed CPU verification (cl_sieve.cpp:502-506) */
#define FS_E_STATE 8       /* call out of order (e.g. segment before begin) */
#define FS_E_LIMIT 10      /* request larger than a fixed, compiled-in limit */

/* Factor record, layout of the reference's `factor` (cl_sieve.h:3-6):
 * nc = -n for p | n! - 1, +n for p | n! + 1 (iterate.cl:69-73). */
typedef struct {
    uint64_t p;
    int32_t nc;
    int32_t pad;
} fs_factor;

/* Device-resident counters shared by the stage-level kernels; the role of
 * the reference's g_primecount[6] and g_sum[] (clearn.cl, clearresult.cl,
 * check.cl:88-109). */
typedef struct {
    uint64_t raw_sum;     /* sum of (s6 + s7) over checked candidates, mod 2^64 */
    uint64_t primecount;  /* candidates counted by fs_check / segments */
    uint32_t ncand;       /* candidates written by fs_getsegprimes (may exceed capacity) */
    uint32_t nhits;       /* factor hits found by fs_iterate (may exceed capacity) */
    uint32_t flags;       /* FS_FLAG_* */
    uint32_t maxcand;     /* largest candidate count of one segment */
} fs_counters;

#define FS_FLAG_VALIDATION 1u
#define FS_FLAG_CAND_OVERFLOW 2u
#define FS_FLAG_HIT_OVERFLOW 4u
#define FS_FLAG_TABLE 8u

typedef struct fs_ctx fs_ctx;

/* Launch tuning; zero fields mean "choose automatically". */
typedef struct {
    uint32_t sieve_blocks_per_sm;   /* resident 256-thread sieve blocks per SM */
    uint32_t gen_blocks_per_sm;     /* candidate-generator blocks per SM */
    uint32_t max_steps_per_launch;  /* split the n-range into launches of at most this many steps */
    uint32_t setup_chunks;          /* split the power table across this many threads per prime (1 = never) */
    uint32_t sieve_variant;         /* sieve kernel build: 3 = two candidates per thread at 3 resident blocks per
                                       SM; 5 (default) = four candidates per thread at 2 (segments whose
                                       candidates share one walk step; a mixed segment runs build 3) */
    uint32_t sieve_block_threads;   /* threads per sieve block: 256 (default) or 128 */
    uint32_t batch_tile_candidates; /* candidates per tile of the batch kernel: 1024 (default), 2048 or 4096 */
} fs_tuning;

/* ---- library / device ---------------------------------------------------- */
int fs_version(void);
const char *fs_strerror(int code);
const char *fs_last_error(fs_ctx *ctx);
int fs_device_count(int *count);

/* Create a context on CUDA device `device` (replaces main.cpp:223-275 and
 * the program/buffer set-up of cl_sieve.cpp:928-958). */
int fs_create(int device, fs_ctx **out);
int fs_destroy(fs_ctx *ctx);
/* Run on an existing cudaStream_t (NULL: the context's own stream). */
int fs_set_stream(fs_ctx *ctx, void *stream);
void *fs_get_stream(fs_ctx *ctx);
int fs_set_tuning(fs_ctx *ctx, const fs_tuning *t);
int fs_get_tuning(fs_ctx *ctx, fs_tuning *t);
int fs_device_info(fs_ctx *ctx, int *sm_count, int *clock_khz, uint64_t *total_mem);
int fs_synchronize(fs_ctx *ctx);

/* ---- whole search (cl_sieve.cpp:918-1270) -------------------------------- */
/* Start a search over p in [pmin, pmax), n in [nmin, nmax): builds and
 * uploads the power table for nmin (cl_sieve.cpp:790-866), sizes the factor
 * buffer (result_cap = 0: the reference's 1e6, or 3e7 when pmin < 2^32,
 * cl_sieve.cpp:591-595), clears the counters (clearresult.cl). */
int fs_search_begin(fs_ctx *ctx, uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax,
                    uint32_t result_cap);
/* Queue one p-segment [low, high): getsegprimes -> (first segment: power
 * table check) -> setup -> iterate -> check, all on the stream, no host
 * synchronisation (cl_sieve.cpp:1142-1230). */
int fs_search_segment(fs_ctx *ctx, uint64_t low, uint64_t high);
/* Wait for the queued work, copy out the hits found since the last collect
 * (unsorted) and the sums, then clear them (getResults' device half,
 * cl_sieve.cpp:439-483, and clearresult.cl).  Returns FS_E_OVERFLOW,
 * FS_E_VALIDATION or FS_E_TABLE when the device flagged one. */
int fs_search_collect(fs_ctx *ctx, fs_factor *out, uint64_t cap, uint64_t *nfactors,
                      uint64_t *raw_sum, uint64_t *primecount, uint32_t *flags);
/* Wait for the queued segments and report how many factor records the next
 * fs_search_collect will return (so a caller can size its buffer); clears
 * nothing.  No counterpart in the reference, whose result buffer has a fixed
 * size (numresults). */
int fs_search_pending(fs_ctx *ctx, uint64_t *nfactors);
/* Convenience: queue segments of width seg_width (0: automatic) over
 * [low, high). */
int fs_search_range(fs_ctx *ctx, uint64_t low, uint64_t high, uint64_t seg_width);
/* Capacity the context reserves for one segment of the given width. */
uint64_t fs_candidate_capacity(uint64_t low, uint64_t high);

/* ---- batches of uneven jobs (one persistent launch) ------------------------ */
typedef struct {
    uint64_t pmin, pmax;   /* p in [pmin, pmax) */
    uint32_t nmin, nmax;   /* n in [nmin, nmax) */
} fs_job;

typedef struct {
    uint64_t raw_sum;      /* sum of (s6 + s7) over the job's candidates, mod 2^64 */
    uint64_t primecount;   /* candidates of the job */
    uint64_t nhits;        /* hits of the job before the 2-PRP filter */
    uint32_t flags;        /* FS_FLAG_* of the job */
    uint32_t pad;
} fs_job_result;

/* Prepare a batch: build every job's setup plan, size its candidate buffer
 * and capture the whole batch -- counter clears, one candidate launch per job
 * and one persistent sieve launch whose blocks take (job, 1024-candidate) tiles
 * from a global queue, heaviest jobs first -- into a CUDA graph.  Replaces any
 * previous batch of the context.  Each job's results are bit-identical to a
 * search of that job alone.  No counterpart in the reference, which runs one
 * range per process. */
int fs_batch_prepare(fs_ctx *ctx, const fs_job *jobs, uint32_t njobs, uint32_t hitcap);
/* Replay the batch graph on the context's stream (asynchronous). */
int fs_batch_launch(fs_ctx *ctx);
/* Wait, then copy per-job results (in the caller's job order) and the hits;
 * each hit's pad word holds its job index.  Returns FS_E_OVERFLOW or
 * FS_E_VALIDATION when a job flagged one. */
int fs_batch_collect(fs_ctx *ctx, fs_job_result *results, fs_factor *hits, uint64_t hitcap, uint64_t *nhits);
/* Free the batch's device memory and graph. */
int fs_batch_release(fs_ctx *ctx);

/* ---- measured launch sizing (cl_sieve.cpp:617-718, 1158-1227) -------------- */
/* The reference times one generator launch and scales a segment's p-range to
 * 1 ms of it (profileGPU), then times one setup and one iterate launch and
 * scales their work to 10-50 ms; it prints the result as
 * "c:%u u:%u t:%u r:%u p:%u s:%u n:%u".  fs_autotune times whole segment
 * searches of a sample of the real workload (its first p-values, the real
 * n-range) for each launch shape -- candidates per thread (sieve_variant 3 or
 * 5), blocks per SM (1x, 2x, 4x the resident ones), threads per block (256 or
 * 128), n-steps per launch (all, or halves) -- applies the fastest to the
 * context and sizes a segment to about target_ms (<= 0: 1000) of kernel time
 * at the measured rate.  The samples together take about a tenth of the
 * run's work; a run too short for that keeps the default shape (nothing is
 * timed, shapes_tried = 0).  The choice is cached in the text file cache_path
 * (NULL: no cache) under the GPU name, SM count and the workload's bucket
 * (log2 of the n-width, of p and of nmin); a cached choice is applied without
 * timing.  Runs its own sample searches on the context: call it before
 * fs_search_begin.  Results never depend on the shape. */
typedef struct {
    fs_tuning tuning;            /* the shape chosen, now the context's (fs_get_tuning form) */
    uint64_t seg_width;          /* p-width of one segment (the reference's range, r:) */
    uint64_t seg_capacity;       /* candidate slots such a segment reserves (psize, p:) */
    uint32_t setup_words;        /* setup-plan words one launch multiplies per candidate (sstep, s:) */
    uint32_t steps_per_launch;   /* n-steps one launch walks (nstep, n:) */
    double rate;                 /* (p,n) steps/s of the chosen shape on the sample; 0 when not timed */
    uint32_t shapes_tried;       /* shapes timed (0: from the cache, or a run too small to sample) */
    uint32_t from_cache;         /* 1 when the choice came from cache_path */
} fs_tune_result;
int fs_autotune(fs_ctx *ctx, uint64_t pmin, uint64_t pmax, uint32_t nmin, uint32_t nmax, double target_ms,
                const char *cache_path, fs_tune_result *out);
/* The tile size of the batch kernel (fs_tuning.batch_tile_candidates: 1024,
 * 2048 or 4096 candidates) for a job mix: each size is timed on the mix with
 * every p-range narrowed scale_down times (0: 16), the fastest is applied to
 * the context and cached under the GPU and a hash of the job list.  Call it
 * before fs_batch_prepare; it releases any prepared batch.  *tile_out gets the
 * size, *ms_out the timed batch-kernel milliseconds (0 from the cache). */
int fs_autotune_batch(fs_ctx *ctx, const fs_job *jobs, uint32_t njobs, uint32_t scale_down, const char *cache_path,
                      uint32_t *tile_out, double *ms_out);

/* ---- serving: continuous batching of search requests ----------------------- */
/* No counterpart in the reference.  Requests queue on the host; each
 * fs_serve_round() admits queued jobs while a slot is free and the device
 * keeps mem_reserve bytes free (cudaMemGetInfo), gives every working job an
 * equal share of round_budget -- starting residues for its next candidates or
 * the next chunk of its n-walk over all of them, residues staying in its
 * device buffer between rounds -- runs all of it as one persistent launch,
 * waits, and retires finished jobs.  A job's result equals a search of that
 * job alone. */
typedef struct {
    uint32_t max_active;     /* jobs resident on the device at once (<= 4096) */
    uint32_t hitcap;         /* hit records one round can hold */
    uint64_t round_budget;   /* (p,n) steps of work per round; 0: 3e10 (about 20 ms) */
    uint64_t mem_reserve;    /* device bytes admission leaves free */
} fs_serve_config;

typedef struct {
    int64_t id;              /* as given to fs_serve_submit */
    uint64_t raw_sum;        /* sum of (s6 + s7) over the job's candidates */
    uint64_t primecount;     /* candidates */
    uint64_t nhits;          /* hits (before the 2-PRP filter), at hits[hit_offset...] */
    uint32_t flags;          /* FS_FLAG_* */
    uint32_t pad;
    double t_submit, t_admit, t_done;   /* fs_clock() seconds */
    uint64_t hit_offset;
} fs_served;

double fs_clock(void);       /* steady clock, seconds */
int fs_serve_create(fs_ctx *ctx, const fs_serve_config *cfg);
int fs_serve_submit(fs_ctx *ctx, const fs_job *job, int64_t id);
/* One round (blocks until its GPU work is done); reports jobs on the device
 * and jobs still queued. */
int fs_serve_round(fs_ctx *ctx, uint32_t *n_active, uint32_t *n_queued);
/* Pop up to cap finished jobs, copying their hits into hits[0..hitcap). */
int fs_serve_poll(fs_ctx *ctx, fs_served *out, uint32_t cap, uint32_t *n, fs_factor *hits, uint64_t hitcap,
                  uint64_t *nhits);
/* Rounds run, (p,n) walk steps served, setup work queued (in walk-step
 * units: 2.7 per Montgomery product) and CUDA-event time of the drained
 * round kernels, so far. */
int fs_serve_stats(fs_ctx *ctx, uint64_t *rounds, uint64_t *served_steps, double *setup_units, double *kernel_ms);
int fs_serve_destroy(fs_ctx *ctx);

/* ---- stage-level kernels on caller device buffers ------------------------ */
/* getsegprimes (getsegprimes.cl:170-239): append the candidates of
 * [low, high) to d_cand at slot d_ctr->ncand (the reference's
 * g_primecount[0]).  Only the first `cap` slots are written. */
int fs_getsegprimes(fs_ctx *ctx, uint64_t low, uint64_t high, uint64_t *d_cand, uint32_t cap,
                    fs_counters *d_ctr);
/* Walk state of the stage-level calls below.  d_residue holds
 * FS_WALK_STATE_WORDS(cap) u64 words: the residues s6 = n! * 2^64 mod p of
 * the cap candidates, then, as cap uint32 values starting at word cap, the n
 * each residue stands at.  The reference keeps that n in each candidate's
 * record as s7 = n * 2^64 mod p, advanced by 2^64 once per step
 * (getsegprimes.cl:214-228, iterate.cl:67-68); fs_check derives s7 from it. */
#define FS_WALK_STATE_WORDS(cap) ((uint64_t)(cap) + ((uint64_t)(cap) + 1) / 2)

/* setup (setup.cl:49-103): residue i = nstart! * 2^64 mod d_cand[i] for
 * i < min(d_ctr->ncand, cap), standing at n = nstart. */
int fs_setup(fs_ctx *ctx, const uint64_t *d_cand, uint32_t cap, fs_counters *d_ctr, uint32_t nstart,
             uint64_t *d_residue);
/* iterate (iterate.cl:54-80): walk every residue through the steps
 * n = nstart .. nend-1 (multiply by n+1, test for +-1), appending hits to
 * d_hits at d_ctr->nhits; each residue's n advances by nend - nstart. */
int fs_iterate(fs_ctx *ctx, const uint64_t *d_cand, uint32_t cap, fs_counters *d_ctr,
               uint64_t *d_residue, uint32_t nstart, uint32_t nend, fs_factor *d_hits,
               uint32_t hitcap);
/* check (check.cl:50-109): add sum(s6 + s7), s7 = n * 2^64 mod p for the n
 * each residue stands at, to d_ctr->raw_sum; set FS_FLAG_VALIDATION unless
 * every n equals nmax (the reference's nmax round trip, check.cl:67-78: a
 * skipped or repeated iterate range fails it); add the candidate count to
 * d_ctr->primecount. */
int fs_check(fs_ctx *ctx, const uint64_t *d_cand, uint32_t cap, fs_counters *d_ctr,
             const uint64_t *d_residue, uint32_t nmax);
/* Power-table self-check (verifyslow/verifypow/verifyreduce/verifyresult.cl):
 * compare nmin! from the table with the direct product modulo d_cand[0];
 * sets FS_FLAG_TABLE in d_ctr->flags on mismatch.  out2 (host, may be NULL)
 * receives {direct, table}. */
int fs_table_check(fs_ctx *ctx, const uint64_t *d_cand, fs_counters *d_ctr, uint32_t nmin,
                   uint64_t *out2);

/* The same check for a setup plan the caller placed in device memory (as
 * fs_setup_plan returns it; e.g. the plan handed to fs_segment_noalloc):
 * FS_FLAG_TABLE is set in d_ctr->flags when it does not multiply to nmin!.
 * d_words must not be NULL when nlayers > 0, even for a plan with no words
 * (n <= 2).  No counterpart in the reference, which only checks the table it
 * built itself (cl_sieve.cpp:903-907). */
int fs_plan_check(fs_ctx *ctx, const uint64_t *d_cand, fs_counters *d_ctr, uint32_t nmin, const uint64_t *d_words,
                  const uint32_t *d_layers4, uint32_t nlayers, uint64_t deficit, uint64_t *out2);

/* ---- measurement ---------------------------------------------------------- */
typedef struct {
    uint64_t launches;        /* kernels this context launched since the last reset */
    uint64_t sieve_launches;  /* of which setup/iterate/check kernels */
    uint64_t gen_launches;    /* of which candidate-generator kernels */
    double sieve_ms;          /* CUDA-event time of the sieve launches (timing on) */
    double gen_ms;            /* CUDA-event time of the generator launches (timing on) */
    uint64_t batch_launches;  /* batch graph replays */
    double batch_ms;          /* CUDA-event time of the batch graph replays (timing on) */
} fs_stats;
/* Record CUDA events around every generator and sieve launch on the
 * context's stream (the reference's profiled enqueue, simpleCL.c:501-550). */
int fs_set_timing(fs_ctx *ctx, int enable);
/* Read (and with timing on, wait for) the statistics since the last reset. */
int fs_get_stats(fs_ctx *ctx, fs_stats *out);
int fs_reset_stats(fs_ctx *ctx);

/* Dependency-free integer stream on every SM: kind 0 IMAD, 1 IMAD.WIDE,
 * 2 IMAD.HI, 3 LOP3 (warp-lane operations per second); and the sieve's own
 * arithmetic register-resident at full occupancy (units per second), the
 * ceilings of its roofline: 4 Montgomery products, 5 half-offset lazy
 * steps, 6 lazy 64-bit steps, 7 lazy 96-bit steps, 8 canonical 96-bit
 * steps, 9 generic Montgomery steps, 10 half-offset lazy 96-bit steps,
 * 11 32-bit half-offset steps, 12 shifted-window half-offset 64-bit steps,
 * 13 half-offset canonical 96-bit steps, 14 half-offset 64-bit steps with
 * the quotient on the FP32 pipe, 15 folding products modulo 2^63 + d,
 * 16 / 17 / 18 the float-quotient steps with a k_max-aware window (window
 * shift at least 32 / at most 32 / a 96-bit product), 19 the half-offset
 * 96-bit step for p >= 2^63 with that quotient.
 * iters in [1, 2^24]; for kinds 16-19 at most 147065, so that the
 * multipliers stay within those steps' bound 46 k_max < 7 2^23. */
int fs_bench_int_pipe(fs_ctx *ctx, uint32_t kind, uint32_t iters, double *ops_per_sec, double *ms);

/* The residue step a segment p in [plo, phi) with multipliers up to kmax
 * runs: 6 / 7 / 9 / 4 / 5 / 8 half-offset 32-bit / shifted-window 64-bit /
 * 64-bit with the quotient on the FP32 pipe / lazy 64-bit / lazy 96-bit /
 * canonical 96-bit, 10 / 11 / 12 half-offset with the FP32 quotient and a
 * window taken from kmax (64-bit product, window shift >= 32 / <= 32;
 * 96-bit product), 13 the half-offset canonical 96-bit step for p >= 2^63
 * with that quotient, 1 lazy 64-bit, 2 lazy 96-bit,
 * 3 canonical 96-bit, 0 chosen per candidate (mixed ranges, or multipliers
 * beyond the forms' limits: generic Montgomery).
 * No counterpart in the reference, whose one step is the Montgomery product. */
int fs_walk_step(uint64_t plo, uint64_t phi, uint32_t kmax);

/* The setup product a segment p in [plo, phi) uses with the default
 * four-candidate kernels and a 96-bit walk: 1 when every p is 2^63 + d with
 * 0 < d < 2^30 (a b mod p folded with 2^64 = -2d, no Montgomery reduction),
 * else 0 (Montgomery products).  The starting residue is the same either way.
 * No counterpart in the reference, whose setup uses Montgomery products. */
int fs_setup_form(uint64_t plo, uint64_t phi);

/* ---- host-side pieces (no GPU needed) -------------------------------------- */
/* Reference-format power table for n! (cl_sieve.cpp:773-838). */
int fs_power_table(uint32_t n, uint64_t *prime, uint32_t *exp, uint32_t *bit, uint32_t cap,
                   uint32_t *len);
/* The bit-layered setup plan the GPU uses for n!: words, layers as
 * {begin, end, dbl, 0} quadruples (from the top exponent bit down), total
 * R-deficit.  Layer b's words multiply to the odd primes whose Legendre
 * exponent has bit b set, packed best fit decreasing (each word starts from
 * the largest prime left and takes the largest that still fits below 2^64);
 * the setup squares between layers and doubles where bit b of the exponent
 * of 2 is set. */
int fs_setup_plan(uint32_t n, uint32_t chunks, uint64_t *words, uint64_t wcap, uint64_t *nwords,
                  uint32_t *layers4, uint32_t lcap, uint32_t *nlayers, uint64_t *deficit);
/* Chunk boundaries of the same plan: chunk c owns layers
 * [bounds[c], bounds[c+1]) and carries deficits[c] (both arrays chunks+1 /
 * chunks long). */
int fs_setup_plan_chunks(uint32_t n, uint32_t chunks, uint32_t *bounds, uint64_t *deficits);
/* Command-line numbers with the reference's suffixes (putil.c:18-116):
 * K/M/G/T/P x1000^k, e<d> x10^d, k/m/g/t/p x2^(10k), b<d> x2^d.
 * 0 ok, -1 unparsable, -2 outside [lo, hi]. */
int fs_parse_uint64(uint64_t *result, const char *str, uint64_t lo, uint64_t hi);
int fs_parse_uint(uint32_t *result, const char *str, uint32_t lo, uint32_t hi);
/* First number >= *start coprime to 30 and its wheel index (cl_sieve.cpp:360-419). */
int fs_find_wheel_offset(uint64_t *start, int32_t *index);
/* 7-base deterministic Miller-Rabin (verifyprime.c:105-141). */
int fs_is_prime(uint64_t p);
/* Slow CPU check that p | n! + c (verifyprime.c:146-173). */
int fs_verify_factor(uint64_t p, uint32_t n, int32_t c);
/* getResults' CPU half (cl_sieve.cpp:484-550): sort hits by (p, |n|),
 * verify each on `threads` CPU threads, drop hits whose p is not prime,
 * compact the kept ones to the front.  *checksum_add = sum of (n + c) over
 * kept hits (32-bit arithmetic as the reference).  Returns FS_E_VERIFY if
 * any hit fails verification. */
int fs_postprocess(fs_factor *f, uint64_t n, int threads, uint64_t *kept, uint64_t *checksum_add,
                   uint64_t *discarded);

/* ---- allocation-free segment search ---------------------------------------- */
/* No counterpart in the reference (it always allocated its buffers with
 * clCreateBuffer).  For callers that cannot call cudaMalloc -- code running
 * while a stream is being captured, services whose device memory all comes
 * from a pool they must not bypass, embedders that only lend preallocated
 * buffers -- this runs one p-segment [low, high) over n in [nmin, nmax)
 * exactly like fs_search_begin + fs_search_segment, but allocates nothing:
 *
 *   inputs   d_words / d_layers4 / nlayers / deficit: the setup plan for nmin
 *            as fs_setup_plan() returns it, copied by the caller into device
 *            memory it owns (layers as {begin, end, dbl, 0} quadruples);
 *   outputs  d_hits (hitcap records) and d_ctr, caller device memory: hits are
 *            appended at d_ctr->nhits, sum(s6+s7) added to d_ctr->raw_sum, the
 *            candidate count to d_ctr->primecount (clear d_ctr before the first
 *            call of a search, as fs_search_begin does);
 *   scratch  the candidate list, in a fixed device array of
 *            FS_NOALLOC_MAX_CANDIDATES entries (8 MiB) that every GPU loading
 *            this library holds until the process exits.
 *
 * The kernels and launch shapes are those fs_search_segment picks for the
 * same segment.  The range checks of fs_search_begin apply (nmin = 0,
 * nmin > nmax, low < nmin: FS_E_ARG).
 * A segment whose candidate bound (fs_candidate_capacity) exceeds that
 * maximum is rejected with FS_E_LIMIT before anything runs; split it.  The
 * first call on a device, with that device current, looks up the array's
 * device address and the launch geometry (no allocation); make that first
 * call before any stream capture.  Work is queued on `stream` (cudaStream_t,
 * NULL for the legacy default stream) and not waited for.  All calls share
 * the one array, which keeps the previous call's contents: calls whose work
 * overlaps on the GPU (other streams, other threads) race on it, so
 * serialize them. */
#define FS_NOALLOC_MAX_CANDIDATES (1u << 20)
int fs_segment_noalloc(uint64_t low, uint64_t high, uint32_t nmin, uint32_t nmax, const uint64_t *d_words,
                       const uint32_t *d_layers4, uint32_t nlayers, uint64_t deficit, fs_factor *d_hits,
                       uint32_t hitcap, fs_counters *d_ctr, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FACTSIEVE_H */
