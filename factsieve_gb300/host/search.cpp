// search.cpp -- host driver of one FactSieve search on libfactsieve.so.
//
// Keeps the reference's external behaviour (cl_sieve.cpp): range checks and
// messages, factors.txt, the A/B checkpoint pair with its additive checksum,
// a checkpoint every 60 s, CPU verification of every GPU hit on -v threads,
// the 2-PRP filter, the final checksum line and the five-range self test.
// The device work is queued through the C ABI one p-segment at a time.
#include "search.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cinttypes>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <vector>

#include "factsieve.h"

namespace {

const char* kResults = "factors.txt";
const char* kStateA = "stateA.ckp";
const char* kStateB = "stateB.ckp";

// stdout and stderr, as the reference does for every message in standalone mode
void both(const char* fmt, ...) {
    va_list a, b;
    va_start(a, fmt);
    va_copy(b, a);
    vfprintf(stdout, fmt, a);
    vfprintf(stderr, fmt, b);
    va_end(a);
    va_end(b);
    fflush(stdout);
}

void say(const char* fmt, ...) {
    va_list a;
    va_start(a, fmt);
    vfprintf(stdout, fmt, a);
    va_end(a);
    fflush(stdout);
}

uint64_t state_sum(const WorkStatus& s) {
    return s.pmin + s.pmax + s.p + s.checksum + s.primecount + s.factorcount + s.last_trickle + s.nmin + s.nmax;
}

// cl_sieve.cpp:100-129: write the other file each time, flip only on success
void write_state(WorkStatus& st, SearchOptions& so) {
    st.state_sum = state_sum(st);
    const char* name = so.write_state_a_next ? kStateA : kStateB;
    FILE* f = fopen(name, "wb");
    if (!f) {
        fprintf(stderr, "Cannot open %s !!!\n", name);
        return;
    }
    if (fwrite(&st, sizeof(WorkStatus), 1, f) != 1) {
        fprintf(stderr, "Cannot write checkpoint to file. Continuing...\n");
        fclose(f);
        return;
    }
    if (fclose(f) == 0) so.write_state_a_next = !so.write_state_a_next;
}

// One checkpoint file: 0 missing/bad, 1 good (cl_sieve.cpp:139-163).
int read_one(const char* name, const WorkStatus& want, WorkStatus* out) {
    FILE* f = fopen(name, "rb");
    if (!f) return 0;
    int ok = 1;
    if (fread(out, sizeof(WorkStatus), 1, f) != 1) {
        both("Cannot parse %s !!!\n", name);
        ok = 0;
    } else if (out->pmin != want.pmin || out->pmax != want.pmax || out->nmin != want.nmin ||
               out->nmax != want.nmax) {
        both("Invalid checkpoint file %s !!!\n", name);
        ok = 0;
    } else if (state_sum(*out) != out->state_sum) {
        both("Checksum error in %s !!!\n", name);
        ok = 0;
    }
    fclose(f);
    return ok;
}

// cl_sieve.cpp:132-222: the newer (larger p) of two good files wins.
int read_state(WorkStatus& st, SearchOptions& so) {
    WorkStatus a{}, b{};
    int ga = read_one(kStateA, st, &a), gb = read_one(kStateB, st, &b);
    if (ga && gb) {
        if (a.p > b.p)
            gb = 0;
        else
            ga = 0;
    }
    if (ga) {
        st = a;
        so.write_state_a_next = false;
        say("Resuming from checkpoint in %s\n", kStateA);
        return 1;
    }
    if (gb) {
        st = b;
        so.write_state_a_next = true;
        say("Resuming from checkpoint in %s\n", kStateB);
        return 1;
    }
    return 0;
}

void checkpoint(WorkStatus& st, SearchOptions& so) {
    write_state(st, so);
    say("Checkpoint, current p: %" PRIu64 "\n", st.p);
}

}  // namespace

int check_ranges(const WorkStatus& st) {
    if (st.pmin == 0 || st.pmax == 0) {
        say("-p and -P arguments are required\nuse -h for help\n");
        fprintf(stderr, "-p and -P arguments are required\n");
        return EXIT_FAILURE;
    }
    if (st.nmin == 0 || st.nmax == 0) {
        say("-n and -N arguments are required\nuse -h for help\n");
        fprintf(stderr, "-n and -N arguments are required\n");
        return EXIT_FAILURE;
    }
    if (st.nmin > st.nmax) {
        say("nmin <= nmax is required\nuse -h for help\n");
        fprintf(stderr, "nmin <= nmax is required\n");
        return EXIT_FAILURE;
    }
    if (st.pmin > st.pmax) {
        say("pmin <= pmax is required\nuse -h for help\n");
        fprintf(stderr, "pmin <= pmax is required\n");
        return EXIT_FAILURE;
    }
    if (st.pmin < st.nmin) {
        say("pmin must be >= nmin, there are no factors when p <= nmin\nuse -h for help\n");
        fprintf(stderr, "pmin must be >= nmin, there are no factors when p <= nmin\n");
        return EXIT_FAILURE;
    }
    return 0;
}

namespace {

// cl_sieve.cpp:557-613
int setup_search(WorkStatus& st, SearchOptions& so) {
    st.p = st.pmin;
    if (check_ranges(st)) return EXIT_FAILURE;
    if (st.pmin < 0xFFFFFFFFull) so.numresults = 30000000;
    both("Starting sieve at p: %" PRIu64 " n: %u\nStopping sieve at P: %" PRIu64 " N: %u\n", st.pmin, st.nmin,
         st.pmax, st.nmax);
    return 0;
}

bool factor_less(const fs_factor& a, const fs_factor& b) {
    if (a.p != b.p) return a.p < b.p;
    const int32_t na = a.nc < 0 ? -a.nc : a.nc, nb = b.nc < 0 ? -b.nc : b.nc;
    if (na != nb) return na < nb;
    return a.nc < b.nc;
}

// cl_sieve.cpp:439-554: fold the device sums in, then sort, CPU-verify,
// 2-PRP-filter and append the factors.
int get_results(fs_ctx* ctx, WorkStatus& st, SearchOptions& so, std::vector<fs_factor>& buf) {
    uint64_t nf = 0, raw = 0, pc = 0;
    uint32_t flags = 0;
    const int rc = fs_search_collect(ctx, buf.data(), buf.size(), &nf, &raw, &pc, &flags);
    st.primecount += pc;
    st.checksum += raw;
    if (flags & FS_FLAG_CAND_OVERFLOW) {
        both("error: gpu prime array overflow\n");
        return EXIT_FAILURE;
    }
    if (flags & FS_FLAG_TABLE) {
        both("error: power table verification failed\n");
        return EXIT_FAILURE;
    }
    if (flags & FS_FLAG_VALIDATION) {
        both("error: gpu validation failure\n");
        return EXIT_FAILURE;
    }
    if ((flags & FS_FLAG_HIT_OVERFLOW) || nf > buf.size()) {
        fprintf(stderr, "Error: number of results (%" PRIu64 ") overflowed array.\n", nf);
        return EXIT_FAILURE;
    }
    if (rc != FS_OK) {
        both("error: %s %s\n", fs_strerror(rc), fs_last_error(ctx));
        return EXIT_FAILURE;
    }
    if (nf == 0) return 0;
    say("processing %" PRIu64 " factors on CPU\n", nf);
    if (nf > 1) {
        say("sorting factors\n");
        std::sort(buf.begin(), buf.begin() + nf, factor_less);
    }
    say("Verifying factors on CPU...\n");
    std::atomic<int64_t> bad{-1};
    std::atomic<uint64_t> tested{0};
    double last = 0.0;
#pragma omp parallel for schedule(dynamic, 1) num_threads((int)so.threads)
    for (int64_t i = 0; i < (int64_t)nf; ++i) {
        const uint32_t fn = (uint32_t)(buf[i].nc < 0 ? -buf[i].nc : buf[i].nc);
        const int32_t fc = buf[i].nc < 0 ? -1 : 1;
        if (!fs_verify_factor(buf[i].p, fn, fc)) {
            int64_t expect = -1;
            bad.compare_exchange_strong(expect, i);
        }
        const uint64_t t = ++tested;
        if (omp_get_thread_num() == 0) {
            const double done = (double)(t + 1) / (double)nf * 100.0;
            if (done > last + 0.1) {
                last = done;
                printf("\r%.1f%%     ", done);
                fflush(stdout);
            }
        }
    }
    if (bad >= 0) {
        const fs_factor& f = buf[bad];
        const uint32_t fn = (uint32_t)(f.nc < 0 ? -f.nc : f.nc);
        both("\nCPU factor verification failed!  %" PRIu64 " is not a factor of %u!%+d\n", f.p, fn,
             f.nc < 0 ? -1 : 1);
        return EXIT_FAILURE;
    }
    fprintf(stderr, "Verified %" PRIu64 " factors.\n", nf);
    say("\rVerified %" PRIu64 " factors.\n", nf);
    FILE* res = fopen(kResults, "a");
    if (!res) {
        fprintf(stderr, "Cannot open %s !!!\n", kResults);
        return EXIT_FAILURE;
    }
    say("writing factors to %s\n", kResults);
    uint64_t last_good = 0;
    for (uint64_t i = 0; i < nf; ++i) {
        const uint64_t fp = buf[i].p;
        const uint32_t fn = (uint32_t)(buf[i].nc < 0 ? -buf[i].nc : buf[i].nc);
        const int32_t fc = buf[i].nc < 0 ? -1 : 1;
        // the GPU keeps base-2 strong probable primes; only prime p are factors
        if (fp == last_good || fs_is_prime(fp)) {
            last_good = fp;
            ++st.factorcount;
            if (fprintf(res, "%" PRIu64 " | %u!%+d\n", fp, fn, fc) < 0) {
                fprintf(stderr, "Cannot write to %s !!!\n", kResults);
                fclose(res);
                return EXIT_FAILURE;
            }
            st.checksum += (uint32_t)(fn + (uint32_t)fc);
        } else {
            both("discarded 2-PRP factor %" PRIu64 "\n", fp);
        }
    }
    if (fclose(res) != 0) {
        fprintf(stderr, "Cannot write to %s !!!\n", kResults);
        return EXIT_FAILURE;
    }
    return 0;
}

// cl_sieve.cpp:721-771
int finalize_results(const WorkStatus& st) {
    if (st.factorcount) {
        FILE* res = fopen(kResults, "r");
        if (!res) {
            fprintf(stderr, "Cannot open %s !!!\n", kResults);
            return EXIT_FAILURE;
        }
        char line[256];
        uint64_t lc = 0;
        while (fgets(line, sizeof(line), res)) ++lc;
        fclose(res);
        if (lc < st.factorcount) {
            both("ERROR: Missing factors in %s !!!\n", kResults);
            return EXIT_FAILURE;
        }
    }
    FILE* res = fopen(kResults, "a");
    if (!res) {
        fprintf(stderr, "Cannot open %s !!!\n", kResults);
        return EXIT_FAILURE;
    }
    int w = st.factorcount ? fprintf(res, "%016" PRIX64 "\n", st.checksum)
                           : fprintf(res, "no factors\n%016" PRIX64 "\n", st.checksum);
    if (w < 0 || fclose(res) != 0) {
        fprintf(stderr, "Cannot write to %s !!!\n", kResults);
        return EXIT_FAILURE;
    }
    return 0;
}

int truncate_results() {
    FILE* f = fopen(kResults, "w");
    if (!f) {
        fprintf(stderr, "Cannot open %s !!!\n", kResults);
        return EXIT_FAILURE;
    }
    fclose(f);
    return 0;
}

}  // namespace

int run_search(WorkStatus& st, SearchOptions& so) {
    if (setup_search(st, so)) return EXIT_FAILURE;
    // checkpoint and results file first (cl_sieve.cpp:998-1024): a finished
    // workunit or an unwritable factors.txt needs no device
    if (so.test) {
        if (truncate_results()) return EXIT_FAILURE;
    } else if (read_state(st, so)) {
        say("Current p: %" PRIu64 "\n", st.p);
        fprintf(stderr, "Resuming from checkpoint, current p: %" PRIu64 "\n", st.p);
        if (st.p == st.pmax) {
            both("Workunit complete.\n");
            return 0;
        }
    } else {
        if (truncate_results()) return EXIT_FAILURE;
        st.last_trickle = (uint64_t)time(nullptr);
    }

    fs_ctx* ctx = nullptr;
    int rc = fs_create(so.device, &ctx);
    if (rc) {
        both("Error: cannot open CUDA device %d: %s\n", so.device, fs_strerror(rc));
        return EXIT_FAILURE;
    }
    struct Closer {
        fs_ctx* c;
        ~Closer() { fs_destroy(c); }
    } closer{ctx};

    std::vector<fs_factor> buf(so.numresults);
    int sms = 0, clk = 0;
    uint64_t mem = 0;
    fs_device_info(ctx, &sms, &clk, &mem);
    // measured launch sizing (profileGPU and the setup/iterate retuning,
    // cl_sieve.cpp:617-718, 1158-1227), on what is left of the range
    fs_tune_result tr{};
    if ((rc = fs_autotune(ctx, st.p, st.pmax, st.nmin, st.nmax, so.segment_ms, getenv("FS_TUNING_CACHE"), &tr))) {
        both("error: %s %s\n", fs_strerror(rc), fs_last_error(ctx));
        return EXIT_FAILURE;
    }
    const uint64_t width = so.seg_width ? so.seg_width : tr.seg_width;
    both("c:1 u:%d t:%u r:%" PRIu64 " p:%" PRIu64 " s:%u n:%u\n", sms, so.threads, width,
         fs_candidate_capacity(st.p, st.p + width), tr.setup_words, tr.steps_per_launch);
    say("launch shape: %u candidates per thread, %u blocks of %u threads per SM%s, %.3g (p,n) steps/s measured%s\n",
        tr.tuning.sieve_variant == 5 ? 4u : 2u, tr.tuning.sieve_blocks_per_sm, tr.tuning.sieve_block_threads,
        tr.tuning.max_steps_per_launch ? ", n-range split" : "", tr.rate,
        tr.from_cache ? " (cached)" : (tr.shapes_tried ? "" : " (run too small to time: defaults)"));

    if ((rc = fs_search_begin(ctx, st.pmin, st.pmax, st.nmin, st.nmax, so.numresults))) {
        both("error: %s %s\n", fs_strerror(rc), fs_last_error(ctx));
        return EXIT_FAILURE;
    }
    const time_t t_start = time(nullptr);
    time_t t_progress = t_start, t_ckpt = t_start;
    const double irsize = 1.0 / (double)(st.pmax - st.pmin ? st.pmax - st.pmin : 1);
    while (st.p < st.pmax) {
        uint64_t stop = st.p + width;
        if (stop > st.pmax || stop < st.p) stop = st.pmax;
        const time_t now = time(nullptr);
        if (now - t_progress > 1) {
            say("Sieve Progress: %.1f%%\n", (double)(st.p - st.pmin) * irsize * 100.0);
            t_progress = now;
            if (difftime(now, t_ckpt) >= so.checkpoint_seconds) {
                if (get_results(ctx, st, so, buf)) return EXIT_FAILURE;
                checkpoint(st, so);
                t_ckpt = now;
            }
        }
        if ((rc = fs_search_segment(ctx, st.p, stop))) {
            both("error: %s %s\n", fs_strerror(rc), fs_last_error(ctx));
            return EXIT_FAILURE;
        }
        if ((rc = fs_synchronize(ctx))) {
            both("error: %s %s\n", fs_strerror(rc), fs_last_error(ctx));
            return EXIT_FAILURE;
        }
        st.p = stop;
    }
    st.p = st.pmax;
    say("Sieve Progress: %.1f%%\n", 100.0);
    if (get_results(ctx, st, so, buf)) return EXIT_FAILURE;
    checkpoint(st, so);
    if (finalize_results(st)) return EXIT_FAILURE;
    fprintf(stderr, "Sieve complete.\nfactors %" PRIu64 ", prime count %" PRIu64 "\n", st.factorcount,
            st.primecount);
    say("Sieve finished in %d sec.\n", (int)(time(nullptr) - t_start));
    say("factors %" PRIu64 ", prime count %" PRIu64 ", checksum %016" PRIX64 "\n", st.factorcount, st.primecount,
        st.checksum);
    return 0;
}

int run_self_test(WorkStatus& st, SearchOptions& so) {
    // the reference's five ranges and golden (factors, primes, checksum),
    // cl_sieve.cpp:1282-1364
    struct Case {
        uint64_t pmin, pmax;
        uint32_t nmin, nmax;
        uint64_t factors, primes, checksum;
    };
    static const Case cases[5] = {
        {100000000ull, 101000000ull, 1000000u, 2000000u, 1071, 54211, 0x000004F4F744CA97ull},
        {1000000000000ull, 1000010000000ull, 10000u, 2000000u, 3, 361727, 0x05052A2D65F3D735ull},
        {127ull, 100000ull, 127u, 1000000u, 42770, 9566, 0x0000000065C074F0ull},
        {2000000000000ull, 2000010000000ull, 2000000u, 6000000u, 3, 352866, 0x09C9742A908451EBull},
        {1000000000000ull, 1000001000000ull, 100000000u, 110000000u, 3, 36249, 0x0081056DC98DA092ull},
    };
    say("Beginning self test of 5 ranges.\n");
    const time_t t0 = time(nullptr);
    int good = 0;
    for (int i = 0; i < 5; ++i) {
        st = WorkStatus{};
        st.pmin = cases[i].pmin;
        st.pmax = cases[i].pmax;
        st.nmin = cases[i].nmin;
        st.nmax = cases[i].nmax;
        so.numresults = 1000000;
        const int rc = run_search(st, so);
        if (rc == 0 && st.factorcount == cases[i].factors && st.primecount == cases[i].primes &&
            st.checksum == cases[i].checksum) {
            say("test case %d passed.\n\n", i + 1);
            fprintf(stderr, "test case %d passed.\n", i + 1);
            ++good;
        } else {
            say("test case %d failed.\n\n", i + 1);
            fprintf(stderr, "test case %d failed.\n", i + 1);
        }
    }
    if (good == 5)
        both("All test cases completed successfully!\n");
    else
        both("Self test FAILED!\n");
    say("Elapsed time: %d sec.\n", (int)(time(nullptr) - t0));
    return good == 5 ? 0 : EXIT_FAILURE;
}
