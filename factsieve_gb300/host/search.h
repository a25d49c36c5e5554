// search.h -- the host driver of a FactSieve search over libfactsieve.so.
#pragma once
#include <stdint.h>

// Checkpoint record, byte-for-byte the reference's workStatus (cl_sieve.h:9-12):
// eight u64 then two u32, 72 bytes, written raw to stateA.ckp / stateB.ckp.
struct WorkStatus {
    uint64_t pmin, pmax, p, checksum, primecount, factorcount, last_trickle, state_sum;
    uint32_t nmin, nmax;
};
static_assert(sizeof(WorkStatus) == 72, "checkpoint record is 72 bytes");

struct SearchOptions {
    uint32_t threads = 2;            // -v: CPU threads for factor verification (main.cpp:195)
    bool test = false;               // -s: self test
    int device = 0;                  // CUDA device
    uint32_t numresults = 1000000;   // factor buffer (main.cpp:193, cl_sieve.cpp:593-595)
    uint64_t seg_width = 0;          // p-width of a GPU segment (0: measured, about segment_ms of kernel time)
    double segment_ms = 2000;        // kernel time a measured segment aims at
    double checkpoint_seconds = 60;  // time between checkpoints (cl_sieve.cpp:1125)
    bool write_state_a_next = true;  // A/B alternation of the checkpoint files
};

// The reference's range checks and messages (cl_sieve.cpp:561-589); 0 if valid.
int check_ranges(const WorkStatus& st);
// One search over st's ranges (cl_sieve.cpp:918-1270).  Returns 0 or an exit status.
int run_search(WorkStatus& st, SearchOptions& so);
// The reference's five-range self test (cl_sieve.cpp:1273-1391).
int run_self_test(WorkStatus& st, SearchOptions& so);
