// factsieve_main.cpp -- the drop-in command line (main.cpp of the reference).
//
//   factsieve -n <nmin> -N <nmax> -p <pmin> -P <pmax> [-v threads] [-s] [-h]
//
// Same options, limits, parse errors and help text as main.cpp:27-166; the
// device is CUDA device 0 (or FS_DEVICE), where the reference took the
// OpenCL GPU that BOINC assigned; -d/--device is accepted and ignored as
// there.
#include <getopt.h>
#include <omp.h>

#include <cstdio>
#include <cstdlib>

#include "factsieve.h"
#include "search.h"

namespace {

[[noreturn]] void help() {
    printf("Welcome to FactSieve, a GB300 CUDA program to find factors of factorial prime candidates of the form n!+-1\n");
    printf("Note that there are no factors for numbers of the form n!+-1 when p <= n because all primes <= n are factors of n!\n");
    printf("Program usage:\n");
    printf("-n #\t\t\tStart factorial n!+-1\n");
    printf("-N #\t\t\tEnd factorial N!+-1, range [-n, -N) exclusive, 127 <= -n <= n < -N < 2^31\n");
    printf("-p #\t\t\tStarting prime factor p\n");
    printf("-P #\t\t\tEnd prime factor P, range [-p, -P) exclusive, 127 <= -n <= -p <= p < -P < 2^64\n");
    printf("-v #\t\t\tOptional, specify the number of CPU threads used to verify factors.  Default is 2, max is 128.\n");
    printf("-s \t\t\tPerform self test to verify proper operation of the program with the current GPU.\n");
    printf("-h\t\t\tPrint this help\n");
    exit(EXIT_FAILURE);
}

const char* short_opts = "p:P:n:N:v:sd:h";
const struct option long_opts[] = {
    {"device", optional_argument, 0, 'd'},
    {"test", no_argument, 0, 's'},
    {0, 0, 0, 0},
};

int parse_option(int opt, const char* arg, WorkStatus& st, SearchOptions& so) {
    switch (opt) {
        case 'p': return fs_parse_uint64(&st.pmin, arg, 127, 0xFFFFFFFFFFFFFFFFull - 1);
        case 'P': return fs_parse_uint64(&st.pmax, arg, 128, 0xFFFFFFFFFFFFFFFFull);
        case 'n': return fs_parse_uint(&st.nmin, arg, 127, 0x7FFFFFFFu - 1);
        case 'N': return fs_parse_uint(&st.nmax, arg, 128, 0x7FFFFFFFu);
        case 'v': return fs_parse_uint(&so.threads, arg, 1, 128);
        case 's':
            so.test = true;
            fprintf(stderr, "Performing self test.\n");
            printf("Performing self test.\n");
            return 0;
        case 'd':
            return 0;
        case 'h':
        case '?':
            help();
    }
    return 0;
}

// main.cpp:103-166
void process_args(int argc, char* argv[], WorkStatus& st, SearchOptions& so) {
    int ind = -1, opt;
    while ((opt = getopt_long(argc, argv, short_opts, long_opts, &ind)) != -1) {
        switch (parse_option(opt, optarg, st, so)) {
            case 0:
                ind = -1;
                break;
            case -1:
                if (ind == -1) {
                    printf("%s: invalid argument -%c %s\n", argv[0], opt, optarg);
                    fprintf(stderr, "%s: invalid argument -%c %s\n", argv[0], opt, optarg);
                } else {
                    printf("%s: invalid argument --%s %s\n", argv[0], long_opts[ind].name, optarg);
                    fprintf(stderr, "%s: invalid argument --%s %s\n", argv[0], long_opts[ind].name, optarg);
                }
                exit(EXIT_FAILURE);
            case -2:
                if (ind == -1) {
                    printf("%s: out of range argument -%c %s\n", argv[0], opt, optarg);
                    fprintf(stderr, "%s: out of range argument -%c %s\n", argv[0], opt, optarg);
                } else {
                    printf("%s: out of range argument --%s %s\n", argv[0], long_opts[ind].name, optarg);
                    fprintf(stderr, "%s: out of range argument --%s %s\n", argv[0], long_opts[ind].name, optarg);
                }
                exit(EXIT_FAILURE);
            default:
                printf("unknown command line argument\n");
                exit(EXIT_FAILURE);
        }
    }
    // non-option arguments go to option zero, which accepts nothing
    while (optind < argc) {
        switch (parse_option(0, argv[optind], st, so)) {
            case 0:
                optind++;
                break;
            default:
                fprintf(stderr, "%s: invalid non-option argument %s\n", argv[0], argv[optind]);
                exit(EXIT_FAILURE);
        }
    }
}

}  // namespace

int main(int argc, char* argv[]) {
    WorkStatus st{};
    SearchOptions so{};
    fprintf(stderr, "\nFactSieve (GB300 CUDA, factsieve_gb300 %d) -- reference behaviour of FactSieve v1.6\n",
            fs_version());
    printf("\nFactSieve (GB300 CUDA, factsieve_gb300 %d) -- reference behaviour of FactSieve v1.6\n",
           fs_version());
    fprintf(stderr, "Command line: ");
    for (int i = 0; i < argc; i++) fprintf(stderr, "%s ", argv[i]);
    fprintf(stderr, "\n");

    process_args(argc, argv, st, so);
    omp_set_num_threads((int)so.threads);
    if (!so.test && check_ranges(st)) return EXIT_FAILURE;
    if (const char* d = getenv("FS_DEVICE")) so.device = atoi(d);
    if (const char* w = getenv("FS_SEGMENT_WIDTH")) so.seg_width = strtoull(w, nullptr, 0);
    if (const char* c = getenv("FS_CHECKPOINT_SECONDS")) so.checkpoint_seconds = atof(c);

    int ndev = 0;
    if (fs_device_count(&ndev) != FS_OK || ndev <= so.device) {
        // reported here; the run fails when it first needs the device, after
        // the checkpoint files are read (a finished workunit needs none)
        printf("No CUDA device %d available.\n", so.device);
        fprintf(stderr, "Error: no CUDA device %d available\n", so.device);
    } else {
        fprintf(stderr, "GPU Info:\n  CUDA device: \t\t%d of %d\n", so.device, ndev);
        printf("GPU Info:\n  CUDA device: \t\t%d of %d\n", so.device, ndev);
    }
    const int rc = so.test ? run_self_test(st, so) : run_search(st, so);
    return rc ? EXIT_FAILURE : EXIT_SUCCESS;
}
