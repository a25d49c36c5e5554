// fs_sieve2.cu -- the fused sieve kernel, two candidates per thread (3 blocks per SM),
// one build per walk step.
#include "fs_walk.cuh"

namespace fs {

template <int MINB, int WALK, int PPT = 2>
static void launch_sieve_w(const SieveArgs& a, int setup, bool fin, int grid, cudaStream_t s, int t) {
    if (setup == SETUP_PLAN || setup == SETUP_PLAN_PM) {   // the pair kernels take every plan with Montgomery products
        if (fin) sieve_kernel<SETUP_PLAN, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
        else sieve_kernel<SETUP_PLAN, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
    } else if (setup == SETUP_PARTIALS) {
        if (fin) sieve_kernel<SETUP_PARTIALS, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
        else sieve_kernel<SETUP_PARTIALS, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
    } else {
        if (fin) sieve_kernel<SETUP_LOAD, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
        else sieve_kernel<SETUP_LOAD, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
    }
}

cudaError_t launch_sieve_pair(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s, int walk,
                              int threads) {
    if (threads != kSieveThreads && threads != kSieveThreads / 2) return cudaErrorInvalidValue;
    switch (walk) {
        case WALK_HF: launch_sieve_w<3, WALK_HF>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HG: launch_sieve_w<3, WALK_HG>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HGL: launch_sieve_w<3, WALK_HGL>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HG96: launch_sieve_w<3, WALK_HG96>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_H64: launch_sieve_w<3, WALK_H64>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_H96: launch_sieve_w<3, WALK_H96>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_H32: launch_sieve_w<3, WALK_H32>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HM: launch_sieve_w<3, WALK_HM>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_C96H: launch_sieve_w<3, WALK_C96H>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_C96G: launch_sieve_w<3, WALK_C96G>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_T64: launch_sieve_w<3, WALK_T64>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_L96: launch_sieve_w<3, WALK_L96>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_C96: launch_sieve_w<3, WALK_C96>(a, setup, final_chunk, grid, s, threads); break;
        default: launch_sieve_w<3, WALK_ANY>(a, setup, final_chunk, grid, s, threads); break;
    }
    return cudaGetLastError();
}

cudaError_t sieve_pair_occupancy(int* blocks_per_sm, int threads) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 3, WALK_ANY, 2>,
                                                         threads, 0);
}

}  // namespace fs
