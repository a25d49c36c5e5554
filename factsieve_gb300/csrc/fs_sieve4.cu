// fs_sieve4.cu -- the fused sieve kernel, four candidates per thread (2 blocks per SM),
// one build per launch-wide walk step.
#include "fs_walk.cuh"

namespace fs {

template <int MINB, int WALK, int PPT = 2>
static void launch_sieve_w(const SieveArgs& a, int setup, bool fin, int grid, cudaStream_t s, int t) {
    if constexpr (WALK == WALK_C96H || WALK == WALK_C96G || WALK == WALK_C96) {
        if (setup == SETUP_PLAN_PM) {
            if (fin) sieve_kernel<SETUP_PLAN_PM, true, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
            else sieve_kernel<SETUP_PLAN_PM, false, MINB, WALK, PPT><<<grid, t, 0, s>>>(a);
            return;
        }
    }
    if (setup == SETUP_PLAN || setup == SETUP_PLAN_PM) {
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

cudaError_t launch_sieve_quad(const SieveArgs& a, int setup, bool final_chunk, int grid, cudaStream_t s, int walk,
                              int threads) {
    if (threads != kSieveThreads && threads != kSieveThreads / 2) return cudaErrorInvalidValue;
    switch (walk) {
        case WALK_HF: launch_sieve_w<2, WALK_HF, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HG: launch_sieve_w<2, WALK_HG, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HGL: launch_sieve_w<2, WALK_HGL, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HG96: launch_sieve_w<2, WALK_HG96, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_H64: launch_sieve_w<2, WALK_H64, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_H96: launch_sieve_w<2, WALK_H96, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_H32: launch_sieve_w<2, WALK_H32, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_HM: launch_sieve_w<2, WALK_HM, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_C96H: launch_sieve_w<2, WALK_C96H, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_C96G: launch_sieve_w<2, WALK_C96G, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_T64: launch_sieve_w<2, WALK_T64, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_L96: launch_sieve_w<2, WALK_L96, 4>(a, setup, final_chunk, grid, s, threads); break;
        case WALK_C96: launch_sieve_w<2, WALK_C96, 4>(a, setup, final_chunk, grid, s, threads); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t sieve_quad_occupancy(int* blocks_per_sm, int threads) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sieve_kernel<SETUP_PLAN, true, 2, WALK_H64, 4>,
                                                         threads, 0);
}

}  // namespace fs
