// fs_multi.cu -- the batch kernel (many uneven jobs in one persistent launch)
// and the serving-round kernel (chunks of resident jobs), four candidates
// per thread with each job's walk step chosen at run time.
#include "fs_walk.cuh"

namespace fs {

// ============================================================ batches ====

// Persistent kernel over many uneven jobs.  A tile is kTileCandidates
// candidates of one job, four per thread; blocks take tiles from a global
// counter until the batch is done.  The host orders jobs by estimated work
// per candidate, heaviest first, so the long tiles start early and the tail
// is made of short ones.  Each job carries the walk step valid for its whole
// p-range, uniform over a tile.
constexpr int kBatchMaxJobs = 1024;

__global__ void __launch_bounds__(kSieveThreads, 2) batch_sieve_kernel(BatchArgs a) {
    __shared__ HitStage st;
    __shared__ u32 tile_end[kBatchMaxJobs];   // inclusive prefix sum of tiles per job
    __shared__ u32 s_tile;
    __shared__ u64 wsum[kSieveThreads / 32];
    __shared__ u32 wbad[kSieveThreads / 32];
    // each thread's checksum and validation count across a tile's passes, in
    // shared memory rather than registers (as in sieve_kernel; 0.9 % on the
    // config 4 mix)
    __shared__ u64 tsum_[kSieveThreads];
    __shared__ u32 tbad_[kSieveThreads];
    volatile u64* tsum = tsum_;
    volatile u32* tbad = tbad_;
    const u32 per_tile = a.tile_candidates;   // a multiple of kTileCandidates: walked in passes of four per thread
    if (threadIdx.x == 0) {
        st.n = 0;
        u32 acc = 0;
        for (u32 j = 0; j < a.njobs; ++j) {
            const u32 nc = a.ctr[j].ncand;
            const u32 n = nc < a.jobs[j].cap ? nc : a.jobs[j].cap;
            acc += (n + per_tile - 1) / per_tile;
            tile_end[j] = acc;
        }
    }
    __syncthreads();
    const u32 total = tile_end[a.njobs - 1];
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const u32 t = s_tile;
        __syncthreads();
        if (t >= total) break;
        // job of tile t: first j with tile_end[j] > t (binary search)
        u32 lo = 0, hi = a.njobs - 1;
        while (lo < hi) {
            const u32 mid = (lo + hi) >> 1;
            if (tile_end[mid] > t) hi = mid;
            else lo = mid + 1;
        }
        const u32 j = lo;
        const BatchJob& J = a.jobs[j];
        const u32 nc = a.ctr[j].ncand;
        const u32 n = nc < J.cap ? nc : J.cap;
        const u32 first = (t - (j ? tile_end[j - 1] : 0)) * per_tile;
        tsum[threadIdx.x] = 0;
        tbad[threadIdx.x] = 0;
        for (u32 pass = 0; pass < per_tile; pass += kTileCandidates) {
            const u32 i0 = first + pass + 4 * threadIdx.x;
            if (i0 >= n) break;
            const WalkOut o{&st, a.hits, a.hitcap, a.gctr, (int)j};
            Prime c[4];
            const u32 nreal = load_quad(J.cand, i0, n, c);
            u64 r[4];
            plan_product4(c, a.words, a.layers, J.layer_begin, J.layer_end, r);
#pragma unroll
            for (int h = 0; h < 4; ++h) r[h] = mont_mul(r[h], mont_pow(c[h].r2, J.deficit, c[h]), c[h].p, c[h].pinv);
            walk_quad_rt((int)J.walk, r, c, nreal, J.nstart, J.nend, o);
            // one launch walks the job's whole n-range: its residues stand at nend = the job's nmax
            u64 qsum = 0;
            u32 qbad = 0;
#pragma unroll
            for (int h = 0; h < 4; ++h)
                if ((u32)h < nreal) final_check(c[h], r[h], J.nend, J.nend, qsum, qbad);
            tsum[threadIdx.x] = tsum[threadIdx.x] + qsum;
            tbad[threadIdx.x] = tbad[threadIdx.x] + qbad;
        }
        u64 sum = tsum[threadIdx.x];
        u32 bad = tbad[threadIdx.x];
#pragma unroll
        for (int d = 16; d; d >>= 1) {
            sum += __shfl_xor_sync(0xffffffffu, sum, d);
            bad += __shfl_xor_sync(0xffffffffu, bad, d);
        }
        if ((threadIdx.x & 31) == 0) {
            wsum[threadIdx.x >> 5] = sum;
            wbad[threadIdx.x >> 5] = bad;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            u64 s = 0;
            u32 b = 0;
            for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
                s += wsum[w];
                b += wbad[w];
            }
            if (s) atomicAdd(&a.ctr[j].raw_sum, s);
            if (b) atomicOr(&a.ctr[j].flags, FLAG_VALIDATION);
        }
    }
    __syncthreads();
    const u32 nh = st.n < kHitStage ? st.n : kHitStage;
    if (nh) {
        __shared__ u32 gbase;
        if (threadIdx.x == 0) gbase = atomicAdd(&a.gctr->nhits, nh);
        __syncthreads();
        for (u32 k = threadIdx.x; k < nh; k += blockDim.x) {
            const u32 g = gbase + k;
            if (g < a.hitcap)
                a.hits[g] = st.buf[k];
            else
                atomicOr(&a.gctr->flags, FLAG_HIT_OVERFLOW);
        }
    }
}

// ============================================================ serving ====

// One round of the serving loop: a list of tiles, each up to PPT x 256
// candidates of one job in one phase (starting residues from the plan, a
// chunk of the walk, the final checksum), PPT candidates per thread, taken
// from a global counter by persistent blocks.  Residues live in each job's
// device buffer between rounds.  PPT = 4 (four chains per thread) is the
// throughput form; PPT = 2 puts a small round's candidates on twice as many
// SMs (lower latency when the GPU would otherwise idle).
template <int PPT>
__global__ void __launch_bounds__(kSieveThreads, PPT == 4 ? 2 : 3) serve_round_kernel(ServeArgs a) {
    __shared__ HitStage st;
    __shared__ u32 s_tile;
    __shared__ u64 wsum[kSieveThreads / 32];
    __shared__ u32 wbad[kSieveThreads / 32];
    if (threadIdx.x == 0) st.n = 0;
    __syncthreads();
    const u32 per_tile = PPT * kSieveThreads;
    const u32 ntiles = a.nchunks ? a.chunks[a.nchunks - 1].tile_end : 0;
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const u32 t = s_tile;
        __syncthreads();
        if (t >= ntiles) break;
        // chunk of tile t: first c with tile_end > t
        u32 lo = 0, hi = a.nchunks - 1;
        while (lo < hi) {
            const u32 mid = (lo + hi) >> 1;
            if (a.chunks[mid].tile_end > t) hi = mid;
            else lo = mid + 1;
        }
        const ServeChunk T = a.chunks[lo];
        const u32 tile0 = lo ? a.chunks[lo - 1].tile_end : 0;
        const u32 i0 = T.first + (t - tile0) * per_tile + PPT * threadIdx.x;
        const u32 end = T.first + T.count;
        u64 sum = 0;
        u32 bad = 0;
        if (i0 < end) {
            const WalkOut o{&st, a.hits, a.hitcap, a.gctr, (int)T.tag};
            if constexpr (PPT == 4) {
                Prime c[4];
                const u32 nreal = load_quad(T.cand, i0, end, c);
                u64 r[4];
                const bool setup = T.flags & SERVE_SETUP;
                if (setup) {
                    plan_product4(c, T.words, T.layers, T.layer_begin, T.layer_end, r);
#pragma unroll
                    for (int h = 0; h < 4; ++h)
                        r[h] = mont_mul(r[h], mont_pow(c[h].r2, T.deficit, c[h]), c[h].p, c[h].pinv);
                } else {
                    r[0] = T.residue[i0];
#pragma unroll
                    for (int h = 1; h < 4; ++h) r[h] = (u32)h < nreal ? T.residue[i0 + h] : r[0];
                }
                walk_quad_rt((int)T.walk, r, c, nreal, T.nstart, T.nend, o);
                const u32 steps = T.nend > T.nstart ? T.nend - T.nstart : 0;
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    if ((u32)h >= nreal) break;
                    // the n this candidate's residue stands at: its tag, advanced by the walk
                    const u32 nw = (setup ? T.nstart : T.walked[i0 + h]) + steps;
                    if (T.flags & SERVE_FINAL) {
                        final_check(c[h], r[h], nw, T.nmax, sum, bad);
                    } else {
                        T.residue[i0 + h] = r[h];
                        T.walked[i0 + h] = nw;
                    }
                }
            } else {
                const bool real_b = i0 + 1 < end;
                const Prime ca = make_prime(T.cand[i0]);
                const Prime cb = real_b ? make_prime(T.cand[i0 + 1]) : ca;
                u64 ra, rb;
                const bool setup = T.flags & SERVE_SETUP;
                if (setup) {
                    plan_product2(ca, cb, T.words, T.layers, T.layer_begin, T.layer_end, ra, rb);
                    ra = mont_mul(ra, mont_pow(ca.r2, T.deficit, ca), ca.p, ca.pinv);
                    rb = mont_mul(rb, mont_pow(cb.r2, T.deficit, cb), cb.p, cb.pinv);
                } else {
                    ra = T.residue[i0];
                    rb = real_b ? T.residue[i0 + 1] : ra;
                }
                walk_pair(ra, rb, ca, cb, real_b, T.nstart, T.nend, o);
                const u32 steps = T.nend > T.nstart ? T.nend - T.nstart : 0;
                const u32 nwa = (setup ? T.nstart : T.walked[i0]) + steps;
                const u32 nwb = real_b ? (setup ? T.nstart : T.walked[i0 + 1]) + steps : nwa;
                if (T.flags & SERVE_FINAL) {
                    final_check(ca, ra, nwa, T.nmax, sum, bad);
                    if (real_b) final_check(cb, rb, nwb, T.nmax, sum, bad);
                } else {
                    T.residue[i0] = ra;
                    T.walked[i0] = nwa;
                    if (real_b) {
                        T.residue[i0 + 1] = rb;
                        T.walked[i0 + 1] = nwb;
                    }
                }
            }
        }
        if (T.flags & SERVE_FINAL) {
#pragma unroll
            for (int d = 16; d; d >>= 1) {
                sum += __shfl_xor_sync(0xffffffffu, sum, d);
                bad += __shfl_xor_sync(0xffffffffu, bad, d);
            }
            if ((threadIdx.x & 31) == 0) {
                wsum[threadIdx.x >> 5] = sum;
                wbad[threadIdx.x >> 5] = bad;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                u64 s = 0;
                u32 b = 0;
                for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
                    s += wsum[w];
                    b += wbad[w];
                }
                if (s) atomicAdd(&T.ctr->raw_sum, s);
                if (b) atomicOr(&T.ctr->flags, FLAG_VALIDATION);
            }
        }
    }
    __syncthreads();
    const u32 nh = st.n < kHitStage ? st.n : kHitStage;
    if (nh) {
        __shared__ u32 gbase;
        if (threadIdx.x == 0) gbase = atomicAdd(&a.gctr->nhits, nh);
        __syncthreads();
        for (u32 k = threadIdx.x; k < nh; k += blockDim.x) {
            const u32 g = gbase + k;
            if (g < a.hitcap)
                a.hits[g] = st.buf[k];
            else
                atomicOr(&a.gctr->flags, FLAG_HIT_OVERFLOW);
        }
    }
}

// ============================================================== launches ===

cudaError_t launch_batch(const BatchArgs& a, int grid, cudaStream_t s) {
    if (a.njobs == 0 || a.njobs > (u32)kBatchMaxJobs || a.tile_candidates == 0 ||
        a.tile_candidates % kTileCandidates)
        return cudaErrorInvalidValue;
    batch_sieve_kernel<<<grid, kSieveThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t batch_occupancy(int* blocks_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, batch_sieve_kernel, kSieveThreads, 0);
}

int batch_max_jobs() { return kBatchMaxJobs; }

cudaError_t launch_serve_round(const ServeArgs& a, int grid, cudaStream_t s, int ppt) {
    if (ppt == 2) serve_round_kernel<2><<<grid, kSieveThreads, 0, s>>>(a);
    else serve_round_kernel<4><<<grid, kSieveThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t serve_occupancy(int* blocks_per_sm, int ppt) {
    if (ppt == 2)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, serve_round_kernel<2>, kSieveThreads, 0);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, serve_round_kernel<4>, kSieveThreads, 0);
}

}  // namespace fs
