// Probabilities and the one-block cumulative distribution shared by the samplers: the float-float
// chunk sums and chunk prefix sums of a block of kBlk probabilities (bs_sample.cu) and the whole
// small-state run (bs_tile.cu), which therefore draw the same shots from the same state and seed.
#pragma once
#include <algorithm>
#include <cstdint>
#include "bs_ff.cuh"

namespace {

constexpr int kBlk = 4096;        // probabilities per CDF block
constexpr int kChunk = 32;        // probabilities per chunk (one warp step of a search)
constexpr int kCpb = kBlk / kChunk;   // chunks per block

// mode bit 0: density matrix (diagonal of the stored matrix); bit 1: complex64 storage
__device__ __forceinline__ double prob_at(const double2* st, int mode, int64_t dim, int64_t i) {
    const float2* st32 = reinterpret_cast<const float2*>(st);
    const bool c64 = (mode & 2) != 0;
    if (mode & 1) return c64 ? (double)st32[i * (dim + 1)].x : st[i * (dim + 1)].x;
    cff x = c64 ? Elem<true>::load(st32[i]) : load_c128(st[i]);
    ffacc a;
    acc_first(a, x.rh, x.rl, x.rh, x.rl);
    acc_add(a, x.ih, x.il, x.ih, x.il);
    ff r = acc_done(a);
    return ff2d(r.h, r.l);
}

__device__ __forceinline__ void ff_warp_sum(ffsum& a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_xor_sync(0xffffffffu, a.h, o), l = __shfl_xor_sync(0xffffffffu, a.l, o);
        fsum_add(a, h, l);
    }
}

// Per block of kBlk probabilities: its float-float sum (*bsum) and the inclusive prefix sums of its
// kCpb chunks relative to the block start (cinc[c]).  W warps (128 threads or more); warp w sums chunks w, w + W, ...
// with coalesced reads, warp 0 scans the chunk sums.  Ends with a barrier.
__device__ __forceinline__ void block_chunk_sums(const double2* __restrict__ st, int dm, int64_t dim, int64_t b,
                                                 float* ch, float* cl, double* bsum, double* cinc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = (int)(blockDim.x >> 5);
    for (int c = warp; c < kCpb; c += nw) {
        if (b * kBlk + (int64_t)c * kChunk >= dim) {   // past the end: an empty chunk sums to zero
            if (lane == 0) { ch[c] = 0.f; cl[c] = 0.f; }
            continue;
        }
        const int64_t i = b * kBlk + (int64_t)c * kChunk + lane;
        ffsum a{0.f, 0.f};
        if (i < dim) {
            const ff f = d2ff(prob_at(st, dm, dim, i));
            a.h = f.h;
            a.l = f.l;
        }
        ff_warp_sum(a);
        if (lane == 0) { ch[c] = a.h; cl[c] = a.l; }
    }
    __syncthreads();
    if (warp == 0) {
        // lane holds chunks 4 lane .. 4 lane + 3: local inclusive sums, then a warp scan of the totals
        ffsum loc[4];
        ffsum run{0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            fsum_add(run, ch[4 * lane + k], cl[4 * lane + k]);
            loc[k] = run;
        }
        ffsum pre = run;   // inclusive scan of the lane totals
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float h = __shfl_up_sync(0xffffffffu, pre.h, o), l = __shfl_up_sync(0xffffffffu, pre.l, o);
            if (lane >= o) fsum_add(pre, h, l);
        }
        ffsum off{__shfl_up_sync(0xffffffffu, pre.h, 1), __shfl_up_sync(0xffffffffu, pre.l, 1)};
        if (lane == 0) off = ffsum{0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            ffsum v = off;
            fsum_add(v, loc[k].h, loc[k].l);
            cinc[4 * lane + k] = ff2d(v.h, v.l);
        }
        if (lane == 31) *bsum = ff2d(pre.h, pre.l);
    }
    __syncthreads();
}

// The same sums from probabilities already formed (prob_at's values, e.g. kept in shared memory).
__device__ __forceinline__ void block_chunk_sums_p(const double* __restrict__ probs, int64_t dim, int64_t b,
                                                 float* ch, float* cl, double* bsum, double* cinc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = (int)(blockDim.x >> 5);
    for (int c = warp; c < kCpb; c += nw) {
        if (b * kBlk + (int64_t)c * kChunk >= dim) {   // past the end: an empty chunk sums to zero
            if (lane == 0) { ch[c] = 0.f; cl[c] = 0.f; }
            continue;
        }
        const int64_t i = b * kBlk + (int64_t)c * kChunk + lane;
        ffsum a{0.f, 0.f};
        if (i < dim) {
            const ff f = d2ff(probs[i]);
            a.h = f.h;
            a.l = f.l;
        }
        ff_warp_sum(a);
        if (lane == 0) { ch[c] = a.h; cl[c] = a.l; }
    }
    __syncthreads();
    if (warp == 0) {
        // lane holds chunks 4 lane .. 4 lane + 3: local inclusive sums, then a warp scan of the totals
        ffsum loc[4];
        ffsum run{0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            fsum_add(run, ch[4 * lane + k], cl[4 * lane + k]);
            loc[k] = run;
        }
        ffsum pre = run;   // inclusive scan of the lane totals
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float h = __shfl_up_sync(0xffffffffu, pre.h, o), l = __shfl_up_sync(0xffffffffu, pre.l, o);
            if (lane >= o) fsum_add(pre, h, l);
        }
        ffsum off{__shfl_up_sync(0xffffffffu, pre.h, 1), __shfl_up_sync(0xffffffffu, pre.l, 1)};
        if (lane == 0) off = ffsum{0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            ffsum v = off;
            fsum_add(v, loc[k].h, loc[k].l);
            cinc[4 * lane + k] = ff2d(v.h, v.l);
        }
        if (lane == 31) *bsum = ff2d(pre.h, pre.l);
    }
    __syncthreads();
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

}  // namespace
