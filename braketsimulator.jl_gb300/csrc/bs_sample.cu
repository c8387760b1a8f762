// Shot sampling.
//
// Reference (src/result_types.jl:56-80): below 30 qubits an alias table is built
// serially (make_alias_table!, :8-54) and each shot draws j uniform in 1..N and
// u uniform in [0,1); at 30 qubits and above StatsBase's inverse CDF is used
// (a linear scan of the running sum per shot).
//
// Here:
//  - bs_alias_build (BS_ALIAS_EXACT) restates the serial table construction
//    operation for operation, so that draws on a supplied (j, u) stream match the
//    reference bit for bit; the classification pass is parallel, the pairing loop
//    runs on one thread because every step depends on the previous comparison;
//  - bs_sample_direct / bs_sample use a two-level inverse CDF: per-block sums of
//    the probabilities (computed from the state on the fly, never materialised),
//    an FP64 scan of the block sums, then per shot a binary search over blocks and
//    a running-sum scan inside one block.
#include <algorithm>
#include <cstring>
#include <vector>
#include "bs_internal.h"
#include "bs_ff.cuh"
#include "bs_cdf.cuh"

namespace {

__global__ void __launch_bounds__(128) k_block_sums(const double2* __restrict__ st, int dm, int64_t dim,
                                                    double* __restrict__ bsum, double* __restrict__ cinc) {
    __shared__ float ch[kCpb], cl[kCpb];
    const int64_t b = blockIdx.x;
    block_chunk_sums(st, dm, dim, b, ch, cl, bsum + b, cinc + b * kCpb);
}

// inclusive prefix of the block sums, one CTA of 1024 threads (nb is at most 2^22): a serial sum
// over each thread's run of blocks, then a parallel scan of the 1024 run totals
__global__ void __launch_bounds__(1024) k_scan_blocks(const double* __restrict__ bsum, int64_t nb, double* __restrict__ incl) {
    __shared__ double part[1024];
    const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const int64_t b0 = threadIdx.x * per, b1 = std::min<int64_t>(nb, b0 + per);
    double s = 0.0;
    for (int64_t b = b0; b < b1; b++) s += bsum[b];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        const double v = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0.0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    double run = threadIdx.x ? part[threadIdx.x - 1] : 0.0;
    for (int64_t b = b0; b < b1; b++) { run += bsum[b]; incl[b] = run; }
}

// first index i with running sum >= t (StatsBase semantics), searching blocks first
__device__ int64_t cdf_find(const double2* st, int dm, int64_t dim, const double* incl, int64_t nb, double t) {
    int64_t lo = 0, hi = nb - 1;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (incl[mid] >= t) hi = mid; else lo = mid + 1;
    }
    double cw = (lo == 0) ? 0.0 : incl[lo - 1];
    int64_t i = lo * kBlk;
    const int64_t end = std::min<int64_t>(dim, (lo + 1) * kBlk);
    cw += prob_at(st, dm, dim, i);
    while (cw < t && i < end - 1) { i++; cw += prob_at(st, dm, dim, i); }
    if (cw < t && lo == nb - 1) return dim - 1;
    return i;
}

__global__ void k_sample_direct(const double2* __restrict__ st, int dm, int64_t dim, const double* __restrict__ incl,
                                int64_t nb, const double* __restrict__ u, double wsum, int64_t shots,
                                int64_t* __restrict__ out) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < shots; s += (int64_t)gridDim.x * blockDim.x) {
        double W = (wsum > 0.0) ? wsum : incl[nb - 1];
        out[s] = cdf_find(st, dm, dim, incl, nb, u[s] * W);
    }
}


// The same search by a whole warp: block by binary search over the block prefix sums, chunk by
// binary search over the block's chunk prefix sums, then 32 probabilities per step with a warp
// prefix sum and a ballot for the first running sum >= t.  The sums associate differently from a
// left-to-right scan, so only exact boundary ties can land on a neighbouring index.
__device__ int64_t cdf_find_warp(const double2* st, int dm, int64_t dim, const double* incl, const double* cinc,
                                 int64_t nb, double t) {
    const int lane = threadIdx.x & 31;
    int64_t lo = 0, hi = nb - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (incl[mid] >= t) hi = mid; else lo = mid + 1;
    }
    const double base = (lo == 0) ? 0.0 : incl[lo - 1];
    const double* ci = cinc + lo * kCpb;
    int clo = 0, chi = kCpb - 1;
    while (clo < chi) {
        const int mid = (clo + chi) >> 1;
        if (base + ci[mid] >= t) chi = mid; else clo = mid + 1;
    }
    double cw = base + (clo == 0 ? 0.0 : ci[clo - 1]);
    const int64_t end = std::min<int64_t>(dim, (lo + 1) * kBlk);
    for (int64_t c = lo * kBlk + (int64_t)clo * kChunk; c < end; c += kChunk) {
        const int64_t i = c + lane;
        double p = (i < end) ? prob_at(st, dm, dim, i) : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double v = __shfl_up_sync(0xffffffffu, p, o);
            if (lane >= o) p += v;
        }
        const unsigned hit = __ballot_sync(0xffffffffu, i < end && cw + p >= t);
        if (hit) return c + __ffs(hit) - 1;
        cw += __shfl_sync(0xffffffffu, p, 31);
    }
    return end - 1;
}

// one shot per warp; uniforms from a counter-based splitmix64 stream
__global__ void k_sample_rng(const double2* __restrict__ st, int dm, int64_t dim, const double* __restrict__ incl,
                             const double* __restrict__ cinc, int64_t nb, uint64_t seed, int64_t shots, int64_t* __restrict__ out) {
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; s < shots; s += warps) {
        const uint64_t r = splitmix64(seed ^ splitmix64((uint64_t)s));
        const double u = (double)(r >> 11) * 0x1.0p-53;
        const int64_t v = cdf_find_warp(st, dm, dim, incl, cinc, nb, u * incl[nb - 1]);
        if ((threadIdx.x & 31) == 0) out[s] = v;
    }
}

// States of at most one CDF block (dim <= kBlk): every CTA forms the block's chunk prefix sums in
// shared memory itself (the arithmetic of k_block_sums, so the same CDF), then its warps draw their
// shots as k_sample_rng does.  One launch instead of three.
__global__ void __launch_bounds__(128) k_sample_small(const double2* __restrict__ st, int dm, int64_t dim,
                                                      uint64_t seed, int64_t shots, int64_t* __restrict__ out) {
    __shared__ float ch[kCpb], cl[kCpb];
    __shared__ double s_cinc[kCpb], s_total;
    block_chunk_sums(st, dm, dim, 0, ch, cl, &s_total, s_cinc);
    const double total = 0.0 + s_total;   // the block-prefix scan's value for one block
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; s < shots; s += warps) {
        const uint64_t r = splitmix64(seed ^ splitmix64((uint64_t)s));
        const double u = (double)(r >> 11) * 0x1.0p-53;
        const int64_t v = cdf_find_warp(st, dm, dim, &s_total, s_cinc, 1, u * total);   // nb = 1: incl unread
        if ((threadIdx.x & 31) == 0) out[s] = v;
    }
}

// ---------------------------------------------------------------- alias table
__global__ void k_alias_scale(const double* __restrict__ p, int64_t n, double ac, double* __restrict__ ap,
                              int64_t* __restrict__ alias) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        ap[i] = __dmul_rn(p[i], ac);
        alias[i] = -1;
    }
}

// Serial pairing (src/result_types.jl:26-52).  larges/smalls hold indices in
// ascending order, as the reference's first loop pushes them.
__global__ void k_alias_serial(double* __restrict__ ap, int64_t* __restrict__ alias, int64_t n,
                               int64_t* __restrict__ larges, int64_t* __restrict__ smalls) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t kl = 0, ks = 0;
    for (int64_t i = 0; i < n; i++) {
        double ai = ap[i];
        if (ai > 1.0) larges[kl++] = i;
        else if (ai < 1.0) smalls[ks++] = i;
    }
    while (kl > 0 && ks > 0) {
        int64_t s = smalls[--ks];
        int64_t l = larges[--kl];
        alias[s] = l;
        double al = __dadd_rn(__dsub_rn(ap[l], 1.0), ap[s]);
        ap[l] = al;
        if (al > 1.0) larges[kl++] = l;
        else smalls[ks++] = l;
    }
    for (int64_t i = 0; i < ks; i++) ap[smalls[i]] = 1.0;
}

__global__ void k_sample_alias(const double* __restrict__ ap, const int64_t* __restrict__ alias, int64_t n,
                               const int64_t* __restrict__ j, const double* __restrict__ u, int64_t shots,
                               int64_t* __restrict__ out, int* __restrict__ bad) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < shots; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t jj = j[s];
        if (jj < 0 || jj >= n) { atomicOr(bad, 1); out[s] = -1; continue; }
        out[s] = (u[s] < ap[jj]) ? jj : alias[jj];
    }
}

__global__ void k_prob_any(const double2* __restrict__ st, int dm, int64_t dim, double* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = prob_at(st, dm, dim, i);
}

int grid(int64_t work, int threads) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, 152 * 8));
}

// Scratch layout: bsum[nb] | incl[nb] | cinc[nb * kCpb] | extra_bytes for the caller (*extra).
int build_cdf(bs_sim* s, double** incl_out, double** cinc_out, int64_t* nb_out, int64_t extra_bytes = 0,
              void** extra = nullptr) {
    const int64_t dim = (int64_t)1 << s->n;
    const int64_t nb = (dim + kBlk - 1) / kBlk;
    const int64_t cdf_bytes = (2 * nb + nb * kCpb) * 8;
    int rc = bs_ensure_scratch(s, cdf_bytes + extra_bytes + 64);
    if (rc) return rc;
    double* bsum = (double*)s->scratch;
    double* incl = bsum + nb;
    double* cinc = incl + nb;
    k_block_sums<<<(unsigned)nb, 128, 0, s->stream>>>((const double2*)s->state, (s->kind == BS_KIND_DM ? 1 : 0) | (s->precision == BS_PREC_C64 ? 2 : 0), dim, bsum, cinc);
    k_scan_blocks<<<1, 1024, 0, s->stream>>>(bsum, nb, incl);
    *incl_out = incl;
    if (cinc_out) *cinc_out = cinc;
    *nb_out = nb;
    if (extra) *extra = (char*)s->scratch + ((cdf_bytes + 15) & ~(int64_t)15);
    return bs_cuda_check(s, cudaGetLastError(), "cdf");
}

int alias_alloc(bs_sim* s, int64_t n) {
    if (s->alias_len >= n && s->alias_ap) return BS_OK;
    if (s->alias_ap) cudaFree(s->alias_ap);
    if (s->alias_ix) cudaFree(s->alias_ix);
    s->alias_ap = nullptr;
    s->alias_ix = nullptr;
    s->alias_len = 0;
    int rc = bs_cuda_check(s, cudaMalloc(&s->alias_ap, (size_t)n * 8), "alias allocation");
    if (rc) return rc;
    rc = bs_cuda_check(s, cudaMalloc(&s->alias_ix, (size_t)n * 8), "alias allocation");
    if (rc) return rc;
    s->alias_len = n;
    return BS_OK;
}

int alias_from_device_probs(bs_sim* s, const double* dprobs, int64_t n, double wsum) {
    int rc = alias_alloc(s, n);
    if (rc) return rc;
    rc = bs_ensure_scratch(s, 2 * n * 8 + 16 * 8 + n * 8);
    if (rc) return rc;
    // dprobs may live in scratch: the scale kernel reads it before the stacks are written
    int64_t* larges = (int64_t*)((char*)s->scratch + n * 8);
    int64_t* smalls = larges + n;
    double ac = (double)n / wsum;
    k_alias_scale<<<grid(n, 256), 256, 0, s->stream>>>(dprobs, n, ac, s->alias_ap, s->alias_ix);
    k_alias_serial<<<1, 32, 0, s->stream>>>(s->alias_ap, s->alias_ix, n, larges, smalls);
    rc = bs_cuda_check(s, cudaGetLastError(), "alias build");
    if (rc) return rc;
    s->alias_valid = true;
    return BS_OK;
}

}  // namespace

extern "C" {

int bs_alias_build(bs_sim* s, double wsum, unsigned flags) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (flags & ~BS_ALIAS_PARALLEL) return bs_fail(s, BS_ERR_INVALID_ARG, "unknown alias flags");
    const int64_t dim = (int64_t)1 << s->n;
    const int mode = (s->kind == BS_KIND_DM ? 1 : 0) | (s->precision == BS_PREC_C64 ? 2 : 0);
    int rc;
    if (flags & BS_ALIAS_PARALLEL) {
        // probabilities, then the parallel builder's work area 256 bytes further on; the builder
        // takes the exact weight total itself when wsum is not given
        rc = alias_alloc(s, dim);
        if (rc) return rc;
        const int64_t pbytes = (dim * 8 + 255) & ~(int64_t)255;
        rc = bs_ensure_scratch(s, pbytes + bs_alias_parallel_scratch(dim));
        if (rc) return rc;
        double* p = (double*)s->scratch;
        k_prob_any<<<grid(dim, 256), 256, 0, s->stream>>>((const double2*)s->state, mode, dim, p);
        rc = bs_alias_parallel(s, p, dim, wsum, s->alias_ap, s->alias_ix, (char*)s->scratch + pbytes);
        if (rc) return rc;
        s->alias_valid = true;
        return BS_OK;
    }
    if (!(wsum > 0.0)) {
        // sum of the weights in float-float on the device (block sums + scan)
        double* incl = nullptr;
        int64_t nb = 0;
        rc = build_cdf(s, &incl, nullptr, &nb);
        if (rc) return rc;
        rc = bs_copy_out(s, &wsum, incl + nb - 1, 8, "weight sum");
        if (rc) return rc;
        if (!(wsum > 0.0)) return bs_fail(s, BS_ERR_STATE, "state has zero norm");
    }
    rc = bs_ensure_scratch(s, 3 * dim * 8 + 128);
    if (rc) return rc;
    double* p = (double*)s->scratch;
    k_prob_any<<<grid(dim, 256), 256, 0, s->stream>>>((const double2*)s->state, mode, dim, p);
    return alias_from_device_probs(s, p, dim, wsum);
}

int bs_alias_build_from(bs_sim* s, const double* probs, int64_t n, double wsum) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!probs || n < 1 || !(wsum > 0.0)) return bs_fail(s, BS_ERR_INVALID_ARG, "bad probabilities or wsum");
    int rc = bs_ensure_scratch(s, 3 * n * 8 + 128);
    if (rc) return rc;
    rc = bs_cuda_check(s, cudaMemcpyAsync(s->scratch, probs, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream), "alias probs");
    if (rc) return rc;
    return alias_from_device_probs(s, (const double*)s->scratch, n, wsum);
}

int bs_alias_table(bs_sim* s, double* ap_out, int64_t* alias_out, int64_t n) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!s->alias_valid || n > s->alias_len) return bs_fail(s, BS_ERR_STATE, "no alias table");
    int rc = BS_OK;
    if (ap_out) rc = bs_cuda_check(s, cudaMemcpyAsync(ap_out, s->alias_ap, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream), "alias copy");
    if (!rc && alias_out) rc = bs_cuda_check(s, cudaMemcpyAsync(alias_out, s->alias_ix, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream), "alias copy");
    if (rc) return rc;
    return bs_cuda_check(s, cudaStreamSynchronize(s->stream), "alias sync");
}

int bs_sample_alias(bs_sim* s, const int64_t* j, const double* u, int64_t shots, int64_t* out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!s->alias_valid) return bs_fail(s, BS_ERR_STATE, "alias table not built");
    if (shots < 0 || (shots > 0 && (!j || !u || !out))) return bs_fail(s, BS_ERR_INVALID_ARG, "bad stream");
    if (shots == 0) return BS_OK;
    // stream buffers after the alias scratch use: j, u, out, flag
    const int64_t bytes = shots * 24 + 64;
    void* buf = nullptr;
    int rc = bs_cuda_check(s, cudaMallocAsync(&buf, (size_t)bytes, s->stream), "sample buffers");
    if (rc) return rc;
    int64_t* dj = (int64_t*)buf;
    double* du = (double*)(dj + shots);
    int64_t* dout = (int64_t*)(du + shots);
    int* bad = (int*)(dout + shots);
    cudaMemcpyAsync(dj, j, (size_t)shots * 8, cudaMemcpyHostToDevice, s->stream);
    cudaMemcpyAsync(du, u, (size_t)shots * 8, cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(bad, 0, 4, s->stream);
    k_sample_alias<<<grid(shots, 256), 256, 0, s->stream>>>(s->alias_ap, s->alias_ix, s->alias_len, dj, du, shots, dout, bad);
    int hbad = 0;
    cudaMemcpyAsync(out, dout, (size_t)shots * 8, cudaMemcpyDeviceToHost, s->stream);
    cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, s->stream);
    cudaFreeAsync(buf, s->stream);
    rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), "sample alias");
    if (rc) return rc;
    if (hbad) return bs_fail(s, BS_ERR_INVALID_ARG, "index stream out of range");
    return BS_OK;
}

int bs_sample_direct(bs_sim* s, const double* u, int64_t shots, double wsum, int64_t* out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (shots < 0 || (shots > 0 && (!u || !out))) return bs_fail(s, BS_ERR_INVALID_ARG, "bad stream");
    if (shots == 0) return BS_OK;
    double* incl = nullptr;
    int64_t nb = 0;
    void* buf = nullptr;
    int rc = build_cdf(s, &incl, nullptr, &nb, shots * 16, &buf);
    if (rc) return rc;
    double* du = (double*)buf;
    int64_t* dout = (int64_t*)(du + shots);
    cudaMemcpyAsync(du, u, (size_t)shots * 8, cudaMemcpyHostToDevice, s->stream);
    const int64_t dim = (int64_t)1 << s->n;
    k_sample_direct<<<grid(shots, 128), 128, 0, s->stream>>>((const double2*)s->state, (s->kind == BS_KIND_DM ? 1 : 0) | (s->precision == BS_PREC_C64 ? 2 : 0), dim, incl, nb,
                                                               du, wsum, shots, dout);
    return bs_copy_out(s, out, dout, (size_t)shots * 8, "sample direct");
}

int bs_sample(bs_sim* s, uint64_t seed, int64_t shots, int64_t* out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (shots < 0 || (shots > 0 && !out)) return bs_fail(s, BS_ERR_INVALID_ARG, "bad shot buffer");
    if (shots == 0) return BS_OK;
    const int64_t dim = (int64_t)1 << s->n;
    const int mode = (s->kind == BS_KIND_DM ? 1 : 0) | (s->precision == BS_PREC_C64 ? 2 : 0);
    int64_t* dout;
    int rc;
    if (dim <= kBlk) {
        rc = bs_ensure_scratch(s, shots * 8);
        if (rc) return rc;
        dout = (int64_t*)s->scratch;
        const unsigned g = (unsigned)std::min<int64_t>(152, std::max<int64_t>(1, (shots + 15) / 16));
        k_sample_small<<<g, 128, 0, s->stream>>>((const double2*)s->state, mode, dim, seed, shots, dout);
    } else {
        double* incl = nullptr;
        double* cinc = nullptr;
        int64_t nb = 0;
        void* buf = nullptr;
        rc = build_cdf(s, &incl, &cinc, &nb, shots * 8, &buf);
        if (rc) return rc;
        dout = (int64_t*)buf;
        k_sample_rng<<<grid(shots * 32, 128), 128, 0, s->stream>>>((const double2*)s->state, mode, dim, incl, cinc, nb,
                                                                seed, shots, dout);
    }
    rc = bs_cuda_check(s, cudaGetLastError(), "sample");
    if (rc) return rc;
    return bs_copy_out(s, out, dout, (size_t)shots * 8, "sample");   // capture: out is the graph owner's pinned buffer
}

}  // extern "C"
