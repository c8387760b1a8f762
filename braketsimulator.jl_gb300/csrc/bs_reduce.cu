// Read-only reductions over the state: probabilities, Pauli-string and matrix
// expectations, marginal probabilities.
//
// Reference: probabilities src/sv_simulator.jl:271 and src/dm_simulator.jl:262;
// expectation src/sv_simulator.jl:240-248 (dot(psi, O psi) on a deep copy),
// src/dm_simulator.jl:253-260 (trace of O applied to S);
// marginal_probability src/result_types.jl:96-113.
// The reference copies the whole state and re-sweeps it per observable factor;
// here each Pauli term is one pair-read of the state and terms that flip the same
// bits share the read.  Every kernel is templated on the storage (complex128 or
// complex64); sums are carried in float-float, i.e. at FP64-level accuracy.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <vector>
#include "bs_internal.h"
#include "bs_ff.cuh"

namespace {

constexpr int kRThreads = 256;
constexpr int kMaxTermsPerPass = 8;

template <bool C64>
__device__ __forceinline__ double prob_of(const typename Elem<C64>::T& v) {
    cff x = Elem<C64>::load(v);
    ffacc a;
    acc_first(a, x.rh, x.rl, x.rh, x.rl);
    acc_add(a, x.ih, x.il, x.ih, x.il);
    ff r = acc_done(a);
    return ff2d(r.h, r.l);
}

template <bool C64>
__global__ void k_prob_sv(const typename Elem<C64>::T* __restrict__ psi, double* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = prob_of<C64>(psi[i]);
}

template <bool C64>
__global__ void k_prob_dm(const typename Elem<C64>::T* __restrict__ S, double* __restrict__ out, int64_t dim) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)S[i * (dim + 1)].x;
}

// One chunk [i0, i0 + cnt) of a result written to a file: mode 0 the state vector as complex128,
// 1 its probabilities, 2 the probabilities (diagonal) of a density matrix of side dim.
template <bool C64>
__global__ void k_file_chunk(const typename Elem<C64>::T* __restrict__ st, int mode, int64_t dim, int64_t i0,
                             int64_t cnt, void* __restrict__ out) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < cnt; j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = i0 + j;
        if (mode == 0) reinterpret_cast<double2*>(out)[j] = make_double2((double)st[i].x, (double)st[i].y);
        else if (mode == 1) reinterpret_cast<double*>(out)[j] = prob_of<C64>(st[i]);
        else reinterpret_cast<double*>(out)[j] = (double)st[i * (dim + 1)].x;
    }
}

struct TermSet {
    int nt;
    uint64_t zm[kMaxTermsPerPass];
    int ph[kMaxTermsPerPass];         // nY mod 4
    int slot[kMaxTermsPerPass];       // output slot
};

// block reduction of per-thread doubles into partial[idx]
__device__ void block_sum_store(double v, double* partial, int64_t idx) {
    __shared__ double red[kRThreads / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) partial[idx] = v;
    }
}

__device__ __forceinline__ void pauli_accumulate(ffsum* acc, const TermSet& ts, int64_t i, float wrh, float wrl,
                                                 float wih, float wil) {
    for (int t = 0; t < ts.nt; t++) {
        bool neg = __popcll((unsigned long long)i & ts.zm[t]) & 1;
        float vh, vl;
        switch (ts.ph[t]) {            // Re((-i)^ph * w)
            case 0: vh = wrh; vl = wrl; break;
            case 1: vh = wih; vl = wil; break;
            case 2: vh = -wrh; vl = -wrl; break;
            default: vh = -wih; vl = -wil; break;
        }
        if (neg) { vh = -vh; vl = -vl; }
        fsum_add(acc[t], vh, vl);
    }
}

// SV Pauli terms sharing flip mask xm.  Pairs (i, i^xm) with the top bit of xm
// clear contribute 2 Re(c(i) conj(psi_i) psi_{i^xm}); xm == 0 gives |psi_i|^2 * sign.
template <bool C64>
__global__ void __launch_bounds__(kRThreads) k_pauli_sv(const typename Elem<C64>::T* __restrict__ psi, int64_t n,
                                                        uint64_t xm, TermSet ts, double* __restrict__ partial, int n_slots) {
    ffsum acc[kMaxTermsPerPass];
    for (int t = 0; t < kMaxTermsPerPass; t++) acc[t] = {0.f, 0.f};
    const int64_t npairs = xm ? n / 2 : n;
    int hb = xm ? 63 - __clzll((long long)xm) : 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npairs; p += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = p;
        if (xm) { int64_t low = p & ((1LL << hb) - 1); i = ((p >> hb) << (hb + 1)) | low; }
        cff a = Elem<C64>::load(psi[i]);
        float wrh, wrl, wih, wil;
        if (xm) {
            cff b = Elem<C64>::load(psi[i ^ (int64_t)xm]);
            ffacc r, m;
            acc_first(r, a.rh, a.rl, b.rh, b.rl);
            acc_add(r, a.ih, a.il, b.ih, b.il);
            acc_first(m, a.rh, a.rl, b.ih, b.il);
            acc_add(m, -a.ih, -a.il, b.rh, b.rl);
            ff rr = acc_done(r), mm = acc_done(m);
            wrh = 2.f * rr.h; wrl = 2.f * rr.l; wih = 2.f * mm.h; wil = 2.f * mm.l;
        } else {
            ffacc r;
            acc_first(r, a.rh, a.rl, a.rh, a.rl);
            acc_add(r, a.ih, a.il, a.ih, a.il);
            ff rr = acc_done(r);
            wrh = rr.h; wrl = rr.l; wih = 0.f; wil = 0.f;
        }
        pauli_accumulate(acc, ts, i, wrh, wrl, wih, wil);
    }
    for (int t = 0; t < ts.nt; t++)
        block_sum_store(ff2d(acc[t].h, acc[t].l), partial, (int64_t)blockIdx.x * n_slots + ts.slot[t]);
}

// DM Pauli terms: E = sum_a Re(P[a, a^xm] S[a, a^xm]), S[r, c] at r + c*dim.
template <bool C64>
__global__ void __launch_bounds__(kRThreads) k_pauli_dm(const typename Elem<C64>::T* __restrict__ S, int64_t dim,
                                                        uint64_t xm, TermSet ts, double* __restrict__ partial, int n_slots) {
    ffsum acc[kMaxTermsPerPass];
    for (int t = 0; t < kMaxTermsPerPass; t++) acc[t] = {0.f, 0.f};
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < dim; a += (int64_t)gridDim.x * blockDim.x) {
        cff v = Elem<C64>::load(S[a + (a ^ (int64_t)xm) * dim]);
        pauli_accumulate(acc, ts, a, v.rh, v.rl, v.ih, v.il);
    }
    for (int t = 0; t < ts.nt; t++)
        block_sum_store(ff2d(acc[t].h, acc[t].l), partial, (int64_t)blockIdx.x * n_slots + ts.slot[t]);
}

__global__ void k_sum_partials(const double* __restrict__ partial, int nblocks, int n_slots, double* __restrict__ out) {
    // one block per slot; FP64 tree sum with a compensated leaf
    int slot = blockIdx.x;
    double s = 0.0, c = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        double y = partial[(int64_t)b * n_slots + slot] - c;
        double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) out[slot] = s;
    }
}

__device__ __forceinline__ double2 cmulD(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <bool C64>
__device__ __forceinline__ double2 ld2(const typename Elem<C64>::T& v) { return make_double2((double)v.x, (double)v.y); }

// <O> for a k-target matrix (FP64): SV sum_g x^H O x, DM sum_g sum_ab O[a,b] S[(a,g),(b,g)]
template <bool C64>
__global__ void __launch_bounds__(kRThreads) k_matrix_expect(const typename Elem<C64>::T* __restrict__ st, int nbits_q,
                                                             int k, const int* __restrict__ eb,
                                                             const double2* __restrict__ O, int dm,
                                                             double* __restrict__ partial) {
    const int D = 1 << k;
    const int64_t dim = (int64_t)1 << nbits_q;
    const int64_t ngroups = dim >> k;
    int ord[BS_MAX_TARGETS];
    for (int q = 0; q < k; q++) ord[q] = eb[q];
    for (int a = 0; a < k; a++)
        for (int b = a + 1; b < k; b++)
            if (ord[b] < ord[a]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
    double acc = 0.0;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < ngroups; g += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = g;
        for (int q = 0; q < k; q++) {
            int64_t low = p & ((1LL << ord[q]) - 1);
            p = ((p >> ord[q]) << (ord[q] + 1)) | low;
        }
        for (int a = 0; a < D; a++) {
            int64_t ia = p;
            for (int q = 0; q < k; q++) if ((a >> q) & 1) ia |= 1LL << eb[q];
            double2 xa = dm ? make_double2(0, 0) : ld2<C64>(st[ia]);
            for (int b = 0; b < D; b++) {
                int64_t ib = p;
                for (int q = 0; q < k; q++) if ((b >> q) & 1) ib |= 1LL << eb[q];
                double2 o = O[a * D + b];
                if (dm) {
                    double2 v = cmulD(o, ld2<C64>(st[ia + ib * dim]));
                    acc += v.x;
                } else {
                    double2 v = cmulD(o, ld2<C64>(st[ib]));   // O[a,b] x_b
                    acc += xa.x * v.x + xa.y * v.y;           // Re(conj(x_a) * v)
                }
            }
        }
    }
    block_sum_store(acc, partial, blockIdx.x);
}

// marginal probabilities: out[o] = sum of p_i over i whose target bits spell o
// (output bit j <-> j-th smallest endian target bit)
template <bool C64>
__global__ void __launch_bounds__(kRThreads) k_marginal(const typename Elem<C64>::T* __restrict__ st, int dm, int nbits_q,
                                                        int k, const int* __restrict__ eb_sorted,
                                                        double* __restrict__ partial) {
    extern __shared__ double hist[];
    const int D = 1 << k;
    const int64_t dim = (int64_t)1 << nbits_q;
    for (int o = threadIdx.x; o < D; o += blockDim.x) hist[o] = 0.0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
        double p = dm ? (double)st[i * (dim + 1)].x : prob_of<C64>(st[i]);
        int o = 0;
        for (int q = 0; q < k; q++) o |= (int)((i >> eb_sorted[q]) & 1) << q;
        atomicAdd(&hist[o], p);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < D; o += blockDim.x) partial[(int64_t)blockIdx.x * D + o] = hist[o];
}

// Marginals over more than 12 targets (no shared-memory histogram): out[o] = sum over the traced
// configurations b of p(place(o, b)), in float-float, per (output, chunk of b); WARP: one warp per
// output with its lanes over b (traced bits include the contiguous low ones), else one thread per
// output.  partial[c * D + o] holds chunk c's sum (hi, lo).
struct WideMarg {
    int nbits;          // vector bits (qubits)
    int k;              // kept bits
    int kbit[64];       // kept endian bits, ascending (output bit q <-> kbit[q])
    int64_t nb, per;    // traced configurations, per chunk
};
__device__ __forceinline__ int64_t wm_place(const WideMarg& d, int64_t o, int64_t b) {
    int64_t g = b;
    for (int q = 0; q < d.k; q++) {
        const int p = d.kbit[q];
        g = ((g >> p) << (p + 1)) | (g & (((int64_t)1 << p) - 1));
    }
    for (int q = 0; q < d.k; q++) g |= ((o >> q) & 1) << d.kbit[q];
    return g;
}
template <bool C64, bool WARP>
__global__ void __launch_bounds__(kRThreads) k_marginal_wide(const typename Elem<C64>::T* __restrict__ st, int dm,
                                                             WideMarg d, float2* __restrict__ partial) {
    const int64_t D = (int64_t)1 << d.k, dim = (int64_t)1 << d.nbits;
    const int64_t c = blockIdx.y;
    const int64_t b0 = c * d.per, b1 = std::min<int64_t>(d.nb, b0 + d.per);
    const int lanes = WARP ? 32 : 1;
    const int64_t o = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / lanes;
    const int lane = WARP ? (threadIdx.x & 31) : 0;
    if (o >= D) return;   // whole warps leave together (D is a multiple of the warp's outputs)
    ffsum acc{0.f, 0.f};
    for (int64_t b = b0 + lane; b < b1; b += lanes) {
        const int64_t i = wm_place(d, o, b);
        const double p = dm ? (double)st[i * (dim + 1)].x : prob_of<C64>(st[i]);
        const ff f = d2ff(p);
        fsum_add(acc, f.h, f.l);
    }
    if (WARP) {
        for (int off = 16; off > 0; off >>= 1) {
            const float h = __shfl_xor_sync(0xffffffffu, acc.h, off), l = __shfl_xor_sync(0xffffffffu, acc.l, off);
            fsum_add(acc, h, l);
        }
    }
    if (lane == 0) partial[c * D + o] = make_float2(acc.h, acc.l);
}
__global__ void k_marginal_wide_sum(const float2* __restrict__ partial, int64_t D, int64_t chunks, double* __restrict__ out) {
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < D; o += (int64_t)gridDim.x * blockDim.x) {
        ffsum acc{0.f, 0.f};
        for (int64_t c = 0; c < chunks; c++) {
            const float2 v = partial[c * D + o];
            fsum_add(acc, v.x, v.y);
        }
        out[o] = ff2d(acc.h, acc.l);
    }
}

int grid_for(int64_t work) {
    int64_t b = (work + kRThreads - 1) / kRThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 8));
}

template <bool C64>
void launch_pauli(bs_sim* s, int nb, int64_t dim, uint64_t xm, const TermSet& set, double* partial, int n_terms) {
    using T = typename Elem<C64>::T;
    if (s->kind == BS_KIND_SV)
        k_pauli_sv<C64><<<nb, kRThreads, 0, s->stream>>>((const T*)s->state, dim, xm, set, partial, n_terms);
    else
        k_pauli_dm<C64><<<nb, kRThreads, 0, s->stream>>>((const T*)s->state, dim, xm, set, partial, n_terms);
}

}  // namespace

// More than 12 targets: chunks of traced configurations so that about 152 x 2048 threads work,
// float-float partial sums per chunk, then one pass over the chunks.
static int marginal_wide(bs_sim* s, int k, const std::vector<int>& eb, double* host_out) {
    WideMarg d{};
    d.nbits = s->n;
    d.k = k;
    for (int q = 0; q < k; q++) d.kbit[q] = eb[(size_t)q];
    const int64_t D = (int64_t)1 << k;
    d.nb = (int64_t)1 << (s->n - k);
    const bool warp = d.nb >= 32 && eb[0] != 0;     // lanes over b where the low bits are traced
    const int64_t lanes = warp ? 32 : 1;
    int64_t chunks = std::max<int64_t>(1, std::min<int64_t>(d.nb / lanes, (152LL * 2048) / (D * lanes) + 1));
    chunks = std::min<int64_t>(chunks, 65535);
    d.per = (d.nb + chunks - 1) / chunks;
    chunks = (d.nb + d.per - 1) / d.per;
    const int64_t pbytes = (chunks * D * 8 + 255) & ~(int64_t)255;
    int rc = bs_ensure_scratch(s, pbytes + D * 8);
    if (rc) return rc;
    float2* partial = (float2*)s->scratch;
    double* out = (double*)((char*)s->scratch + pbytes);
    const dim3 grid((unsigned)((D * lanes + kRThreads - 1) / kRThreads), (unsigned)chunks);
    const int dm = s->kind == BS_KIND_DM;
    if (s->precision == BS_PREC_C64) {
        if (warp) k_marginal_wide<true, true><<<grid, kRThreads, 0, s->stream>>>((const float2*)s->state, dm, d, partial);
        else k_marginal_wide<true, false><<<grid, kRThreads, 0, s->stream>>>((const float2*)s->state, dm, d, partial);
    } else {
        if (warp) k_marginal_wide<false, true><<<grid, kRThreads, 0, s->stream>>>((const double2*)s->state, dm, d, partial);
        else k_marginal_wide<false, false><<<grid, kRThreads, 0, s->stream>>>((const double2*)s->state, dm, d, partial);
    }
    k_marginal_wide_sum<<<grid_for(D), kRThreads, 0, s->stream>>>(partial, D, chunks, out);
    rc = bs_cuda_check(s, cudaGetLastError(), "marginal");
    if (rc) return rc;
    return bs_copy_out(s, host_out, out, (size_t)D * 8, "marginal");
}

extern "C" {

int bs_probabilities(bs_sim* s, double* host_out, int64_t n) {
    if (!s) return BS_ERR_INVALID_ARG;
    const int64_t dim = (int64_t)1 << s->n;
    if (!host_out || n != dim) return bs_fail(s, BS_ERR_INVALID_ARG, "probability buffer length must be 2^n");
    int rc = bs_ensure_scratch(s, dim * 8);
    if (rc) return rc;
    double* d = (double*)s->scratch;
    const bool c64 = s->precision == BS_PREC_C64;
    if (s->kind == BS_KIND_SV) {
        if (c64) k_prob_sv<true><<<grid_for(dim), kRThreads, 0, s->stream>>>((const float2*)s->state, d, dim);
        else k_prob_sv<false><<<grid_for(dim), kRThreads, 0, s->stream>>>((const double2*)s->state, d, dim);
    } else {
        if (c64) k_prob_dm<true><<<grid_for(dim), kRThreads, 0, s->stream>>>((const float2*)s->state, d, dim);
        else k_prob_dm<false><<<grid_for(dim), kRThreads, 0, s->stream>>>((const double2*)s->state, d, dim);
    }
    return bs_copy_out(s, host_out, d, (size_t)dim * 8, "probabilities");
}

int bs_expectation_pauli(bs_sim* s, int n_terms, const uint64_t* xmask, const uint64_t* zmask, const double* coeffs,
                         double* out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (n_terms < 0 || (n_terms > 0 && (!xmask || !zmask || !out))) return bs_fail(s, BS_ERR_INVALID_ARG, "bad term arrays");
    if (n_terms == 0) return BS_OK;
    const int n = s->n;
    const uint64_t qmask = (n >= 64) ? ~0ULL : ((1ULL << n) - 1);
    // group by flip mask on endian bits
    std::map<uint64_t, std::vector<int>> groups;
    std::vector<uint64_t> zme(n_terms);
    std::vector<int> ph(n_terms);
    for (int t = 0; t < n_terms; t++) {
        if ((xmask[t] | zmask[t]) & ~qmask) return bs_fail(s, BS_ERR_INVALID_ARG, "Pauli mask names a qubit outside the register");
        uint64_t xe = 0, ze = 0;
        int ny = 0;
        for (int q = 0; q < n; q++) {
            bool x = (xmask[t] >> q) & 1ULL, z = (zmask[t] >> q) & 1ULL;
            if (x) xe |= 1ULL << (n - 1 - q);
            if (z) ze |= 1ULL << (n - 1 - q);
            if (x && z) ny++;
        }
        zme[t] = ze;
        ph[t] = ny & 3;
        groups[xe].push_back(t);
    }
    const int64_t dim = (int64_t)1 << n;
    const int nb = grid_for(dim);
    int rc = bs_ensure_scratch(s, ((int64_t)nb * n_terms + n_terms) * 8);
    if (rc) return rc;
    double* partial = (double*)s->scratch;
    double* res = partial + (int64_t)nb * n_terms;
    rc = bs_cuda_check(s, cudaMemsetAsync(partial, 0, (size_t)nb * n_terms * 8, s->stream), "clear partials");
    if (rc) return rc;
    for (auto& kv : groups) {
        const std::vector<int>& ts = kv.second;
        for (size_t c0 = 0; c0 < ts.size(); c0 += kMaxTermsPerPass) {
            TermSet set{};
            set.nt = (int)std::min<size_t>(kMaxTermsPerPass, ts.size() - c0);
            for (int j = 0; j < set.nt; j++) {
                int t = ts[c0 + (size_t)j];
                set.zm[j] = zme[t];
                set.ph[j] = ph[t];
                set.slot[j] = t;
            }
            if (s->precision == BS_PREC_C64) launch_pauli<true>(s, nb, dim, kv.first, set, partial, n_terms);
            else launch_pauli<false>(s, nb, dim, kv.first, set, partial, n_terms);
        }
    }
    k_sum_partials<<<n_terms, 256, 0, s->stream>>>(partial, nb, n_terms, res);
    if (s->capturing && coeffs) return bs_fail(s, BS_ERR_INVALID_ARG, "coefficients are applied after a captured graph runs");
    // during capture out is the graph owner's pinned buffer, filled on every replay
    rc = bs_copy_out(s, out, res, (size_t)n_terms * 8, "expectation");
    if (rc || s->capturing) return rc;
    if (coeffs)
        for (int t = 0; t < n_terms; t++) out[t] *= coeffs[t];
    return BS_OK;
}

int bs_expectation_matrix(bs_sim* s, const double* matrix, int k, const int* targets, unsigned flags, double* out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!matrix || !targets || !out || k < 1 || k > BS_MAX_TARGETS) return bs_fail(s, BS_ERR_INVALID_ARG, "bad observable");
    uint64_t seen = 0;
    for (int i = 0; i < k; i++) {
        if (targets[i] < 0 || targets[i] >= s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "target qubit out of range");
        if ((seen >> targets[i]) & 1ULL) return bs_fail(s, BS_ERR_INVALID_ARG, "repeated qubit");
        seen |= 1ULL << targets[i];
    }
    std::vector<int> ct(targets, targets + k);
    if (flags & BS_GATE_SORTED_TARGETS) std::sort(ct.begin(), ct.end(), [](int a, int b) { return a > b; });
    else if (flags & BS_GATE_MSB_FIRST) std::reverse(ct.begin(), ct.end());
    std::vector<int> eb(k);
    for (int j = 0; j < k; j++) eb[j] = s->n - 1 - ct[j];
    const int D = 1 << k;
    const int64_t dim = (int64_t)1 << s->n;
    const int nb = grid_for(dim >> k);
    const int64_t mbytes = (int64_t)D * D * 16;
    int rc = bs_ensure_plan(s, 256 + mbytes);
    if (rc) return rc;
    rc = bs_ensure_scratch(s, ((int64_t)nb + 1) * 8);
    if (rc) return rc;
    std::vector<char> host((size_t)(256 + mbytes), 0);
    std::memcpy(host.data(), eb.data(), sizeof(int) * (size_t)k);
    std::memcpy(host.data() + 256, matrix, (size_t)mbytes);
    rc = bs_cuda_check(s, cudaMemcpyAsync(s->plan_buf, host.data(), host.size(), cudaMemcpyHostToDevice, s->stream), "observable upload");
    if (rc) return rc;
    double* partial = (double*)s->scratch;
    const int* d_eb = (const int*)s->plan_buf;
    const double2* d_o = (const double2*)((char*)s->plan_buf + 256);
    const int dm = s->kind == BS_KIND_DM;
    if (s->precision == BS_PREC_C64)
        k_matrix_expect<true><<<nb, kRThreads, 0, s->stream>>>((const float2*)s->state, s->n, k, d_eb, d_o, dm, partial);
    else
        k_matrix_expect<false><<<nb, kRThreads, 0, s->stream>>>((const double2*)s->state, s->n, k, d_eb, d_o, dm, partial);
    k_sum_partials<<<1, 256, 0, s->stream>>>(partial, nb, 1, partial + nb);
    return bs_copy_out(s, out, partial + nb, 8, "expectation");
}

int bs_marginal_probabilities(bs_sim* s, int k, const int* targets, double* host_out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!targets || !host_out || k < 1 || k > s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "marginal needs 1..n targets");
    uint64_t seen = 0;
    for (int i = 0; i < k; i++) {
        if (targets[i] < 0 || targets[i] >= s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "target qubit out of range");
        if ((seen >> targets[i]) & 1ULL) return bs_fail(s, BS_ERR_INVALID_ARG, "repeated qubit");
        seen |= 1ULL << targets[i];
    }
    std::vector<int> eb(k);
    for (int j = 0; j < k; j++) eb[j] = s->n - 1 - targets[j];
    std::sort(eb.begin(), eb.end());
    if (k > 12) return marginal_wide(s, k, eb, host_out);
    const int D = 1 << k;
    const int64_t dim = (int64_t)1 << s->n;
    const int nb = grid_for(dim);
    int rc = bs_ensure_plan(s, 256);
    if (rc) return rc;
    rc = bs_ensure_scratch(s, ((int64_t)nb * D + D) * 8);
    if (rc) return rc;
    rc = bs_cuda_check(s, cudaMemcpyAsync(s->plan_buf, eb.data(), sizeof(int) * (size_t)k, cudaMemcpyHostToDevice, s->stream), "marginal upload");
    if (rc) return rc;
    double* partial = (double*)s->scratch;
    const int dm = s->kind == BS_KIND_DM;
    if (s->precision == BS_PREC_C64)
        k_marginal<true><<<nb, kRThreads, (size_t)D * 8, s->stream>>>((const float2*)s->state, dm, s->n, k, (const int*)s->plan_buf, partial);
    else
        k_marginal<false><<<nb, kRThreads, (size_t)D * 8, s->stream>>>((const double2*)s->state, dm, s->n, k, (const int*)s->plan_buf, partial);
    k_sum_partials<<<D, 256, 0, s->stream>>>(partial, nb, D, partial + (int64_t)nb * D);
    return bs_copy_out(s, host_out, partial + (int64_t)nb * D, (size_t)D * 8, "marginal");
}

// Large results straight from the device to a file (the reference writes result values above
// 1 MiB to temporary files for its external callers, _mmap_large_result_values,
// src/BraketSimulator.jl:410-428).  Chunks go through two pinned buffers, so that the copy of one
// overlaps the write of the other; no host copy of the whole result is made.
int bs_write_result_file(bs_sim* s, int what, const char* path, int64_t* bytes_out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!path) return bs_fail(s, BS_ERR_INVALID_ARG, "null path");
    if (what != BS_FILE_STATE && what != BS_FILE_PROBABILITIES) return bs_fail(s, BS_ERR_INVALID_ARG, "unknown result kind");
    if (what == BS_FILE_STATE && s->kind != BS_KIND_SV)
        return bs_fail(s, BS_ERR_INVALID_ARG, "the state-vector file needs a state-vector simulator");
    const bool c64 = s->precision == BS_PREC_C64, dm = s->kind == BS_KIND_DM;
    const int64_t dim = (int64_t)1 << s->n;
    const int64_t eb = what == BS_FILE_STATE ? 16 : 8, ch = ((int64_t)32 << 20) / eb;
    const bool direct = what == BS_FILE_STATE && !c64;   // complex128 state: plain copies
    if (!direct) {
        const int rc = bs_ensure_scratch(s, 2 * ch * eb);
        if (rc) return rc;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return bs_fail(s, BS_ERR_IO, std::string("cannot open ") + path);
    void* hb[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int rc = BS_OK;
    int64_t pending = -1;   // chunk whose copy is in flight in slot pending & 1
    for (int i = 0; i < 2 && !rc; i++) {
        rc = bs_cuda_check(s, cudaHostAlloc(&hb[i], (size_t)(ch * eb), cudaHostAllocDefault), "file staging");
        if (!rc) rc = bs_cuda_check(s, cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming), "file staging");
    }
    auto flush = [&](int64_t k) {
        const int slot = (int)(k & 1);
        const int64_t cnt = std::min<int64_t>(ch, dim - k * ch);
        int r = bs_cuda_check(s, cudaEventSynchronize(ev[slot]), "file copy");
        if (!r && std::fwrite(hb[slot], (size_t)eb, (size_t)cnt, f) != (size_t)cnt) r = bs_fail(s, BS_ERR_IO, std::string("write failed: ") + path);
        return r;
    };
    const int mode = what == BS_FILE_STATE ? 0 : (dm ? 2 : 1);
    for (int64_t k = 0; !rc && k * ch < dim; k++) {
        const int slot = (int)(k & 1);
        const int64_t i0 = k * ch, cnt = std::min<int64_t>(ch, dim - i0);
        const void* src;
        if (direct) {
            src = (const double2*)s->state + i0;
        } else {
            void* dst = (char*)s->scratch + (size_t)(slot * ch * eb);
            const int nb = grid_for(cnt);
            if (c64) k_file_chunk<true><<<nb, kRThreads, 0, s->stream>>>((const float2*)s->state, mode, dim, i0, cnt, dst);
            else k_file_chunk<false><<<nb, kRThreads, 0, s->stream>>>((const double2*)s->state, mode, dim, i0, cnt, dst);
            src = dst;
        }
        rc = bs_cuda_check(s, cudaMemcpyAsync(hb[slot], src, (size_t)(cnt * eb), cudaMemcpyDeviceToHost, s->stream), "file copy");
        if (!rc) rc = bs_cuda_check(s, cudaEventRecord(ev[slot], s->stream), "file copy");
        if (!rc && pending >= 0) rc = flush(pending);
        pending = k;
    }
    if (!rc && pending >= 0) rc = flush(pending);
    cudaStreamSynchronize(s->stream);
    if (std::fclose(f) != 0 && !rc) rc = bs_fail(s, BS_ERR_IO, std::string("close failed: ") + path);
    for (int i = 0; i < 2; i++) {
        if (hb[i]) cudaFreeHost(hb[i]);
        if (ev[i]) cudaEventDestroy(ev[i]);
    }
    if (!rc && bytes_out) *bytes_out = dim * eb;
    return rc;
}

}  // extern "C"
