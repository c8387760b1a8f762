// Density-matrix Kraus channels in the reference's own update rule.
//
// The reference applies sum_q K_q rho_blk K_q^dagger only to the blocks of the
// stored matrix whose row and column share every non-target bit
// (src/noise_kernels.jl:105-133 for 1 target, :135-168 for 2, :170-196 for k).
// BS_NOISE_REFERENCE reproduces exactly that set of updated elements; the full
// channel is BS_NOISE_PHYSICAL (tile sweeps, bs_plan.cpp).  The work here is
// O(2^n * 4^k) elements, negligible next to a 4^n sweep, so it runs in FP64.
#include <algorithm>
#include <cstring>
#include <vector>
#include "bs_internal.h"

namespace {

__device__ __forceinline__ double2 cmulD(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulDc(double2 a, double2 b) {   // a * conj(b)
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

__device__ __forceinline__ double2 to_d2(double2 v) { return v; }
__device__ __forceinline__ double2 to_d2(float2 v) { return make_double2(v.x, v.y); }
template <typename ST> __device__ __forceinline__ ST from_d2(double2 v);
template <> __device__ __forceinline__ double2 from_d2<double2>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 from_d2<float2>(double2 v) { return make_float2((float)v.x, (float)v.y); }

// ST: storage type of the density matrix (double2 for complex128, float2 for complex64)
template <int K, typename ST>
__global__ void k_kraus_ref(ST* __restrict__ S, int n, const int* __restrict__ eb, const double2* __restrict__ kr, int nk) {
    constexpr int D = 1 << K;
    const int64_t dim = (int64_t)1 << n;
    const int64_t nblk = dim >> K;
    int ord[K];
    for (int q = 0; q < K; q++) ord[q] = eb[q];
    for (int a = 0; a < K; a++)
        for (int b = a + 1; b < K; b++)
            if (ord[b] < ord[a]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
    for (int64_t ix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ix < nblk; ix += (int64_t)gridDim.x * blockDim.x) {
        int64_t p = ix;
        for (int q = 0; q < K; q++) {
            int64_t low = p & ((1LL << ord[q]) - 1);
            p = ((p >> ord[q]) << (ord[q] + 1)) | low;
        }
        int64_t idx[D];
        for (int m = 0; m < D; m++) {
            int64_t f = p;
            for (int q = 0; q < K; q++) if ((m >> q) & 1) f |= 1LL << eb[q];
            idx[m] = f;
        }
        double2 rho[D][D], acc[D][D];
        for (int i = 0; i < D; i++)
            for (int j = 0; j < D; j++) { rho[i][j] = to_d2(S[idx[i] + idx[j] * dim]); acc[i][j] = make_double2(0, 0); }
        for (int q = 0; q < nk; q++) {
            const double2* Kq = kr + (int64_t)q * D * D;
            double2 t[D][D];
            for (int i = 0; i < D; i++)
                for (int j = 0; j < D; j++) {
                    double2 s = make_double2(0, 0);
                    for (int l = 0; l < D; l++) { double2 v = cmulD(Kq[i * D + l], rho[l][j]); s.x += v.x; s.y += v.y; }
                    t[i][j] = s;
                }
            for (int i = 0; i < D; i++)
                for (int j = 0; j < D; j++) {
                    double2 s = make_double2(0, 0);
                    for (int l = 0; l < D; l++) { double2 v = cmulDc(t[i][l], Kq[j * D + l]); s.x += v.x; s.y += v.y; }
                    acc[i][j].x += s.x; acc[i][j].y += s.y;
                }
        }
        for (int i = 0; i < D; i++)
            for (int j = 0; j < D; j++) S[idx[i] + idx[j] * dim] = from_d2<ST>(acc[i][j]);
    }
}

// k >= 3: one CTA per block, the D x D block and a work copy in shared memory
template <typename ST>
__global__ void k_kraus_ref_big(ST* __restrict__ S, int n, int k, const int* __restrict__ eb,
                                const double2* __restrict__ kr, int nk) {
    extern __shared__ double2 sm[];
    const int D = 1 << k;
    const int64_t dim = (int64_t)1 << n;
    double2* rho = sm;
    double2* tmp = sm + D * D;
    double2* acc = sm + 2 * D * D;
    int64_t* idx = (int64_t*)(sm + 3 * D * D);
    if (threadIdx.x == 0) {
        int ord[BS_MAX_TARGETS];
        for (int q = 0; q < k; q++) ord[q] = eb[q];
        for (int a = 0; a < k; a++)
            for (int b = a + 1; b < k; b++)
                if (ord[b] < ord[a]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
        int64_t p = blockIdx.x;
        for (int q = 0; q < k; q++) {
            int64_t low = p & ((1LL << ord[q]) - 1);
            p = ((p >> ord[q]) << (ord[q] + 1)) | low;
        }
        for (int m = 0; m < D; m++) {
            int64_t f = p;
            for (int q = 0; q < k; q++) if ((m >> q) & 1) f |= 1LL << eb[q];
            idx[m] = f;
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
        int i = e / D, j = e % D;
        rho[e] = to_d2(S[idx[i] + idx[j] * dim]);
        acc[e] = make_double2(0, 0);
    }
    __syncthreads();
    for (int q = 0; q < nk; q++) {
        const double2* Kq = kr + (int64_t)q * D * D;
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
            int i = e / D, j = e % D;
            double2 s = make_double2(0, 0);
            for (int l = 0; l < D; l++) { double2 v = cmulD(Kq[i * D + l], rho[l * D + j]); s.x += v.x; s.y += v.y; }
            tmp[e] = s;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
            int i = e / D, j = e % D;
            double2 s = make_double2(0, 0);
            for (int l = 0; l < D; l++) { double2 v = cmulDc(tmp[i * D + l], Kq[j * D + l]); s.x += v.x; s.y += v.y; }
            acc[e].x += s.x; acc[e].y += s.y;
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
        int i = e / D, j = e % D;
        S[idx[i] + idx[j] * dim] = from_d2<ST>(acc[e]);
    }
}

}  // namespace

// A 1- or 2-target channel in the reference's update rule as a tile gate of a density-matrix sweep
// (kind 5): ebit[0..k-1] are the row endian bits of the targets (matrix bit j <-> ebit[j], the
// canonical order of bs_kraus_reference), ebit[k..2k-1] the column endian bits; mat holds the nk
// Kraus matrices, row-major D x D complex each.
int bs_lower_kraus_reference(bs_sim* s, const double* kraus, int nk, int k, const int* targets, unsigned flags,
                             std::vector<HostGate>& out) {
    if (s->kind != BS_KIND_DM) return bs_fail(s, BS_ERR_STATE, "noise needs a density-matrix simulator");
    if (k < 1 || k > 2) return bs_fail(s, BS_ERR_INVALID_ARG, "in-sweep reference channels take 1 or 2 targets");
    if (nk < 1 || !kraus) return bs_fail(s, BS_ERR_INVALID_ARG, "no Kraus matrices");
    uint64_t seen = 0;
    for (int i = 0; i < k; i++) {
        if (targets[i] < 0 || targets[i] >= s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "target qubit out of range");
        if ((seen >> targets[i]) & 1ULL) return bs_fail(s, BS_ERR_INVALID_ARG, "repeated qubit");
        seen |= 1ULL << targets[i];
    }
    std::vector<int> ct(targets, targets + k);
    if (flags & BS_GATE_SORTED_TARGETS) std::sort(ct.begin(), ct.end(), [](int a, int b) { return a > b; });
    else if (flags & BS_GATE_MSB_FIRST) std::reverse(ct.begin(), ct.end());
    HostGate g;
    g.kind = 5;
    g.k = k;
    for (int j = 0; j < k; j++) {
        g.ebit[j] = s->n - 1 - ct[(size_t)j];
        g.ebit[k + j] = g.ebit[j] + s->n;
    }
    const int D = 1 << k;
    g.mat.assign(kraus, kraus + (size_t)nk * D * D * 2);
    out.push_back(std::move(g));
    return BS_OK;
}

int bs_kraus_reference(bs_sim* s, const double* kraus, int nk, int k, const int* targets, unsigned flags) {
    if (s->kind != BS_KIND_DM) return bs_fail(s, BS_ERR_STATE, "noise needs a density-matrix simulator");
    if (k < 1 || k > BS_MAX_TARGETS) return bs_fail(s, BS_ERR_INVALID_ARG, "channel needs 1..10 targets");
    if (nk < 1) return bs_fail(s, BS_ERR_INVALID_ARG, "no Kraus matrices");
    uint64_t seen = 0;
    for (int i = 0; i < k; i++) {
        if (targets[i] < 0 || targets[i] >= s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "target qubit out of range");
        if ((seen >> targets[i]) & 1ULL) return bs_fail(s, BS_ERR_INVALID_ARG, "repeated qubit");
        seen |= 1ULL << targets[i];
    }
    // canonical: bit j <-> ct[j]
    std::vector<int> ct(targets, targets + k);
    if (flags & BS_GATE_SORTED_TARGETS) std::sort(ct.begin(), ct.end(), [](int a, int b) { return a > b; });
    else if (flags & BS_GATE_MSB_FIRST) std::reverse(ct.begin(), ct.end());
    std::vector<int> eb(k);
    for (int j = 0; j < k; j++) eb[j] = s->n - 1 - ct[j];
    const int D = 1 << k;
    const int64_t mat_doubles = (int64_t)nk * D * D * 2;
    const int64_t bytes = 256 + mat_doubles * 8;
    int rc = bs_ensure_plan(s, bytes);
    if (rc) return rc;
    std::vector<char> host((size_t)bytes, 0);
    std::memcpy(host.data(), eb.data(), sizeof(int) * (size_t)k);
    std::memcpy(host.data() + 256, kraus, (size_t)mat_doubles * 8);
    rc = bs_cuda_check(s, cudaMemcpyAsync(s->plan_buf, host.data(), (size_t)bytes, cudaMemcpyHostToDevice, s->stream), "kraus upload");
    if (rc) return rc;
    const int* d_eb = (const int*)s->plan_buf;
    const double2* d_k = (const double2*)((char*)s->plan_buf + 256);
    const int64_t nblk = ((int64_t)1 << s->n) >> k;
    const int threads = 128;
    const int blocks = (int)std::min<int64_t>((nblk + threads - 1) / threads, 152 * 16);
    auto run = [&](auto* S) -> int {
        using ST = std::remove_pointer_t<decltype(S)>;
        switch (k) {
            case 1: k_kraus_ref<1, ST><<<blocks, threads, 0, s->stream>>>(S, s->n, d_eb, d_k, nk); break;
            case 2: k_kraus_ref<2, ST><<<blocks, threads, 0, s->stream>>>(S, s->n, d_eb, d_k, nk); break;
            default: {
                size_t sm = (size_t)3 * D * D * sizeof(double2) + (size_t)D * sizeof(int64_t);
                if (sm > 200 * 1024) return bs_fail(s, BS_ERR_UNSUPPORTED, "channel too large");
                cudaFuncSetAttribute(k_kraus_ref_big<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
                k_kraus_ref_big<ST><<<(unsigned)nblk, 256, sm, s->stream>>>(S, s->n, k, d_eb, d_k, nk);
            }
        }
        return BS_OK;
    };
    rc = (s->precision == BS_PREC_C64) ? run((float2*)s->state) : run((double2*)s->state);
    if (rc) return rc;
    s->stats.kernel_launches++;
    return bs_cuda_check(s, cudaGetLastError(), "kraus launch");
}
