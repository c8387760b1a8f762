// Reduced density matrices on the device.
//
// Reference: partial_trace (src/sv_simulator.jl:273-318 for a state vector,
// src/dm_simulator.jl:280-323 for a density matrix), reached through the
// DensityMatrix result type (src/result_types.jl:239-246); keeping every qubit of a state vector
// gives its density matrix psi psi^dagger (density_matrix, src/sv_simulator.jl:151-152).  The
// reference loops
// over the traced configurations on the host; here the sum runs in float-float on
// the device and only the 2^k x 2^k result is copied back.
//
//   state vector:   R[i, j] = sum_b psi[pad(i, b)] conj(psi[pad(j, b)])
//   density matrix: R[i, j] = sum_b S[pad(i, b), pad(j, b)]
//
// where pad(i, b) places the bits of i on the kept endian bits (ascending) and the
// bits of b on the traced ones.  The output index bit r belongs to the r-th smallest
// kept endian bit (the order the reference's loops produce before its own final
// permutation, which the host layer applies).  Output tiles of up to 64 x 64 entries,
// one CTA per (tile, chunk of b), float-float partial sums, then one reduction pass.
#include <algorithm>
#include <cstring>
#include <vector>
#include "bs_internal.h"
#include "bs_ff.cuh"

#define BS_RDM_MAX_KEEP 16   // a 2^16 x 2^16 complex128 result is 64 GiB

namespace {

constexpr int kRT = 256;    // threads per CTA
constexpr int kTS = 64;     // output tile edge
constexpr int kBB = 16;     // traced configurations staged per step

struct RdmDesc {
    int n_bits;            // vector bits (n for SV; the matrix side n for DM)
    int k;                 // kept bits
    int kbit[BS_RDM_MAX_KEEP];   // kept endian bits, ascending
    int64_t nb;            // traced configurations, 2^(n-k)
    int64_t per;           // configurations per chunk
    int ts;                // tile edge (<= 64)
    int tiles;             // tiles per side
};

__device__ __forceinline__ int64_t place(const RdmDesc& d, int64_t i, int64_t b) {
    // b's bits spread over the traced positions (zeros inserted at the kept bits), i's bits on the kept ones
    int64_t g = b;
    for (int q = 0; q < d.k; q++) {
        const int p = d.kbit[q];
        g = ((g >> p) << (p + 1)) | (g & (((int64_t)1 << p) - 1));
    }
    for (int q = 0; q < d.k; q++) g |= ((i >> q) & 1) << d.kbit[q];
    return g;
}

template <bool C64>
__device__ __forceinline__ cff ld(const void* st, int64_t g) {
    if (C64) return Elem<true>::load(reinterpret_cast<const float2*>(st)[g]);
    return load_c128(reinterpret_cast<const double2*>(st)[g]);
}

// mode 0: state vector, mode 1: density matrix.  Entry (ii, jj) of the CTA's tile for thread t:
// e = t + kRT * r, r < ts*ts/kRT (at most 16).
template <int MODE, bool C64>
__global__ void __launch_bounds__(kRT) k_rdm(const void* __restrict__ st, RdmDesc d, float4* __restrict__ partial) {
    __shared__ float4 xi[kBB][kTS], xj[kBB][kTS];
    const int tile = blockIdx.x, ti = tile / d.tiles, tj = tile % d.tiles;
    const int64_t b0 = (int64_t)blockIdx.y * d.per, b1 = std::min<int64_t>(d.nb, b0 + d.per);
    const int ts = d.ts, ne = ts * ts;
    ffacc ar[16], ai[16];
    bool first[16];
#pragma unroll
    for (int r = 0; r < 16; r++) first[r] = true;
    const int64_t dim = (int64_t)1 << d.n_bits;
    for (int64_t bb0 = b0; bb0 < b1; bb0 += kBB) {
        if (MODE == 0) {
            for (int idx = threadIdx.x; idx < kBB * ts; idx += kRT) {
                const int bb = idx / ts, e = idx % ts;
                const int64_t b = bb0 + bb;
                cff zi{0.f, 0.f, 0.f, 0.f}, zj{0.f, 0.f, 0.f, 0.f};
                if (b < b1) {
                    zi = ld<C64>(st, place(d, (int64_t)ti * ts + e, b));
                    zj = ld<C64>(st, place(d, (int64_t)tj * ts + e, b));
                }
                xi[bb][e] = make_float4(zi.rh, zi.rl, zi.ih, zi.il);
                xj[bb][e] = make_float4(zj.rh, zj.rl, zj.ih, zj.il);
            }
            __syncthreads();
        }
        const int nbb = (int)std::min<int64_t>(kBB, b1 - bb0);
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int e = threadIdx.x + kRT * r;
            if (e >= ne) break;
            const int ii = e / ts, jj = e % ts;
            for (int bb = 0; bb < nbb; bb++) {
                float xr, xrl, xim, xil, yr, yrl, yim, yil;
                if (MODE == 0) {
                    const float4 a = xi[bb][ii], c = xj[bb][jj];
                    // x * conj(y): re = xr yr + xi yi, im = xi yr - xr yi
                    xr = a.x; xrl = a.y; xim = a.z; xil = a.w;
                    yr = c.x; yrl = c.y; yim = c.z; yil = c.w;
                    if (first[r]) {
                        acc_first(ar[r], xr, xrl, yr, yrl);
                        acc_first(ai[r], xim, xil, yr, yrl);
                        first[r] = false;
                    } else {
                        acc_add(ar[r], xr, xrl, yr, yrl);
                        acc_add(ai[r], xim, xil, yr, yrl);
                    }
                    acc_add(ar[r], xim, xil, yim, yil);
                    acc_add(ai[r], -xr, -xrl, yim, yil);
                } else {
                    const int64_t b = bb0 + bb;
                    const int64_t gr = place(d, (int64_t)ti * ts + ii, b), gc = place(d, (int64_t)tj * ts + jj, b);
                    const cff v = ld<C64>(st, gr + gc * dim);
                    if (first[r]) {
                        acc_first(ar[r], v.rh, v.rl, 1.f, 0.f);
                        acc_first(ai[r], v.ih, v.il, 1.f, 0.f);
                        first[r] = false;
                    } else {
                        acc_add(ar[r], v.rh, v.rl, 1.f, 0.f);
                        acc_add(ai[r], v.ih, v.il, 1.f, 0.f);
                    }
                }
            }
        }
        if (MODE == 0) __syncthreads();
    }
    float4* out = partial + ((size_t)blockIdx.y * gridDim.x + tile) * (size_t)ne;
#pragma unroll
    for (int r = 0; r < 16; r++) {
        const int e = threadIdx.x + kRT * r;
        if (e >= ne) break;
        ff re{0.f, 0.f}, im{0.f, 0.f};
        if (!first[r]) { re = acc_done(ar[r]); im = acc_done(ai[r]); }
        out[e] = make_float4(re.h, re.l, im.h, im.l);
    }
}

// Sum the chunks' partial tiles into the 2^k x 2^k row-major complex128 result.
__global__ void k_rdm_reduce(const float4* __restrict__ partial, RdmDesc d, int chunks, double2* __restrict__ out) {
    const int64_t D = (int64_t)1 << d.k;
    const int ts = d.ts, ne = ts * ts, tiles2 = d.tiles * d.tiles;
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < D * D; o += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = o / D, j = o % D;
        const int tile = (int)((i / ts) * d.tiles + j / ts), e = (int)((i % ts) * ts + j % ts);
        ffsum sr{0.f, 0.f}, si{0.f, 0.f};
        for (int c = 0; c < chunks; c++) {
            const float4 v = partial[((size_t)c * tiles2 + tile) * (size_t)ne + e];
            fsum_add(sr, v.x, v.y);
            fsum_add(si, v.z, v.w);
        }
        out[o] = make_double2(ff2d(sr.h, sr.l), ff2d(si.h, si.l));
    }
}

}  // namespace

extern "C" int bs_reduced_density_matrix(bs_sim* s, int n_keep, const int* qubits, double* out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (n_keep < 1 || !qubits || !out) return bs_fail(s, BS_ERR_INVALID_ARG, "keep at least one qubit");
    if (n_keep > BS_RDM_MAX_KEEP) return bs_fail(s, BS_ERR_UNSUPPORTED, "at most 16 kept qubits (a 64 GiB result)");
    if (n_keep > s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "more kept qubits than the register has");
    uint64_t seen = 0;
    RdmDesc d{};
    d.n_bits = s->n;
    d.k = n_keep;
    std::vector<int> kb;
    for (int q = 0; q < n_keep; q++) {
        if (qubits[q] < 0 || qubits[q] >= s->n) return bs_fail(s, BS_ERR_INVALID_ARG, "qubit out of range");
        if ((seen >> qubits[q]) & 1ULL) return bs_fail(s, BS_ERR_INVALID_ARG, "repeated qubit");
        seen |= 1ULL << qubits[q];
        kb.push_back(s->n - 1 - qubits[q]);
    }
    std::sort(kb.begin(), kb.end());
    for (int q = 0; q < n_keep; q++) d.kbit[q] = kb[(size_t)q];
    d.nb = (int64_t)1 << (s->n - n_keep);
    const int64_t D = (int64_t)1 << n_keep;
    d.ts = (int)std::min<int64_t>(D, kTS);
    d.tiles = (int)(D / d.ts);
    const int tiles2 = d.tiles * d.tiles;
    // chunks of traced configurations: enough CTAs for the GPU, partial sums within 256 MiB
    const int64_t ne = (int64_t)d.ts * d.ts;
    int64_t chunks = std::max<int64_t>(1, std::min<int64_t>(d.nb, (152 * 8 + tiles2 - 1) / tiles2));
    chunks = std::min<int64_t>(chunks, std::max<int64_t>(1, (256LL << 20) / (16 * ne * tiles2)));
    chunks = std::min<int64_t>(chunks, 65535);
    d.per = (d.nb + chunks - 1) / chunks;
    chunks = (d.nb + d.per - 1) / d.per;
    const int64_t pbytes = chunks * tiles2 * ne * 16, obytes = D * D * 16;
    int rc = bs_ensure_scratch(s, pbytes + obytes + 256);
    if (rc) return rc;
    float4* partial = (float4*)s->scratch;
    double2* dout = (double2*)((char*)s->scratch + ((pbytes + 255) & ~255LL));
    const dim3 grid((unsigned)tiles2, (unsigned)chunks);
    const bool c64 = s->precision == BS_PREC_C64;
    if (s->kind == BS_KIND_DM) {
        if (c64) k_rdm<1, true><<<grid, kRT, 0, s->stream>>>(s->state, d, partial);
        else k_rdm<1, false><<<grid, kRT, 0, s->stream>>>(s->state, d, partial);
    } else {
        if (c64) k_rdm<0, true><<<grid, kRT, 0, s->stream>>>(s->state, d, partial);
        else k_rdm<0, false><<<grid, kRT, 0, s->stream>>>(s->state, d, partial);
    }
    k_rdm_reduce<<<(unsigned)std::min<int64_t>((D * D + 255) / 256, 152 * 8), 256, 0, s->stream>>>(partial, d, (int)chunks, dout);
    rc = bs_cuda_check(s, cudaGetLastError(), "reduced density matrix");
    if (rc) return rc;
    return bs_copy_out(s, out, dout, (size_t)obytes, "reduced density matrix");
}
