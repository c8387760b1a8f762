// Adjoint-method gradients of <H> for parameterised circuits.
//
// No reference counterpart: BraketSimulator.jl declares AdjointGradient
// (src/results.jl:90-159) but rejects it at parse time (src/pragmas.jl:67-68).
// Algorithm (Jones & Gacon, arXiv:2009.02823): forward |psi_L>, |lambda> = H|psi_L>,
// then for l = L..1: gradient of gate l from <lambda| dU_l |psi_{l-1}>, and
// psi <- U_l^dag psi, lambda <- U_l^dag lambda.  Gates exp(-i theta G/2) with a
// Pauli-string generator G give dE/dtheta = Im <lambda|G|psi_l>; PhaseShift gives
// -2 Im <lambda|P1|psi_l>.
//
// Both backward states are swept together: one tile sweep loads the same tile of
// psi and lambda, applies the daggered gates of a run to both, and accumulates
// the inner products of the run's parameterised gates before applying them.
//
// Checkpoints: the forward pass runs in S segments and keeps psi after each of the
// first S-1; the backward pass, entering a segment, replaces the uncomputed psi by
// that checkpoint, so the rounding drift of uncomputation never spans more than
// one segment.  S comes from the handle's tuning (BS_TUNE_ADJ_SEGMENTS) or, by
// default, from the parameterised gate count and a quarter of the free device
// memory; when memory binds (an allocation fails) S is halved down to 1, pure
// uncomputation.
#include <algorithm>
#include <complex>
#include <cstring>
#include <vector>
#include "bs_internal.h"
#include "bs_ff.cuh"

namespace {

constexpr int kAThreads = 256;

struct PauliTerm {
    uint64_t xm, zm;     // endian masks
    int ph;              // nY mod 4
    float ch, cl;        // coefficient as float-float
};

__device__ __forceinline__ cff f4c(float4 v) { return {v.x, v.y, v.z, v.w}; }
__device__ __forceinline__ float4 c4f(const cff& c) { return make_float4(c.rh, c.rl, c.ih, c.il); }

// lambda_i = sum_t c_t (-i)^ph_t (-1)^popc(i & zm_t) psi_{i ^ xm_t}
// C64: complex64 storage; the arithmetic and the sums stay float-float either way.
template <bool C64>
__global__ void __launch_bounds__(kAThreads) k_pauli_sum(const typename Elem<C64>::T* __restrict__ psi,
                                                         typename Elem<C64>::T* __restrict__ lam, int64_t n,
                                                         const PauliTerm* __restrict__ terms, int nt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        ffacc ar{0.f, 0.f}, ai{0.f, 0.f};
        for (int t = 0; t < nt; t++) {
            PauliTerm p = terms[t];
            cff x = Elem<C64>::load(psi[i ^ (int64_t)p.xm]);
            int ph = p.ph + ((__popcll((unsigned long long)i & p.zm) & 1) ? 2 : 0);
            // (-i)^ph: multiply x by i^(4-ph)
            x = cmul_ipow(x, (4 - (ph & 3)) & 3);
            acc_add(ar, p.ch, p.cl, x.rh, x.rl);
            acc_add(ai, p.ch, p.cl, x.ih, x.il);
        }
        lam[i] = Elem<C64>::store(cdone(ar, ai));
    }
}

__device__ void block_sum2(double a, double b, double* out2) {
    __shared__ double ra[kAThreads / 32], rb[kAThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { ra[w] = a; rb[w] = b; }
    __syncthreads();
    if (w == 0) {
        a = (l < (int)(blockDim.x >> 5)) ? ra[l] : 0.0;
        b = (l < (int)(blockDim.x >> 5)) ? rb[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if (l == 0) { atomicAdd(out2, a); atomicAdd(out2 + 1, b); }
    }
}

// <a|b> (complex) into out2[0..1]
template <bool C64>
__global__ void __launch_bounds__(kAThreads) k_inner(const typename Elem<C64>::T* __restrict__ a,
                                                     const typename Elem<C64>::T* __restrict__ b, int64_t n,
                                                     double* __restrict__ out2) {
    ffsum sr{0.f, 0.f}, si{0.f, 0.f};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        cff x = Elem<C64>::load(a[i]), y = Elem<C64>::load(b[i]);
        ffacc r, m;
        acc_first(r, x.rh, x.rl, y.rh, y.rl);
        acc_add(r, x.ih, x.il, y.ih, y.il);
        acc_first(m, x.rh, x.rl, y.ih, y.il);
        acc_add(m, -x.ih, -x.il, y.rh, y.rl);
        ff rr = acc_done(r), mm = acc_done(m);
        fsum_add(sr, rr.h, rr.l);
        fsum_add(si, mm.h, mm.l);
    }
    block_sum2(ff2d(sr.h, sr.l), ff2d(si.h, si.l), out2);
}

// Dual-state tile sweep for the backward pass.
//   kind 0 dense / 1 diagonal / 2 monomial: applied to both psi and lambda tiles;
//   kind 3 gradient marker: acc[slot] += w * Im <lambda|G|psi> over the tile, G a
//          Pauli string (xm on tile-local bits, zm on global bits, phase ph) or,
//          when k == 1, the projector P1 on global bit gbit[0].
struct AdjGate {
    TileGate g;
    uint32_t xm_local;
    int32_t ph;
    uint64_t zm;
    int32_t slot;
    int32_t projector;
    double weight;
};

template <int K>
__device__ void adj_dense(float4* sm, int T, const TileGate& g, const float4* __restrict__ mats) {
    constexpr int D = 1 << K;
    int pos[K];
    for (int q = 0; q < K; q++) pos[q] = g.tbit[q];
    for (int a = 0; a < K; a++)
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int ngroups = 1 << (T - K);
    const float4* m = mats + g.mat_off;
    for (int gr = threadIdx.x; gr < ngroups; gr += blockDim.x) {
        int jb = gr;
        for (int q = 0; q < K; q++) { int low = jb & ((1 << pos[q]) - 1); jb = ((jb >> pos[q]) << (pos[q] + 1)) | low; }
        if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
        cff x[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << g.tbit[q];
            idx[c] = j;
            x[c] = f4c(sm[j]);
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            ffacc ar, ai;
            cmac_first(ar, ai, f4c(__ldg(m + r * D)), x[0]);
#pragma unroll
            for (int c = 1; c < D; c++) cmac(ar, ai, f4c(__ldg(m + r * D + c)), x[c]);
            sm[idx[r]] = c4f(cdone(ar, ai));
        }
    }
}

__device__ void adj_apply(float4* sm, int T, int L, const TileGate& g, const float4* mats, const int32_t* perms,
                          int64_t base, const int64_t* off_tab) {
    const int nt = 1 << T, lowmask = (1 << L) - 1;
    if (g.kind == 1) {
        const float4* m = mats + g.mat_off;
        for (int j = threadIdx.x; j < nt; j += blockDim.x) {
            if ((j & (int)g.lc_mask) != (int)g.lc_val) continue;
            int64_t gi = base | off_tab[j >> L] | (int64_t)(j & lowmask);
            int di = 0;
            for (int q = 0; q < g.k; q++) di |= (int)((gi >> g.gbit[q]) & 1) << q;
            sm[j] = c4f(cmul(f4c(__ldg(m + di)), f4c(sm[j])));
        }
    } else if (g.kind == 0) {
        switch (g.k) {
            case 1: adj_dense<1>(sm, T, g, mats); break;
            case 2: adj_dense<2>(sm, T, g, mats); break;
            case 3: adj_dense<3>(sm, T, g, mats); break;
            default: adj_dense<4>(sm, T, g, mats); break;
        }
    } else {
        // monomial
        const int D = 1 << g.k;
        int pos[BS_TILE_MAXK];
        for (int q = 0; q < g.k; q++) pos[q] = g.tbit[q];
        for (int a = 0; a < g.k; a++)
            for (int b = a + 1; b < g.k; b++)
                if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
        const int32_t* p = perms + g.perm_off;
        for (int gr = threadIdx.x; gr < (1 << (T - g.k)); gr += blockDim.x) {
            int jb = gr;
            for (int q = 0; q < g.k; q++) { int low = jb & ((1 << pos[q]) - 1); jb = ((jb >> pos[q]) << (pos[q] + 1)) | low; }
            if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
            float4 x[16];
            int idx[16];
            for (int c = 0; c < D; c++) {
                int j = jb;
                for (int q = 0; q < g.k; q++) if ((c >> q) & 1) j |= 1 << g.tbit[q];
                idx[c] = j;
                x[c] = sm[j];
            }
            for (int c = 0; c < D; c++) sm[idx[__ldg(p + 2 * c)]] = c4f(cmul_ipow(f4c(x[c]), __ldg(p + 2 * c + 1)));
        }
    }
}

// The same gate on both tiles of the sweep (psi and lambda) in one pass: the index arithmetic and the
// matrix reads are shared.  Dense gates on 1 or 2 targets and diagonal gates; others go through
// adj_apply once per tile.
template <int K>
__device__ void adj_dense2(float4* sa, float4* sb, int T, const TileGate& g, const float4* __restrict__ mats) {
    constexpr int D = 1 << K;
    int pos[K];
    for (int q = 0; q < K; q++) pos[q] = g.tbit[q];
    for (int a = 0; a < K; a++)
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int ngroups = 1 << (T - K);
    const float4* m = mats + g.mat_off;
    for (int gr = threadIdx.x; gr < ngroups; gr += blockDim.x) {
        int jb = gr;
        for (int q = 0; q < K; q++) { int low = jb & ((1 << pos[q]) - 1); jb = ((jb >> pos[q]) << (pos[q] + 1)) | low; }
        if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
        cff x[D], y[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << g.tbit[q];
            idx[c] = j;
            x[c] = f4c(sa[j]);
            y[c] = f4c(sb[j]);
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            ffacc ar, ai, br, bi;
            const cff m0 = f4c(__ldg(m + r * D));
            cmac_first(ar, ai, m0, x[0]);
            cmac_first(br, bi, m0, y[0]);
#pragma unroll
            for (int c = 1; c < D; c++) {
                const cff mc = f4c(__ldg(m + r * D + c));
                cmac(ar, ai, mc, x[c]);
                cmac(br, bi, mc, y[c]);
            }
            sa[idx[r]] = c4f(cdone(ar, ai));
            sb[idx[r]] = c4f(cdone(br, bi));
        }
    }
}

__device__ void adj_apply2(float4* sa, float4* sb, int T, int L, const TileGate& g, const float4* mats,
                           const int32_t* perms, int64_t base, const int64_t* off_tab) {
    if (g.kind == 1) {
        const int nt = 1 << T, lowmask = (1 << L) - 1;
        const float4* m = mats + g.mat_off;
        for (int j = threadIdx.x; j < nt; j += blockDim.x) {
            if ((j & (int)g.lc_mask) != (int)g.lc_val) continue;
            const int64_t gi = base | off_tab[j >> L] | (int64_t)(j & lowmask);
            int di = 0;
            for (int q = 0; q < g.k; q++) di |= (int)((gi >> g.gbit[q]) & 1) << q;
            const cff dv = f4c(__ldg(m + di));
            sa[j] = c4f(cmul(dv, f4c(sa[j])));
            sb[j] = c4f(cmul(dv, f4c(sb[j])));
        }
    } else if (g.kind == 0 && g.k == 1) {
        adj_dense2<1>(sa, sb, T, g, mats);
    } else if (g.kind == 0 && g.k == 2) {
        adj_dense2<2>(sa, sb, T, g, mats);
    } else {
        adj_apply(sa, T, L, g, mats, perms, base, off_tab);
        adj_apply(sb, T, L, g, mats, perms, base, off_tab);
    }
}

template <bool C64>
__global__ void __launch_bounds__(kAThreads) k_adjoint_sweep(typename Elem<C64>::T* __restrict__ psi,
                                                             typename Elem<C64>::T* __restrict__ lam, SweepDesc d,
                                                             const AdjGate* __restrict__ ag,
                                                             double* __restrict__ grad_acc, int64_t tile0) {
    extern __shared__ float4 smem[];
    const int T = d.T, L = d.L, H = T - L;
    const int nt = 1 << T;
    float4* sp = smem;
    float4* sl = smem + nt;
    int64_t* off_tab = reinterpret_cast<int64_t*>(smem + 2 * nt);
    __shared__ int64_t s_base;
    const int64_t tile = tile0 + (int64_t)blockIdx.x;
    if (threadIdx.x == 0) {
        int64_t base = 0;
        int src = 0;
        for (int bit = 0; bit < d.n_bits; bit++)
            if (!((d.tile_mask >> bit) & 1ULL)) { base |= ((tile >> src) & 1LL) << bit; src++; }
        s_base = base;
    }
    for (int i = threadIdx.x; i < (1 << H); i += blockDim.x) {
        int64_t o = 0;
        for (int j = 0; j < H; j++) if ((i >> j) & 1) o |= 1LL << d.hi_bits[j];
        off_tab[i] = o;
    }
    __syncthreads();
    const int64_t base = s_base;
    const int lowmask = (1 << L) - 1;
    // tile loads: four positions (eight loads) per thread in flight at a time (tiles <= 2^12)
#pragma unroll
    for (int r = 0; r < 4096 / kAThreads; r += 4) {
        typename Elem<C64>::T xp[4], xl[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int j = (r + i) * kAThreads + (int)threadIdx.x;
            if (j < nt) {
                const int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
                xp[i] = psi[gidx];
                xl[i] = lam[gidx];
            }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int j = (r + i) * kAThreads + (int)threadIdx.x;
            if (j < nt) {
                sp[j] = c4f(Elem<C64>::load(xp[i]));
                sl[j] = c4f(Elem<C64>::load(xl[i]));
            }
        }
    }
    __syncthreads();
    for (int gi = 0; gi < d.n_gates; gi++) {
        const AdjGate& a = ag[gi];   // fields read where used (a copy of the whole descriptor went to local memory)
        if (a.g.kind == 3) {
            // Im <lambda| G |psi> over the tile
            ffsum acc{0.f, 0.f};
            for (int j = threadIdx.x; j < nt; j += blockDim.x) {
                int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
                cff l = f4c(sl[j]);
                cff x;
                if (a.projector) {
                    if (!((gidx >> a.g.gbit[0]) & 1)) continue;
                    x = f4c(sp[j]);
                } else {
                    x = f4c(sp[j ^ (int)a.xm_local]);
                    int ph = a.ph + ((__popcll((unsigned long long)gidx & a.zm) & 1) ? 2 : 0);
                    x = cmul_ipow(x, (4 - (ph & 3)) & 3);
                }
                // Im(conj(l) * x) = l.r x.i - l.i x.r
                ffacc m;
                acc_first(m, l.rh, l.rl, x.ih, x.il);
                acc_add(m, -l.ih, -l.il, x.rh, x.rl);
                ff v = acc_done(m);
                fsum_add(acc, v.h, v.l);
            }
            double v = ff2d(acc.h, acc.l) * a.weight;
            __shared__ double red[kAThreads / 32];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                double s = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
                atomicAdd(grad_acc + a.slot, s);
            }
            __syncthreads();
            continue;
        }
        if ((base & (int64_t)a.g.gc_mask) != (int64_t)a.g.gc_val) continue;
        adj_apply2(sp, sl, T, L, a.g, d.mats, d.perms, base, off_tab);
        __syncthreads();
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
        psi[gidx] = Elem<C64>::store(f4c(sp[j]));
        lam[gidx] = Elem<C64>::store(f4c(sl[j]));
    }
}

// ---- complex64 states: the backward sweep's gates in FP32 on float2 tiles (the state's own
// precision; half the shared memory and a sixth of the instructions of the float-float path), the
// gradient inner products from the FP32 values with exact products and float-float sums.
__device__ __forceinline__ float2 c32mul(float2 m, float2 x) {
    return make_float2(__fmaf_rn(m.x, x.x, -m.y * x.y), __fmaf_rn(m.x, x.y, m.y * x.x));
}
__device__ __forceinline__ float2 c32ipow(float2 x, int p) {
    switch (p & 3) {
        case 0: return x;
        case 1: return make_float2(-x.y, x.x);
        case 2: return make_float2(-x.x, -x.y);
        default: return make_float2(x.y, -x.x);
    }
}
// matrix entry (float4 re hi, re lo, im hi, im lo) as the nearest complex64 value
__device__ __forceinline__ float2 m32(float4 v) { return make_float2(v.x, v.z); }

template <int K>
__device__ void adj32_dense2(float2* sa, float2* sb, int T, const TileGate& g, const float4* __restrict__ mats) {
    constexpr int D = 1 << K;
    int pos[K];
    for (int q = 0; q < K; q++) pos[q] = g.tbit[q];
    for (int a = 0; a < K; a++)
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const float4* m = mats + g.mat_off;
    for (int gr = threadIdx.x; gr < (1 << (T - K)); gr += blockDim.x) {
        int jb = gr;
        for (int q = 0; q < K; q++) { int low = jb & ((1 << pos[q]) - 1); jb = ((jb >> pos[q]) << (pos[q] + 1)) | low; }
        if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
        float2 x[D], y[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << g.tbit[q];
            idx[c] = j;
            x[c] = sa[j];
            y[c] = sb[j];
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            float2 u = make_float2(0.f, 0.f), v = make_float2(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < D; c++) {
                const float2 mc = m32(__ldg(m + r * D + c));
                u.x = __fmaf_rn(mc.x, x[c].x, __fmaf_rn(-mc.y, x[c].y, u.x));
                u.y = __fmaf_rn(mc.x, x[c].y, __fmaf_rn(mc.y, x[c].x, u.y));
                v.x = __fmaf_rn(mc.x, y[c].x, __fmaf_rn(-mc.y, y[c].y, v.x));
                v.y = __fmaf_rn(mc.x, y[c].y, __fmaf_rn(mc.y, y[c].x, v.y));
            }
            sa[idx[r]] = u;
            sb[idx[r]] = v;
        }
    }
}

__device__ void adj32_apply2(float2* sa, float2* sb, int T, int L, const TileGate& g, const float4* mats,
                             const int32_t* perms, int64_t base, const int64_t* off_tab) {
    const int nt = 1 << T, lowmask = (1 << L) - 1;
    if (g.kind == 1) {
        const float4* m = mats + g.mat_off;
        for (int j = threadIdx.x; j < nt; j += blockDim.x) {
            if ((j & (int)g.lc_mask) != (int)g.lc_val) continue;
            const int64_t gi = base | off_tab[j >> L] | (int64_t)(j & lowmask);
            int di = 0;
            for (int q = 0; q < g.k; q++) di |= (int)((gi >> g.gbit[q]) & 1) << q;
            const float2 d = m32(__ldg(m + di));
            sa[j] = c32mul(d, sa[j]);
            sb[j] = c32mul(d, sb[j]);
        }
    } else if (g.kind == 0) {
        switch (g.k) {
            case 1: adj32_dense2<1>(sa, sb, T, g, mats); break;
            case 2: adj32_dense2<2>(sa, sb, T, g, mats); break;
            case 3: adj32_dense2<3>(sa, sb, T, g, mats); break;
            default: adj32_dense2<4>(sa, sb, T, g, mats); break;
        }
    } else {
        // monomial: column c goes to row perm[2c] with phase i^perm[2c+1]
        const int D = 1 << g.k;
        int pos[BS_TILE_MAXK];
        for (int q = 0; q < g.k; q++) pos[q] = g.tbit[q];
        for (int a = 0; a < g.k; a++)
            for (int b = a + 1; b < g.k; b++)
                if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
        const int32_t* p = perms + g.perm_off;
        for (int gr = threadIdx.x; gr < (1 << (T - g.k)); gr += blockDim.x) {
            int jb = gr;
            for (int q = 0; q < g.k; q++) { int low = jb & ((1 << pos[q]) - 1); jb = ((jb >> pos[q]) << (pos[q] + 1)) | low; }
            if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
            float2 x[16], y[16];
            int idx[16];
            for (int c = 0; c < D; c++) {
                int j = jb;
                for (int q = 0; q < g.k; q++) if ((c >> q) & 1) j |= 1 << g.tbit[q];
                idx[c] = j;
                x[c] = sa[j];
                y[c] = sb[j];
            }
            for (int c = 0; c < D; c++) {
                const int r = __ldg(p + 2 * c), ph = __ldg(p + 2 * c + 1);
                sa[idx[r]] = c32ipow(x[c], ph);
                sb[idx[r]] = c32ipow(y[c], ph);
            }
        }
    }
}

__global__ void __launch_bounds__(kAThreads) k_adjoint_sweep_c64(float2* __restrict__ psi, float2* __restrict__ lam,
                                                                 SweepDesc d, const AdjGate* __restrict__ ag,
                                                                 double* __restrict__ grad_acc, int64_t tile0) {
    extern __shared__ float4 smem4[];
    const int T = d.T, L = d.L, H = T - L;
    const int nt = 1 << T;
    float2* sp = reinterpret_cast<float2*>(smem4);
    float2* sl = sp + nt;
    int64_t* off_tab = reinterpret_cast<int64_t*>(sl + nt);
    __shared__ int64_t s_base;
    __shared__ double red[kAThreads / 32];
    const int64_t tile = tile0 + (int64_t)blockIdx.x;
    if (threadIdx.x == 0) {
        int64_t base = 0;
        int src = 0;
        for (int bit = 0; bit < d.n_bits; bit++)
            if (!((d.tile_mask >> bit) & 1ULL)) { base |= ((tile >> src) & 1LL) << bit; src++; }
        s_base = base;
    }
    for (int i = threadIdx.x; i < (1 << H); i += blockDim.x) {
        int64_t o = 0;
        for (int j = 0; j < H; j++) if ((i >> j) & 1) o |= 1LL << d.hi_bits[j];
        off_tab[i] = o;
    }
    __syncthreads();
    const int64_t base = s_base;
    const int lowmask = (1 << L) - 1;
#pragma unroll 4
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
        sp[j] = psi[gidx];
        sl[j] = lam[gidx];
    }
    __syncthreads();
    for (int gi = 0; gi < d.n_gates; gi++) {
        const AdjGate& a = ag[gi];
        if (a.g.kind == 3) {
            // Im <lambda| G |psi> over the tile: exact FP32 products, float-float sums
            ffsum acc{0.f, 0.f};
            for (int j = threadIdx.x; j < nt; j += blockDim.x) {
                const int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
                const float2 l = sl[j];
                float2 x;
                if (a.projector) {
                    if (!((gidx >> a.g.gbit[0]) & 1)) continue;
                    x = sp[j];
                } else {
                    const int ph = a.ph + ((__popcll((unsigned long long)gidx & a.zm) & 1) ? 2 : 0);
                    x = c32ipow(sp[j ^ (int)a.xm_local], (4 - (ph & 3)) & 3);
                }
                ffacc m;
                acc_first(m, l.x, 0.f, x.y, 0.f);
                acc_add(m, -l.y, 0.f, x.x, 0.f);
                const ff v = acc_done(m);
                fsum_add(acc, v.h, v.l);
            }
            double v = ff2d(acc.h, acc.l) * a.weight;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
                atomicAdd(grad_acc + a.slot, t);
            }
            __syncthreads();
            continue;
        }
        if ((base & (int64_t)a.g.gc_mask) != (int64_t)a.g.gc_val) continue;
        adj32_apply2(sp, sl, T, L, a.g, d.mats, d.perms, base, off_tab);
        __syncthreads();
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
        psi[gidx] = sp[j];
        lam[gidx] = sl[j];
    }
}

inline float4 to_cff(double re, double im) {
    float4 v;
    v.x = (float)re; v.y = (float)(re - (double)v.x);
    v.z = (float)im; v.w = (float)(im - (double)v.z);
    return v;
}

struct BwdItem {          // one element of the reversed gate list
    HostGate g;
    bool marker = false;
    int slot = 0;
    int projector = 0;
    uint64_t xm = 0, zm = 0;   // endian masks of the generator
    int ph = 0;
    double weight = 1.0;
};

// U^dagger of a lowered gate (same targets and controls)
HostGate dagger(const HostGate& h) {
    HostGate d = h;
    const int D = 1 << h.k;
    if (h.kind == 1) {
        for (int i = 0; i < D; i++) d.mat[2 * i + 1] = -h.mat[2 * i + 1];
    } else if (h.kind == 0) {
        for (int r = 0; r < D; r++)
            for (int c = 0; c < D; c++) {
                d.mat[2 * (r * D + c)] = h.mat[2 * (c * D + r)];
                d.mat[2 * (r * D + c) + 1] = -h.mat[2 * (c * D + r) + 1];
            }
    } else {
        // column c -> row r with phase p  ==>  column r -> row c with phase -p
        for (int c = 0; c < D; c++) {
            int r = h.perm[2 * c], p = h.perm[2 * c + 1];
            d.perm[2 * r] = c;
            d.perm[2 * r + 1] = (4 - p) & 3;
        }
    }
    return d;
}

}  // namespace

extern "C" int bs_adjoint_gradient(bs_sim* s, const bs_op* ops, int64_t n_ops, const int32_t* param_index,
                                   const int32_t* gen_kind, const uint64_t* gen_xmask, const uint64_t* gen_zmask,
                                   int n_params, int n_terms, const uint64_t* xmask, const uint64_t* zmask,
                                   const double* coeffs, double* energy_out, double* grad_out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (s->kind != BS_KIND_SV) return bs_fail(s, BS_ERR_UNSUPPORTED, "adjoint gradients need a state-vector simulator");
    const bool c64 = s->precision == BS_PREC_C64;
    const size_t esz = c64 ? 8 : 16;
    if (n_ops < 0 || (n_ops && (!ops || !param_index || !gen_kind || !gen_xmask || !gen_zmask)) || n_params < 0 ||
        n_terms < 1 || !xmask || !zmask || !coeffs || !energy_out || (n_params && !grad_out))
        return bs_fail(s, BS_ERR_INVALID_ARG, "bad adjoint arguments");
    const int n = s->n;
    const int64_t len = s->len;
    auto to_endian = [n](uint64_t m) {
        uint64_t e = 0;
        for (int q = 0; q < n; q++) if ((m >> q) & 1ULL) e |= 1ULL << (n - 1 - q);
        return e;
    };
    // 0. segments and checkpoint buffers
    int n_param_gates = 0;
    for (int64_t i = 0; i < n_ops; i++) n_param_gates += (ops[i].kind == 0 && param_index[i] >= 0) ? 1 : 0;
    int S = s->tune.adj_segments;
    const size_t state_bytes = (size_t)len * esz;
    if (S < 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        const int by_mem = (int)std::min<size_t>(64, fr / 4 / std::max<size_t>(state_bytes, 1));
        S = std::min(std::min(16, 1 + n_param_gates / 16), by_mem + 1);
    }
    S = std::max(1, std::min<int>(S, (int)std::max<int64_t>(1, n_ops)));
    std::vector<void*> ckpt;
    for (;;) {
        bool ok = true;
        for (int j = 0; j + 1 < S; j++) {
            void* p = nullptr;
            if (cudaMalloc(&p, state_bytes) != cudaSuccess) { ok = false; break; }
            ckpt.push_back(p);
        }
        if (ok) break;
        cudaGetLastError();
        for (void* p : ckpt) cudaFree(p);
        ckpt.clear();
        S = std::max(1, S / 2);   // memory binds: fewer checkpoints, more uncomputation
        if (S == 1) break;
    }
    auto free_ckpt = [&]() { for (void* p : ckpt) cudaFree(p); ckpt.clear(); };
    // segment j covers ops [seg[j], seg[j+1]), split evenly by gate count
    std::vector<int64_t> seg(1, 0);
    {
        int64_t n_gates = 0;
        for (int64_t i = 0; i < n_ops; i++) n_gates += ops[i].kind == 0;
        int64_t cnt = 0;
        for (int64_t i = 0; i < n_ops && (int)seg.size() < S; i++) {
            cnt += ops[i].kind == 0;
            if (cnt * S >= n_gates * (int64_t)seg.size() && i + 1 < n_ops) seg.push_back(i + 1);
        }
        seg.push_back(n_ops);
        S = (int)seg.size() - 1;
        while ((int)ckpt.size() > S - 1) { cudaFree(ckpt.back()); ckpt.pop_back(); }
    }
    // 1. forward pass, keeping psi after every segment but the last
    bs_stats fwd{};
    int rc = BS_OK;
    // segments are queued back to back: the host plans segment j+1 while the GPU runs segment j
    cudaEventRecord(s->ev0, s->stream);
    s->tc_events_used = 0;
    s->defer_sync = true;
    for (int j = 0; j < S && !rc; j++) {
        rc = bs_evolve(s, ops + seg[(size_t)j], seg[(size_t)j + 1] - seg[(size_t)j], 0);
        if (rc) break;
        fwd.sweeps += s->stats.sweeps;
        fwd.kernel_launches += s->stats.kernel_launches;
        fwd.gates += s->stats.gates;
        fwd.bytes_moved += s->stats.bytes_moved;
        fwd.tc_gates += s->stats.tc_gates;
        fwd.tc_launches += s->stats.tc_launches;
        if (j + 1 < S) rc = bs_cuda_check(s, cudaMemcpyAsync(ckpt[(size_t)j], s->state, state_bytes, cudaMemcpyDeviceToDevice, s->stream), "checkpoint");
    }
    s->defer_sync = false;
    if (rc) { cudaStreamSynchronize(s->stream); free_ckpt(); return rc; }
    s->stats = fwd;
    // 2. lambda = H psi
    void* lam = nullptr;
    rc = bs_cuda_check(s, cudaMallocAsync(&lam, (size_t)len * esz, s->stream), "lambda allocation");
    if (rc) { free_ckpt(); return rc; }
    std::vector<PauliTerm> terms((size_t)n_terms);
    for (int t = 0; t < n_terms; t++) {
        uint64_t x = xmask[t], z = zmask[t];
        int ny = __builtin_popcountll(x & z);
        terms[(size_t)t].xm = to_endian(x);
        terms[(size_t)t].zm = to_endian(z);
        terms[(size_t)t].ph = ny & 3;
        terms[(size_t)t].ch = (float)coeffs[t];
        terms[(size_t)t].cl = (float)(coeffs[t] - (double)terms[(size_t)t].ch);
    }
    rc = bs_ensure_scratch(s, (int64_t)n_terms * (int64_t)sizeof(PauliTerm) + (int64_t)(n_params + 2) * 8 + 256);
    if (rc) { cudaFreeAsync(lam, s->stream); free_ckpt(); return rc; }
    PauliTerm* d_terms = (PauliTerm*)s->scratch;
    double* d_acc = (double*)((char*)s->scratch + (((int64_t)n_terms * (int64_t)sizeof(PauliTerm) + 255) & ~255LL));
    cudaMemcpyAsync(d_terms, terms.data(), terms.size() * sizeof(PauliTerm), cudaMemcpyHostToDevice, s->stream);
    cudaMemsetAsync(d_acc, 0, (size_t)(n_params + 2) * 8, s->stream);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((len + kAThreads - 1) / kAThreads, 152 * 8));
    if (c64) {
        k_pauli_sum<true><<<blocks, kAThreads, 0, s->stream>>>((const float2*)s->state, (float2*)lam, len, d_terms, n_terms);
        k_inner<true><<<blocks, kAThreads, 0, s->stream>>>((const float2*)s->state, (const float2*)lam, len, d_acc + n_params);
    } else {
        k_pauli_sum<false><<<blocks, kAThreads, 0, s->stream>>>((const double2*)s->state, (double2*)lam, len, d_terms,
                                                                 n_terms);
        k_inner<false><<<blocks, kAThreads, 0, s->stream>>>((const double2*)s->state, (const double2*)lam, len,
                                                             d_acc + n_params);
    }
    // 3. backward: reversed, daggered gate list with gradient markers before each parameterised gate
    std::vector<BwdItem> items;
    std::vector<size_t> seg_item(1, 0);   // items of segment S-1-r start at seg_item[r]
    int cur_seg = S - 1;
    for (int64_t i = n_ops - 1; i >= 0; i--) {
        while (cur_seg > 0 && i < seg[(size_t)cur_seg]) {
            cur_seg--;
            seg_item.push_back(items.size());
        }
        const bs_op& op = ops[i];
        if (op.kind != 0) continue;
        std::vector<HostGate> hg;
        rc = bs_lower_gate(s, op.matrix, op.n_targets, op.targets, op.n_controls, op.controls, op.control_values,
                           op.flags, false, hg);
        if (rc) { cudaFreeAsync(lam, s->stream); free_ckpt(); return rc; }
        if (param_index[i] >= 0) {
            if (param_index[i] >= n_params) { cudaFreeAsync(lam, s->stream); free_ckpt(); return bs_fail(s, BS_ERR_INVALID_ARG, "parameter index out of range"); }
            BwdItem m;
            m.marker = true;
            m.slot = param_index[i];
            m.projector = gen_kind[i] == 1;
            if (m.projector) {
                // PhaseShift on its target: weight -2, projector on the target's endian bit
                m.g.k = 1;
                m.g.ebit[0] = n - 1 - op.targets[0];
                m.weight = -2.0;
            } else {
                m.xm = to_endian(gen_xmask[i]);
                m.zm = to_endian(gen_zmask[i]);
                m.ph = __builtin_popcountll(gen_xmask[i] & gen_zmask[i]) & 3;
                m.g.k = 0;
                for (int q = 0; q < n; q++)
                    if ((m.xm >> q) & 1ULL) m.g.ebit[m.g.k++] = q;
                m.weight = 1.0;
            }
            m.g.kind = 3;
            items.push_back(m);
        }
        for (const HostGate& h : hg) {
            BwdItem it;
            it.g = dagger(h);
            items.push_back(it);
        }
    }
    while ((int)seg_item.size() < S) seg_item.push_back(items.size());
    seg_item.push_back(items.size());
    // plan sweeps segment by segment: markers need their flip bits in the tile, and they must not
    // move past a gate sharing bits (they read the current psi and lambda)
    const int n_bits = n;
    const int T = std::min(BS_TILE_MAX_BITS, n_bits);
    const int L = std::min(BS_TILE_LOW_BITS, T);
    const int cap = T - L;
    std::vector<std::vector<int>> sweeps_items;
    std::vector<std::vector<int>> sweeps_hi;
    std::vector<int> sweep_restore;   // checkpoint to restore psi from before the sweep, -1 if none
    for (int r = 0; r < S; r++) {
        const size_t G = seg_item[(size_t)r + 1];
        std::vector<char> done(G, 0);
        size_t remaining = G - seg_item[(size_t)r], first = seg_item[(size_t)r];
        bool seg_first = true;
        auto touch = [&](const BwdItem& it) {
            uint64_t m = it.g.cmask | it.zm | it.xm;
            for (int q = 0; q < it.g.k; q++) m |= 1ULL << it.g.ebit[q];
            return m;
        };
        auto need = [&](const BwdItem& it) -> uint64_t {
            uint64_t m = 0;
            if (!it.marker && it.g.kind == 1) return m;
            if (it.marker) return it.xm & ~(((uint64_t)1 << L) - 1);
            for (int q = 0; q < it.g.k; q++) if (it.g.ebit[q] >= L) m |= 1ULL << it.g.ebit[q];
            return m;
        };
        while (remaining) {
            std::vector<int> idx;
            uint64_t chosen = 0, blocked = 0;
            int nch = 0;
            for (size_t i = first; i < G; i++) {
                if (done[i]) continue;
                uint64_t t = touch(items[i]);
                if (t & blocked) { blocked |= t; continue; }
                uint64_t nb = need(items[i]) & ~chosen;
                int add = __builtin_popcountll(nb);
                bool too_big = !items[i].marker && items[i].g.kind != 1 &&
                               (items[i].g.k > BS_TILE_MAXK || __builtin_popcountll(need(items[i])) > cap);
                if (too_big || (items[i].marker && __builtin_popcountll(need(items[i])) > cap)) {
                    cudaFreeAsync(lam, s->stream);
                    free_ckpt();
                    return bs_fail(s, BS_ERR_UNSUPPORTED, "adjoint gate too wide for a tile");
                }
                if (nch + add <= cap) {
                    chosen |= nb;
                    nch += add;
                    idx.push_back((int)i);
                    done[i] = 1;
                    remaining--;
                } else {
                    blocked |= t;
                }
            }
            while (first < G && done[first]) first++;
            std::vector<int> hi;
            for (int b = L; b < n_bits; b++) if ((chosen >> b) & 1ULL) hi.push_back(b);
            for (int b = L; b < n_bits && (int)hi.size() < cap; b++) if (!((chosen >> b) & 1ULL)) hi.push_back(b);
            std::sort(hi.begin(), hi.end());
            sweeps_items.push_back(idx);
            sweeps_hi.push_back(hi);
            // entering segment S-1-r (r > 0): psi is its end state, kept by the forward pass
            sweep_restore.push_back(seg_first && r > 0 ? S - 1 - r : -1);
            seg_first = false;
        }
    }
    // pack device data
    std::vector<AdjGate> ag;
    std::vector<float4> mats;
    std::vector<int32_t> perms;
    std::vector<int64_t> sweep_first;
    for (size_t sw = 0; sw < sweeps_items.size(); sw++) {
        int local[64];
        for (int b = 0; b < 64; b++) local[b] = -1;
        for (int b = 0; b < L; b++) local[b] = b;
        for (size_t i = 0; i < sweeps_hi[sw].size(); i++) local[sweeps_hi[sw][i]] = L + (int)i;
        sweep_first.push_back((int64_t)ag.size());
        for (int ii : sweeps_items[sw]) {
            const BwdItem& it = items[(size_t)ii];
            AdjGate a{};
            a.g.kind = it.marker ? 3 : it.g.kind;
            a.g.k = it.g.k;
            if (it.marker) {
                a.slot = it.slot;
                a.projector = it.projector;
                a.weight = it.weight;
                a.zm = it.zm;
                a.ph = it.ph;
                uint32_t xl = 0;
                for (int b = 0; b < n_bits; b++) if ((it.xm >> b) & 1ULL) xl |= 1u << local[b];
                a.xm_local = xl;
                if (it.projector) a.g.gbit[0] = it.g.ebit[0];
                ag.push_back(a);
                continue;
            }
            const HostGate& hg = it.g;
            uint64_t gcm = 0, gcv = 0;
            uint32_t lcm = 0, lcv = 0;
            for (int b = 0; b < n_bits; b++) {
                if (!((hg.cmask >> b) & 1ULL)) continue;
                uint64_t v = (hg.cval >> b) & 1ULL;
                if (local[b] >= 0) { lcm |= 1u << local[b]; lcv |= (uint32_t)v << local[b]; }
                else { gcm |= 1ULL << b; gcv |= v << b; }
            }
            a.g.lc_mask = lcm; a.g.lc_val = lcv; a.g.gc_mask = gcm; a.g.gc_val = gcv;
            for (int q = 0; q < hg.k; q++) {
                a.g.gbit[q] = hg.ebit[q];
                if (q < BS_TILE_MAXK) a.g.tbit[q] = local[hg.ebit[q]];
            }
            a.g.mat_off = (int32_t)mats.size();
            a.g.perm_off = (int32_t)perms.size();
            if (hg.kind == 0) for (int e = 0; e < (1 << (2 * hg.k)); e++) mats.push_back(to_cff(hg.mat[2 * e], hg.mat[2 * e + 1]));
            else if (hg.kind == 1) for (int e = 0; e < (1 << hg.k); e++) mats.push_back(to_cff(hg.mat[2 * e], hg.mat[2 * e + 1]));
            else perms.insert(perms.end(), hg.perm.begin(), hg.perm.end());
            ag.push_back(a);
        }
    }
    sweep_first.push_back((int64_t)ag.size());
    auto al = [](int64_t x) { return (x + 255) & ~(int64_t)255; };
    const int64_t b_ag = al((int64_t)ag.size() * (int64_t)sizeof(AdjGate));
    const int64_t b_m = al((int64_t)mats.size() * (int64_t)sizeof(float4));
    const int64_t b_p = al((int64_t)(perms.size() + 1) * 4);
    rc = bs_ensure_plan(s, b_ag + b_m + b_p);
    if (rc) { cudaFreeAsync(lam, s->stream); free_ckpt(); return rc; }
    std::vector<char> host((size_t)(b_ag + b_m + b_p), 0);
    if (!ag.empty()) std::memcpy(host.data(), ag.data(), ag.size() * sizeof(AdjGate));
    if (!mats.empty()) std::memcpy(host.data() + b_ag, mats.data(), mats.size() * sizeof(float4));
    if (!perms.empty()) std::memcpy(host.data() + b_ag + b_m, perms.data(), perms.size() * 4);
    cudaMemcpyAsync(s->plan_buf, host.data(), host.size(), cudaMemcpyHostToDevice, s->stream);
    const AdjGate* d_ag = (const AdjGate*)s->plan_buf;
    const float4* d_m = (const float4*)((char*)s->plan_buf + b_ag);
    const int32_t* d_p = (const int32_t*)((char*)s->plan_buf + b_ag + b_m);
    const int H = T - L;
    const size_t smem = (size_t)2 * ((size_t)1 << T) * sizeof(float4) + ((size_t)1 << H) * sizeof(int64_t);
    cudaFuncSetAttribute(k_adjoint_sweep<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_adjoint_sweep_c64, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    const size_t smem64 = (size_t)2 * ((size_t)1 << T) * sizeof(float2) + ((size_t)1 << H) * sizeof(int64_t);
    const int64_t ntiles = (int64_t)1 << (n_bits - T);
    for (size_t sw = 0; sw < sweeps_items.size(); sw++) {
        if (sweep_restore[sw] >= 0)
            cudaMemcpyAsync(s->state, ckpt[(size_t)sweep_restore[sw]], state_bytes, cudaMemcpyDeviceToDevice, s->stream);
        SweepDesc d{};
        d.n_bits = n_bits;
        d.T = T;
        d.L = L;
        d.n_gates = (int)(sweep_first[sw + 1] - sweep_first[sw]);
        uint64_t tm = (1ULL << L) - 1;
        for (int i = 0; i < H; i++) { d.hi_bits[i] = sweeps_hi[sw][(size_t)i]; tm |= 1ULL << sweeps_hi[sw][(size_t)i]; }
        d.tile_mask = tm;
        d.mats = d_m;
        d.perms = d_p;
        for (int64_t t0 = 0; t0 < ntiles; t0 += (1LL << 30)) {
            int64_t nb = std::min<int64_t>(ntiles - t0, 1LL << 30);
            if (c64)
                k_adjoint_sweep_c64<<<(unsigned)nb, kAThreads, smem64, s->stream>>>((float2*)s->state, (float2*)lam, d,
                                                                                    d_ag + sweep_first[sw], d_acc, t0);
            else
                k_adjoint_sweep<false><<<(unsigned)nb, kAThreads, smem, s->stream>>>((double2*)s->state, (double2*)lam, d,
                                                                                      d_ag + sweep_first[sw], d_acc, t0);
        }
        s->stats.kernel_launches++;
        s->stats.sweeps++;
        s->stats.bytes_moved += 4.0 * (double)esz * (double)len;
    }
    std::vector<double> res((size_t)n_params + 2);
    cudaMemcpyAsync(res.data(), d_acc, res.size() * 8, cudaMemcpyDeviceToHost, s->stream);
    cudaFreeAsync(lam, s->stream);
    cudaEventRecord(s->ev1, s->stream);
    rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), "adjoint");
    free_ckpt();
    if (rc) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->stats.gpu_ms = ms;   // forward and backward
    bs_collect_tc_time(s);
    rc = bs_check_device_flag(s);
    if (rc) return rc;
    *energy_out = res[(size_t)n_params];
    for (int p = 0; p < n_params; p++) grad_out[p] = res[(size_t)p];
    return BS_OK;
}
