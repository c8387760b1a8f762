// Tile sweeps: one CTA owns 2^T amplitudes of the state (the L lowest endian bits
// plus T-L chosen higher bits, all other bits fixed by the CTA index), converts
// them once to float-float in shared memory, applies every gate of the sweep
// whose targets lie inside the tile, and writes them back.  A sweep therefore
// reads and writes the state once however many gates it carries.
//
// Reference kernels replaced (src/gate_kernels.jl): 1q :489-537, 2q :540-576,
// controlled :579-670, generic k-target :753-775, custom diagonal/excitation
// kernels src/custom_gates.jl:364-416; the density-matrix gate of
// src/dm_simulator.jl:130-140 is two tile gates (column bits U, row bits conj U).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstring>
#include <thread>
#include "bs_internal.h"
#include "bs_ff.cuh"
#include "bs_tc.cuh"
#include "bs_cdf.cuh"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int insert0(int x, int bit) {
    int low = x & ((1 << bit) - 1);
    return ((x >> bit) << (bit + 1)) | low;
}
// shared-memory index of tile element j: swizzled (tensor-core sweep) or plain
template <bool SW>
__device__ __forceinline__ int sx(int j) { return SW ? tc::sw(j) : j; }
// Tile amplitudes in shared memory are float4 (re hi, im hi, re lo, im lo): the two high words and
// the two low words each form an aligned register pair for the packed f32x2 arithmetic of the
// tensor-core sweep.  Matrix entries in global memory are float4 (re hi, re lo, im hi, im lo).
// Gate descriptors of a sweep are staged in shared memory in chunks (one coalesced copy per chunk
// instead of dependent global loads of every field by every thread at every gate).
constexpr int kGateChunk = 32;
__device__ __forceinline__ void stage_gates(TileGate* dst, const TileGate* __restrict__ src, int ng) {
    __syncthreads();   // the previous chunk is no longer read
    const int words = ng * (int)(sizeof(TileGate) / 4);
    const int* s = reinterpret_cast<const int*>(src);
    int* t = reinterpret_cast<int*>(dst);
    for (int w = threadIdx.x; w < words; w += blockDim.x) t[w] = __ldg(s + w);
    __syncthreads();
}

__device__ __forceinline__ cff f4c(float4 v) { return {v.x, v.z, v.y, v.w}; }
__device__ __forceinline__ float4 c4f(const cff& c) { return make_float4(c.rh, c.ih, c.rl, c.il); }
__device__ __forceinline__ cff f4m(float4 v) { return {v.x, v.y, v.z, v.w}; }
// read-only operand load: through the non-coherent cache from global memory, or plainly from shared
// memory (operands staged there)
template <bool S, typename V>
__device__ __forceinline__ V ldro(const V* p) {
    if constexpr (S) return *p;
    else return __ldg(p);
}

template <int K, bool SW = false, bool SM = false>
__device__ void tile_dense(float4* sm, int T, const TileGate& g, const float4* __restrict__ mats) {
    constexpr int D = 1 << K;
    int pos[K];
#pragma unroll
    for (int q = 0; q < K; q++) pos[q] = g.tbit[q];
    // ascending order for padding
#pragma unroll
    for (int a = 0; a < K; a++)
#pragma unroll
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int ngroups = 1 << (T - K);
    const float4* m = mats + g.mat_off;
    const uint32_t lcm = g.lc_mask, lcv = g.lc_val;
    int tb[K];
#pragma unroll
    for (int q = 0; q < K; q++) tb[q] = g.tbit[q];
    if (K == 1) {
        // 2x2: matrix held in registers across the thread's pairs
        const cff m00 = f4m(ldro<SM>(m)), m01 = f4m(ldro<SM>(m + 1)), m10 = f4m(ldro<SM>(m + 2)), m11 = f4m(ldro<SM>(m + 3));
        const int b0 = 1 << tb[0];
#pragma unroll 2
        for (int gr = threadIdx.x; gr < ngroups; gr += blockDim.x) {
            const int jb = insert0(gr, pos[0]);
            if ((jb & (int)lcm) != (int)lcv) continue;
            const int ia = sx<SW>(jb), ib = sx<SW>(jb | b0);
            const cff a = f4c(sm[ia]), b = f4c(sm[ib]);
            ffacc ar, ai;
            cmac_first(ar, ai, m00, a);
            cmac(ar, ai, m01, b);
            const cff ya = cdone(ar, ai);
            cmac_first(ar, ai, m10, a);
            cmac(ar, ai, m11, b);
            sm[ib] = c4f(cdone(ar, ai));
            sm[ia] = c4f(ya);
        }
        return;
    }
    for (int gr = threadIdx.x; gr < ngroups; gr += blockDim.x) {
        int jb = gr;
#pragma unroll
        for (int q = 0; q < K; q++) jb = insert0(jb, pos[q]);
        if ((jb & (int)lcm) != (int)lcv) continue;
        cff x[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
#pragma unroll
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << tb[q];
            idx[c] = sx<SW>(j);
            x[c] = f4c(sm[idx[c]]);
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            ffacc ar, ai;
            cmac_first(ar, ai, f4m(ldro<SM>(m + r * D)), x[0]);
#pragma unroll
            for (int c = 1; c < D; c++) cmac(ar, ai, f4m(ldro<SM>(m + r * D + c)), x[c]);
            sm[idx[r]] = c4f(cdone(ar, ai));
        }
    }
}

// monomial gate: column c goes to row perm[2c] with phase i^perm[2c+1]
template <int K, bool SW = false, bool SM = false>
__device__ void tile_monomial(float4* sm, int T, const TileGate& g, const int32_t* __restrict__ perms) {
    constexpr int D = 1 << K;
    int pos[K];
#pragma unroll
    for (int q = 0; q < K; q++) pos[q] = g.tbit[q];
#pragma unroll
    for (int a = 0; a < K; a++)
#pragma unroll
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int ngroups = 1 << (T - K);
    const int32_t* p = perms + g.perm_off;
    for (int gr = threadIdx.x; gr < ngroups; gr += blockDim.x) {
        int jb = gr;
#pragma unroll
        for (int q = 0; q < K; q++) jb = insert0(jb, pos[q]);
        if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
        float4 x[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
#pragma unroll
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << g.tbit[q];
            idx[c] = sx<SW>(j);
            x[c] = sm[idx[c]];
        }
#pragma unroll
        for (int c = 0; c < D; c++) {
            const int r = ldro<SM>(p + 2 * c), ph = ldro<SM>(p + 2 * c + 1);
            int j = jb;
#pragma unroll
            for (int q = 0; q < K; q++) if ((r >> q) & 1) j |= 1 << g.tbit[q];
            sm[sx<SW>(j)] = c4f(cmul_ipow(f4c(x[c]), ph));
        }
    }
}

// phase of a merged run of CZ gates at global index gi: odd parity -> -1
__device__ __forceinline__ bool parity_odd(const TileGate& g, int64_t gi) {
    int par = 0;
    for (int q = 0; q < g.npar; q++)
        par ^= __popcll((unsigned long long)(gi & (gi >> g.pshift[q])) & g.pmask[q]);
    return par & 1;
}

// off_tab[h] << osh: global offset of the tile's high-bit pattern h
template <typename OT, bool SW = false, bool SM = false>
__device__ void tile_diag(float4* sm, int T, int L, const TileGate& g, const float4* __restrict__ mats,
                          int64_t base, OT off_tab, int osh) {
    const int nt = 1 << T, lowmask = (1 << L) - 1;
    const float4* m = mats + g.mat_off;
    // pattern bit q: tile bit tbit[q] (32-bit), or a CTA constant for a bit outside the tile;
    // gates with more than BS_TILE_MAXK bits take the pattern from the 64-bit global index
    const bool fast = g.k <= BS_TILE_MAXK;
    int cst = 0, nk = 0;
    uint32_t enc = 0;   // per in-tile pattern bit: tile position (5 bits) | q << 5, one byte each
    if (fast)
        for (int q = 0; q < g.k; q++) {
            if (g.tbit[q] >= 0) enc |= (uint32_t)(g.tbit[q] | (q << 5)) << (8 * nk++);
            else cst |= (int)((base >> g.gbit[q]) & 1) << q;
        }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        if ((j & (int)g.lc_mask) != (int)g.lc_val) continue;
        const int js = sx<SW>(j);
        int di = cst;
        if (fast) {
            for (int u = 0; u < nk; u++) {
                const uint32_t b = (enc >> (8 * u)) & 255u;
                di |= ((j >> (b & 31u)) & 1) << (b >> 5);
            }
        } else {
            const int64_t gi = base | ((int64_t)off_tab[j >> L] << osh) | (int64_t)(j & lowmask);
            for (int q = 0; q < g.k; q++) di |= (int)((gi >> g.gbit[q]) & 1) << q;
        }
        float4 d = ldro<SM>(m + di);
        if (d.y == 0.f && d.w == 0.f) {
            if (d.z == 0.f && d.x == 1.f) continue;
            if (d.z == 0.f && d.x == -1.f) { sm[js] = c4f(cmul_ipow(f4c(sm[js]), 2)); continue; }
            if (d.x == 0.f && d.z == 1.f) { sm[js] = c4f(cmul_ipow(f4c(sm[js]), 1)); continue; }
            if (d.x == 0.f && d.z == -1.f) { sm[js] = c4f(cmul_ipow(f4c(sm[js]), 3)); continue; }
        }
        sm[js] = c4f(cmul(f4m(d), f4c(sm[js])));
    }
}

// Kraus channel on K <= 2 targets in the reference's update rule (src/noise_kernels.jl:105-168): the
// stored matrix S gets B <- sum_q K_q B K_q^dagger on every D x D block B whose row and column agree on
// all non-target bits (vec(S) index = row + column 2^n); other elements are left alone.  tbit[0..K-1]:
// tile positions of the row target bits (matrix bit j <-> tbit[j]), tbit[K..2K-1]: of the column
// target bits; pmask[0]: row-index mask of the non-target bits; pmask[1]: the non-target bits whose
// row and column bits both lie outside the tile (so that part of the test is uniform in the CTA);
// npar: number of Kraus matrices, row-major D x D each at mat_off.
// With few registers (the tensor-core sweep's threads have none to spare, and the float-float
// sweep's 2-target variant would otherwise need the 4-bit kernel): candidate blocks are tested and
// the ones that pass the row/column test collected (all candidates tested in one pass), then one
// thread per output element
// of a collected block sums over the Kraus matrices reading the block from shared memory; all reads
// of the collected blocks finish before any of their outputs is written.  s_act: 32 ints of shared
// scratch.
template <int K, bool SW, typename OT>
__device__ void tile_kraus_ref_lr(float4* sm, int T, int L, const TileGate& g, const float4* __restrict__ mats,
                                  int64_t base, OT off_tab, int osh, int n, int* s_act, int* s_cnt) {
    constexpr int D = 1 << K, DD = D * D, kChunkG = 32;   // capacity of s_act: at most this many blocks pass
    const int64_t rmask = ((int64_t)1 << n) - 1;
    if ((((base & rmask) ^ (base >> n)) & (int64_t)g.pmask[1]) != 0) return;   // uniform in the CTA
    int pos[2 * K];
#pragma unroll
    for (int q = 0; q < 2 * K; q++) pos[q] = g.tbit[q];
#pragma unroll
    for (int a = 0; a < 2 * K; a++)
#pragma unroll
        for (int b = a + 1; b < 2 * K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int lowmask = (1 << L) - 1, ngroups = 1 << (T - 2 * K);
    const float4* km = mats + g.mat_off;
    // Every candidate block is tested in one pass by all threads.  A block passes when, for every
    // non-target qubit, its row and column bits agree; each non-target tile bit belongs to a qubit
    // whose other bit is either in the tile (one constraint per pair) or constant in the CTA (one per
    // bit), so at most 2^((T - 2K) / 2) <= 32 blocks pass (T <= 12): s_act holds them all.
    if (threadIdx.x == 0) *s_cnt = 0;
    __syncthreads();
    for (int b = (int)threadIdx.x; b < ngroups; b += (int)blockDim.x) {
        int j0 = b;
#pragma unroll
        for (int q = 0; q < 2 * K; q++) j0 = insert0(j0, pos[q]);
        const int64_t gi = base | ((int64_t)off_tab[j0 >> L] << osh) | (int64_t)(j0 & lowmask);
        if (((((gi & rmask) ^ (gi >> n)) & (int64_t)g.pmask[0]) == 0)) {
            const int slot = atomicAdd(s_cnt, 1);
            if (slot < kChunkG) s_act[slot] = j0;
        }
    }
    __syncthreads();
    const int nact = min(*s_cnt, kChunkG);
    const int items = nact * DD;
    for (int it0 = 0; it0 < items; it0 += blockDim.x) {
        const int it = it0 + (int)threadIdx.x;
        float4 outv = make_float4(0.f, 0.f, 0.f, 0.f);
        int dst = -1;
        if (it < items) {
            const int j0 = s_act[it / DD], e = it % DD, i = e / D, jj = e % D;
            auto at = [&](int r, int c) {
                int j = j0;
#pragma unroll
                for (int q = 0; q < K; q++) {
                    if ((r >> q) & 1) j |= 1 << g.tbit[q];
                    if ((c >> q) & 1) j |= 1 << g.tbit[K + q];
                }
                return sx<SW>(j);
            };
            ffacc ar{0.f, 0.f}, ai{0.f, 0.f};
            bool first = true;
            for (int q = 0; q < g.npar; q++) {
                const float4* Kq = km + q * DD;
                for (int c = 0; c < D; c++) {
                    ffacc tr, ti;
                    cmac_first(tr, ti, f4m(__ldg(Kq + i * D)), f4c(sm[at(0, c)]));
                    for (int r = 1; r < D; r++) cmac(tr, ti, f4m(__ldg(Kq + i * D + r)), f4c(sm[at(r, c)]));
                    const cff t = cdone(tr, ti);
                    const float4 kj = __ldg(Kq + jj * D + c);
                    const cff kc = {kj.x, kj.y, -kj.z, -kj.w};
                    if (first) { cmac_first(ar, ai, kc, t); first = false; }
                    else cmac(ar, ai, kc, t);
                }
            }
            outv = c4f(cdone(ar, ai));
            dst = at(i, jj);
        }
        __syncthreads();   // every read of the collected blocks is done
        if (dst >= 0) sm[dst] = outv;
        __syncthreads();
    }
}

// KMAX: widest dense/monomial gate of the sweep (2 or 4); narrow sweeps get a
// kernel with fewer live registers and therefore more resident warps.
template <int KMAX, int NT>
__global__ void __launch_bounds__(NT) k_tile_sweep(double2* __restrict__ psi, SweepDesc d, int64_t tile0) {
    extern __shared__ float4 smem[];
    const int T = d.T, L = d.L, H = T - L;
    const int nt = 1 << T;
    int64_t* off_tab = reinterpret_cast<int64_t*>(smem + nt);
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
    // tile load: eight loads per thread in flight at a time (tiles are at most 2^12 amplitudes)
#pragma unroll
    for (int r = 0; r < 4096 / NT; r += 8) {
        double2 x[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int j = (r + i) * NT + (int)threadIdx.x;
            if (j < nt) x[i] = __ldcs(psi + (base | off_tab[j >> L] | (int64_t)(j & lowmask)));
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int j = (r + i) * NT + (int)threadIdx.x;
            if (j < nt) smem[j] = c4f(load_c128(x[i]));
        }
    }
    __syncthreads();
    __shared__ TileGate s_gates[kGateChunk];
    __shared__ int s_act[32], s_cnt;   // kind 5: blocks passing the row/column test
    for (int g0 = 0; g0 < d.n_gates; g0 += kGateChunk) {
    const int ng = min(kGateChunk, d.n_gates - g0);
    stage_gates(s_gates, d.gates + g0, ng);
    for (int gl = 0; gl < ng; gl++) {
        const TileGate& g = s_gates[gl];
        if ((base & (int64_t)g.gc_mask) != (int64_t)g.gc_val) continue;   // uniform in the CTA
        const int kind = g.kind, k = g.k;
        if (kind == 3) {
            for (int j = threadIdx.x; j < nt; j += blockDim.x) {
                const int64_t gi = base | off_tab[j >> L] | (int64_t)(j & lowmask);
                if (parity_odd(g, gi)) { float4 v = smem[j]; smem[j] = make_float4(-v.x, -v.y, -v.z, -v.w); }
            }
        } else if (kind == 1) {
            tile_diag(smem, T, L, g, d.mats, base, off_tab, 0);
        } else if (kind == 5) {
            if (k == 1) tile_kraus_ref_lr<1, false>(smem, T, L, g, d.mats, base, off_tab, 0, d.n_bits / 2, s_act, &s_cnt);
            else tile_kraus_ref_lr<2, false>(smem, T, L, g, d.mats, base, off_tab, 0, d.n_bits / 2, s_act, &s_cnt);
        } else if (kind == 0) {
            if (k == 1) tile_dense<1>(smem, T, g, d.mats);
            else if (k == 2 || KMAX == 2) tile_dense<2>(smem, T, g, d.mats);
            else if (KMAX > 2 && k == 3) tile_dense<3>(smem, T, g, d.mats);
            else if (KMAX > 2) tile_dense<4>(smem, T, g, d.mats);
        } else {
            if (k == 1) tile_monomial<1>(smem, T, g, d.perms);
            else if (k == 2 || KMAX == 2) tile_monomial<2>(smem, T, g, d.perms);
            else if (KMAX > 2 && k == 3) tile_monomial<3>(smem, T, g, d.perms);
            else if (KMAX > 2) tile_monomial<4>(smem, T, g, d.perms);
        }
        __syncthreads();
    }
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        int64_t gidx = base | off_tab[j >> L] | (int64_t)(j & lowmask);
        __stcs(psi + gidx, store_c128(f4c(smem[j])));
    }
}

// Sweep with fused 5-bit unitaries on the tensor cores (gate kind 4), T = 12, L = 5.
// Dynamic shared memory: 48 KiB matrix digit slices | 64 KiB tile (static: split offset tables, the
// per-warp exponents, kind-5 scratch), so that two CTAs fit on an SM; each holds 256 of the SM's 512 TMEM columns (from its first to its last
// fused gate), so one CTA's MMAs overlap the other's CUDA-core work.  The tile is stored with the
// bank swizzle tc::sw.
#ifndef BS_TC_THREADS
#define BS_TC_THREADS 256
#endif
constexpr int kTcThreads = BS_TC_THREADS;   // 256 (128 registers) or 512 (64 registers, spills; measured slower)
constexpr int kTcSmem = 49152 + 65536;

// Global offset (>> 5) of the tile's high-bit pattern i (7 bits) from two small tables:
// a[i & 7] | b[i >> 3].
struct HiOff {
    const uint32_t* a;
    const uint32_t* b;
    __device__ __forceinline__ uint32_t operator[](int i) const { return a[i & 7] | b[i >> 3]; }
};

__global__ void __launch_bounds__(kTcThreads, 2) k_tile_sweep_tc(double2* __restrict__ psi, SweepDesc d, int64_t tile0,
                                                                 int tc_last) {
    // 128-byte alignment: each 128-byte core matrix of the matrix operand sits in one shared-memory line
    extern __shared__ __align__(128) unsigned char dsm[];
    uint16_t* sB = reinterpret_cast<uint16_t*>(dsm);
    float4* smem = reinterpret_cast<float4*>(dsm + 49152);
    __shared__ __align__(8) uint64_t bars[7];   // digit copy, MMAs into D0 / D1, D0 / D1 read, D1 free, D2
    __shared__ uint32_t s_tmem;
    __shared__ int64_t s_base;
    __shared__ int s_fail;
    __shared__ int s_tsw[32];
    __shared__ uint32_t s_offa[8], s_offb[16];
    __shared__ uint32_t s_wmax[kTcThreads / 32];   // per-warp largest high-word exponent field
    __shared__ int s_act[32], s_cnt;                 // kind 5: blocks passing the row/column test
    __shared__ int s_tcq[16], s_ntc;                 // the tile's first 16 fused gates, in order
    __shared__ const uint16_t* s_nsrc;
    const HiOff off32{s_offa, s_offb};
    constexpr int T = 12, L = 5, H = 7, nt = 1 << T, lowmask = (1 << L) - 1;
    const int64_t tile = tile0 + (int64_t)blockIdx.x;
    if (threadIdx.x == 0) {
        int64_t base = 0;
        int src = 0;
        for (int bit = 0; bit < d.n_bits; bit++)
            if (!((d.tile_mask >> bit) & 1ULL)) { base |= ((tile >> src) & 1LL) << bit; src++; }
        s_base = base;
        s_fail = 0;
        tc::mbar_init(tc::su32(&bars[0]));
        tc::mbar_init(tc::su32(&bars[1]));
        tc::mbar_init(tc::su32(&bars[2]));
        tc::mbar_init_n(tc::su32(&bars[3]), kTcThreads / 32);
        tc::mbar_init_n(tc::su32(&bars[4]), kTcThreads / 32);
        tc::mbar_init(tc::su32(&bars[5]));
        tc::mbar_init(tc::su32(&bars[6]));
    }
    if (threadIdx.x < 24) {
        const int i = threadIdx.x < 8 ? threadIdx.x : (threadIdx.x - 8) << 3;
        int64_t o = 0;
        for (int j = 0; j < H; j++) if ((i >> j) & 1) o |= 1LL << d.hi_bits[j];
        if (threadIdx.x < 8) s_offa[threadIdx.x] = (uint32_t)(o >> L);
        else s_offb[threadIdx.x - 8] = (uint32_t)(o >> L);
    }
    __syncthreads();
    const int64_t base = s_base;
    const int warp = threadIdx.x >> 5;
    // tile load: each thread's 16 loads are issued together (coalesced 512 B rows), then converted to
    // float-float at the swizzled positions
    {
        constexpr int NL = nt / kTcThreads;
        double2 x[NL];
#pragma unroll
        for (int i = 0; i < NL; i++) {
            const int j = i * kTcThreads + (int)threadIdx.x;
            x[i] = __ldcs(psi + (base | ((int64_t)off32[j >> L] << L) | (int64_t)(j & lowmask)));
        }
        if (warp == kTcThreads / 32 - 1) {
            // while the loads are in flight: the fused gates this tile runs (those whose controls its
            // base satisfies), and the copy of the first one's digit slices
            const int lane = threadIdx.x & 31;
            int cnt = 0, first = -1;
            for (int c0 = 0; c0 < d.n_gates; c0 += 32) {
                const int gi = c0 + lane;
                bool f = false;
                if (gi < d.n_gates) {
                    const TileGate& g = d.gates[gi];
                    f = g.kind == 4 && (base & (int64_t)g.gc_mask) == (int64_t)g.gc_val;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, f);
                if (f) {
                    const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
                    if (pos < 16) s_tcq[pos] = gi;
                }
                if (first < 0 && bal) first = c0 + __ffs((int)bal) - 1;
                cnt += __popc(bal);
            }
            if (lane == 0) {
                s_ntc = cnt < 16 ? cnt : 16;
                if (first >= 0) tc::copy_slices(tc::su32(sB), tc::slice_src(d.gates[first], d.tc_pool, base), tc::su32(&bars[0]));
            }
        }
        uint32_t eb = 0;
#pragma unroll
        for (int i = 0; i < NL; i++) {
            const float4 v = c4f(load_c128(x[i]));
            smem[tc::sw(i * kTcThreads + (int)threadIdx.x)] = v;
            eb = max(eb, max(__float_as_uint(v.x) & 0x7F800000u, __float_as_uint(v.y) & 0x7F800000u));
        }
        eb = __reduce_max_sync(0xffffffffu, eb);
        if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = eb;
    }
    __syncthreads();
    tc::State st{0u, tc::su32(&bars[0]), 0u, s_ntc > 0};
    int q = 0;   // fused gates run so far
    bool have = false;
    bool emax_ok = true;   // s_wmax holds the tile's largest exponent (no magnitude-changing gate since)
    for (int gi = 0; gi < d.n_gates; gi++) {
        const TileGate& g = d.gates[gi];
        if ((base & (int64_t)g.gc_mask) != (int64_t)g.gc_val) continue;
        const int kind = g.kind, k = g.k;
        if (kind == 0 || kind == 1 || kind == 5) emax_ok = false;   // these may change magnitudes
        if (kind == 4) {
            if (s_fail) continue;
            if (!have) {
                if (warp == 0) tc::tmem_alloc(tc::su32(&s_tmem));
                tc::fence_before();
                __syncthreads();
                tc::fence_after();
                st.tmem = s_tmem;
                have = true;
            }
            const TileGate* gn = q + 1 < s_ntc ? d.gates + s_tcq[q + 1] : nullptr;
            tc::apply<kTcThreads>(smem, g, gn, d.tc_pool, reinterpret_cast<const uint16_t*>(d.perms + g.perm_off), sB,
                                  st, base, s_wmax, emax_ok, s_tsw, &s_nsrc, &s_fail,
                                  d.err);
            q++;
            emax_ok = true;
            if (gi == tc_last) {
                __syncthreads();
                if (warp == 0) tc::tmem_dealloc(st.tmem);
                have = false;
            }
        } else if (kind == 3) {
            for (int j = threadIdx.x; j < nt; j += blockDim.x) {
                const int64_t gg = base | ((int64_t)off32[j >> L] << L) | (int64_t)(j & lowmask);
                if (parity_odd(g, gg)) {
                    const int js = tc::sw(j);
                    float4 v = smem[js];
                    smem[js] = make_float4(-v.x, -v.y, -v.z, -v.w);
                }
            }
        } else if (kind == 1) {
            tile_diag<HiOff, true>(smem, T, L, g, d.mats, base, off32, L);
        } else if (kind == 5) {
            if (k == 1) tile_kraus_ref_lr<1, true, HiOff>(smem, T, L, g, d.mats, base, off32, L, d.n_bits / 2, s_act, &s_cnt);
            else tile_kraus_ref_lr<2, true, HiOff>(smem, T, L, g, d.mats, base, off32, L, d.n_bits / 2, s_act, &s_cnt);

        } else if (kind == 0) {   // the planner routes sweeps with unfused 3- or 4-target gates elsewhere
            if (k == 1) tile_dense<1, true>(smem, T, g, d.mats);
            else tile_dense<2, true>(smem, T, g, d.mats);
        } else {
            if (k == 1) tile_monomial<1, true>(smem, T, g, d.perms);
            else tile_monomial<2, true>(smem, T, g, d.perms);
        }
        __syncthreads();
    }
    if (have) {
        // a wait gave up: give the copies and MMAs in flight a bounded time to land before releasing TMEM
        if (threadIdx.x == 0 && s_fail) {
            tc::mbar_wait(st.bar, st.ph & 1u);
            tc::mbar_wait(st.bar + 8u, (st.ph >> 1) & 1u);
            tc::mbar_wait(st.bar + 16u, (st.ph >> 2) & 1u);
            tc::mbar_wait(st.bar + 48u, (st.ph >> 6) & 1u);
        }
        __syncthreads();
        if (warp == 0) tc::tmem_dealloc(st.tmem);
    }
    // tile store: streaming stores, nothing waits for them
#pragma unroll 4
    for (int i = 0; i < nt / kTcThreads; i++) {
        const int j = i * kTcThreads + (int)threadIdx.x;
        __stcs(psi + (base | ((int64_t)off32[j >> L] << L) | (int64_t)(j & lowmask)), store_c128(f4c(smem[tc::sw(j)])));
    }
}

// Digit slices of the fused matrices for the tensor-core sweep, one CTA per matrix variant.
// mats: complex 32x32 row-major FP64 per variant; scale[v] = 2^(7 - eu) of the variant's gate.
// Entry (n, k) of the real 64x64 embedding (n = 2t'+c' output re/im, k = 2t+c input re/im) is split
// into six balanced digits d_i in [-128, 128] (u 2^(7-eu) = sum_i d_i 2^(-8i), each digit rounded to
// nearest even), digit i stored as the bf16 of d_i 2^(-8i) at its place in the K-major no-swizzle
// operand layout (per digit and k-step a 2 KiB block of 8x8 core matrices: row group n/8 at 256 B,
// K half at 128 B, row n%8 at 16 B).
__global__ void __launch_bounds__(256) k_tc_digits(const double* __restrict__ mats, const double* __restrict__ scale,
                                                   uint16_t* __restrict__ pool) {
    const int v = blockIdx.x;
    const double* m = mats + (size_t)v * 2048;
    uint16_t* dst = pool + (size_t)v * tc::kPoolBlock;
    const double sc = scale[v];
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
        const int n = e >> 6, k = e & 63;
        const int tp = n >> 1, cp = n & 1, t = k >> 1, c = k & 1;
        const double re = m[2 * (tp * 32 + t)], im = m[2 * (tp * 32 + t) + 1];
        const double u = (cp == c) ? re : (cp == 0 ? -im : im);
        double x = u * sc;
        const int s = k >> 4, kc = (k >> 3) & 1, rg = n >> 3, r = n & 7, el = k & 7;
        const int pos = rg * 128 + kc * 64 + r * 8 + el;
#pragma unroll
        for (int i = 0; i < 6; i++) {
            const double d = rint(x);
            x = (x - d) * 256.0;
            const float f = __double2float_rn(d) * __int_as_float((127 - 8 * i) << 23);   // exact: |d| <= 128
            dst[(size_t)(i * 4 + s) * 1024 + pos] = (uint16_t)(__float_as_uint(f) >> 16);
        }
    }
}

// Dense gate with more targets than a tile holds: one CTA per group of 2^k
// amplitudes, gathered into shared memory, rows computed by the CTA's threads.
__global__ void __launch_bounds__(kThreads) k_dense_big(double2* __restrict__ psi, int n_bits, int k,
                                                        const int* __restrict__ ebits, uint64_t cmask,
                                                        uint64_t cval, const float4* __restrict__ mat,
                                                        int64_t group0) {
    extern __shared__ float4 smem[];
    const int D = 1 << k;
    __shared__ int64_t s_base;
    __shared__ int s_skip;
    if (threadIdx.x == 0) {
        // insert zeros at the sorted target bits
        int ord[BS_MAX_TARGETS];
        for (int q = 0; q < k; q++) ord[q] = ebits[q];
        for (int a = 0; a < k; a++)
            for (int b = a + 1; b < k; b++)
                if (ord[b] < ord[a]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
        int64_t x = group0 + (int64_t)blockIdx.x;
        for (int q = 0; q < k; q++) {
            int64_t low = x & ((1LL << ord[q]) - 1);
            x = ((x >> ord[q]) << (ord[q] + 1)) | low;
        }
        s_base = x;
        s_skip = ((uint64_t)x & cmask) != cval;
    }
    __syncthreads();
    if (s_skip) return;
    const int64_t base = s_base;
    for (int c = threadIdx.x; c < D; c += blockDim.x) {
        int64_t gi = base;
        for (int q = 0; q < k; q++) if ((c >> q) & 1) gi |= 1LL << ebits[q];
        smem[c] = c4f(load_c128(psi[gi]));
    }
    __syncthreads();
    float4* outv = smem + D;
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
        ffacc ar, ai;
        cmac_first(ar, ai, f4m(mat[(int64_t)r * D]), f4c(smem[0]));
        for (int c = 1; c < D; c++) cmac(ar, ai, f4m(mat[(int64_t)r * D + c]), f4c(smem[c]));
        outv[r] = c4f(cdone(ar, ai));
    }
    __syncthreads();
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
        int64_t gi = base;
        for (int q = 0; q < k; q++) if ((r >> q) & 1) gi |= 1LL << ebits[q];
        psi[gi] = store_c128(f4c(outv[r]));
    }
}

inline void split_d(double x, float& h, float& l) {
    h = (float)x;
    l = (float)(x - (double)h);
}
// ---------------------------------------------------------------------------
// complex64 states: the same tiles and gate tables, FP32 complex arithmetic
// (the matrix entries are the FP32-rounded hi parts of the float-float table).
__device__ __forceinline__ float2 c64_mul(float4 m, float2 x) {
    return make_float2(fmaf(m.x, x.x, -m.z * x.y), fmaf(m.x, x.y, m.z * x.x));
}
__device__ __forceinline__ float2 c64_ipow(float2 x, int p) {
    switch (p & 3) {
        case 0: return x;
        case 1: return make_float2(-x.y, x.x);
        case 2: return make_float2(-x.x, -x.y);
        default: return make_float2(x.y, -x.x);
    }
}

template <int K>
__device__ void tile_dense_c64(float2* sm, int T, const TileGate& g, const float4* __restrict__ mats) {
    constexpr int D = 1 << K;
    int pos[K], tb[K];
#pragma unroll
    for (int q = 0; q < K; q++) pos[q] = tb[q] = g.tbit[q];
#pragma unroll
    for (int a = 0; a < K; a++)
#pragma unroll
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int ngroups = 1 << (T - K);
    const float4* m = mats + g.mat_off;
    const uint32_t lcm = g.lc_mask, lcv = g.lc_val;
    // 1- and 2-target matrices are held in registers across the thread's groups
    constexpr int MR = K <= 2 ? D * D : 1;
    float mre[MR], mim[MR];
    if (K <= 2) {
#pragma unroll
        for (int e = 0; e < MR; e++) {
            const float4 mv = __ldg(m + e);
            mre[e] = mv.x;
            mim[e] = mv.z;
        }
    }
    for (int gr = threadIdx.x; gr < ngroups; gr += blockDim.x) {
        int jb = gr;
#pragma unroll
        for (int q = 0; q < K; q++) jb = insert0(jb, pos[q]);
        if ((jb & (int)lcm) != (int)lcv) continue;
        float2 x[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
#pragma unroll
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << tb[q];
            idx[c] = j;
            x[c] = sm[j];
        }
#pragma unroll
        for (int r = 0; r < D; r++) {
            float re = 0.f, im = 0.f;
#pragma unroll
            for (int c = 0; c < D; c++) {
                float ar, ai;
                if (K <= 2) { ar = mre[(r * D + c) % MR]; ai = mim[(r * D + c) % MR]; }
                else { const float4 mv = __ldg(m + r * D + c); ar = mv.x; ai = mv.z; }
                re = fmaf(ar, x[c].x, fmaf(-ai, x[c].y, re));
                im = fmaf(ar, x[c].y, fmaf(ai, x[c].x, im));
            }
            sm[idx[r]] = make_float2(re, im);
        }
    }
}

template <int K>
__device__ void tile_mono_c64(float2* sm, int T, const TileGate& g, const int32_t* __restrict__ perms) {
    constexpr int D = 1 << K;
    int pos[K], tb[K];
#pragma unroll
    for (int q = 0; q < K; q++) pos[q] = tb[q] = g.tbit[q];
#pragma unroll
    for (int a = 0; a < K; a++)
#pragma unroll
        for (int b = a + 1; b < K; b++)
            if (pos[b] < pos[a]) { int t = pos[a]; pos[a] = pos[b]; pos[b] = t; }
    const int32_t* p = perms + g.perm_off;
    for (int gr = threadIdx.x; gr < (1 << (T - K)); gr += blockDim.x) {
        int jb = gr;
#pragma unroll
        for (int q = 0; q < K; q++) jb = insert0(jb, pos[q]);
        if ((jb & (int)g.lc_mask) != (int)g.lc_val) continue;
        float2 x[D];
        int idx[D];
#pragma unroll
        for (int c = 0; c < D; c++) {
            int j = jb;
#pragma unroll
            for (int q = 0; q < K; q++) if ((c >> q) & 1) j |= 1 << tb[q];
            idx[c] = j;
            x[c] = sm[j];
        }
#pragma unroll
        for (int c = 0; c < D; c++) {
            const int r = __ldg(p + 2 * c);
            int j = jb;
#pragma unroll
            for (int q = 0; q < K; q++) if ((r >> q) & 1) j |= 1 << tb[q];
            sm[j] = c64_ipow(x[c], __ldg(p + 2 * c + 1));
        }
    }
}

__device__ void tile_diag_c64(float2* sm, int T, int L, const TileGate& g, const float4* __restrict__ mats, int64_t base,
                              const int64_t* off_tab) {
    const int nt = 1 << T, lowmask = (1 << L) - 1;
    const float4* m = mats + g.mat_off;
    if (g.k <= BS_TILE_MAXK) {
        // bit q of the pattern: tile bit tbit[q], or a constant of the CTA when the bit is outside the tile
        int cst = 0, nk = 0;
        uint32_t enc = 0;   // per in-tile pattern bit: tile position (5 bits) | q << 5, one byte each
        for (int q = 0; q < g.k; q++) {
            if (g.tbit[q] >= 0) enc |= (uint32_t)(g.tbit[q] | (q << 5)) << (8 * nk++);
            else cst |= (int)((base >> g.gbit[q]) & 1) << q;
        }
        for (int j = threadIdx.x; j < nt; j += blockDim.x) {
            if ((j & (int)g.lc_mask) != (int)g.lc_val) continue;
            int di = cst;
            for (int u = 0; u < nk; u++) {
                const uint32_t b = (enc >> (8 * u)) & 255u;
                di |= ((j >> (b & 31u)) & 1) << (b >> 5);
            }
            const float4 d = __ldg(m + di);
            if (d.z == 0.f && d.x == 1.f && d.y == 0.f) continue;
            sm[j] = c64_mul(d, sm[j]);
        }
        return;
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        if ((j & (int)g.lc_mask) != (int)g.lc_val) continue;
        const int64_t gi = base | off_tab[j >> L] | (int64_t)(j & lowmask);
        int di = 0;
        for (int q = 0; q < g.k; q++) di |= (int)((gi >> g.gbit[q]) & 1) << q;
        const float4 d = __ldg(m + di);
        if (d.z == 0.f && d.x == 1.f && d.y == 0.f) continue;
        sm[j] = c64_mul(d, sm[j]);
    }
}

template <int KMAX>
__global__ void __launch_bounds__(kThreads, KMAX == 2 ? 4 : 3) k_tile_sweep_c64(float2* __restrict__ psi, SweepDesc d, int64_t tile0) {
    extern __shared__ float4 smem4[];
    float2* smem = reinterpret_cast<float2*>(smem4);
    const int T = d.T, L = d.L, H = T - L;
    const int nt = 1 << T;
    int64_t* off_tab = reinterpret_cast<int64_t*>(smem + nt);
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
    // tile load: eight loads per thread in flight at a time (tiles are at most 2^12 amplitudes)
#pragma unroll
    for (int r = 0; r < 4096 / kThreads; r += 8) {
        float2 x[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int j = (r + i) * kThreads + (int)threadIdx.x;
            if (j < nt) x[i] = __ldcs(psi + (base | off_tab[j >> L] | (int64_t)(j & lowmask)));
        }
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int j = (r + i) * kThreads + (int)threadIdx.x;
            if (j < nt) smem[j] = x[i];
        }
    }
    __syncthreads();
    __shared__ TileGate s_gates[kGateChunk];
    for (int g0 = 0; g0 < d.n_gates; g0 += kGateChunk) {
    const int ng = min(kGateChunk, d.n_gates - g0);
    stage_gates(s_gates, d.gates + g0, ng);
    for (int gl = 0; gl < ng; gl++) {
        const TileGate& g = s_gates[gl];
        if ((base & (int64_t)g.gc_mask) != (int64_t)g.gc_val) continue;
        const int kind = g.kind, k = g.k;
        if (kind == 3) {
            for (int j = threadIdx.x; j < nt; j += blockDim.x) {
                const int64_t gi = base | off_tab[j >> L] | (int64_t)(j & lowmask);
                if (parity_odd(g, gi)) { float2 v = smem[j]; smem[j] = make_float2(-v.x, -v.y); }
            }
        } else if (kind == 1) {
            tile_diag_c64(smem, T, L, g, d.mats, base, off_tab);
        } else if (kind == 0) {
            if (k == 1) tile_dense_c64<1>(smem, T, g, d.mats);
            else if (k == 2 || KMAX == 2) tile_dense_c64<2>(smem, T, g, d.mats);
            else if (KMAX > 2 && k == 3) tile_dense_c64<3>(smem, T, g, d.mats);
            else if (KMAX > 2) tile_dense_c64<4>(smem, T, g, d.mats);
        } else {
            if (k == 1) tile_mono_c64<1>(smem, T, g, d.perms);
            else if (k == 2 || KMAX == 2) tile_mono_c64<2>(smem, T, g, d.perms);
            else if (KMAX > 2 && k == 3) tile_mono_c64<3>(smem, T, g, d.perms);
            else if (KMAX > 2) tile_mono_c64<4>(smem, T, g, d.perms);
        }
        __syncthreads();
    }
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x)
        __stcs(psi + (base | off_tab[j >> L] | (int64_t)(j & lowmask)), smem[j]);
}

__global__ void __launch_bounds__(kThreads) k_dense_big_c64(float2* __restrict__ psi, int n_bits, int k,
                                                            const int* __restrict__ ebits, uint64_t cmask, uint64_t cval,
                                                            const float4* __restrict__ mat, int64_t group0) {
    extern __shared__ float4 smem4[];
    float2* smem = reinterpret_cast<float2*>(smem4);
    const int D = 1 << k;
    __shared__ int64_t s_base;
    __shared__ int s_skip;
    if (threadIdx.x == 0) {
        int ord[BS_MAX_TARGETS];
        for (int q = 0; q < k; q++) ord[q] = ebits[q];
        for (int a = 0; a < k; a++)
            for (int b = a + 1; b < k; b++)
                if (ord[b] < ord[a]) { int t = ord[a]; ord[a] = ord[b]; ord[b] = t; }
        int64_t x = group0 + (int64_t)blockIdx.x;
        for (int q = 0; q < k; q++) {
            int64_t low = x & ((1LL << ord[q]) - 1);
            x = ((x >> ord[q]) << (ord[q] + 1)) | low;
        }
        s_base = x;
        s_skip = ((uint64_t)x & cmask) != cval;
    }
    __syncthreads();
    if (s_skip) return;
    const int64_t base = s_base;
    for (int c = threadIdx.x; c < D; c += blockDim.x) {
        int64_t gi = base;
        for (int q = 0; q < k; q++) if ((c >> q) & 1) gi |= 1LL << ebits[q];
        smem[c] = psi[gi];
    }
    __syncthreads();
    float2* outv = smem + D;
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
        float re = 0.f, im = 0.f;
        for (int c = 0; c < D; c++) {
            const float4 mv = mat[(int64_t)r * D + c];
            re = fmaf(mv.x, smem[c].x, fmaf(-mv.z, smem[c].y, re));
            im = fmaf(mv.x, smem[c].y, fmaf(mv.z, smem[c].x, im));
        }
        outv[r] = make_float2(re, im);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < D; r += blockDim.x) {
        int64_t gi = base;
        for (int q = 0; q < k; q++) if ((r >> q) & 1) gi |= 1LL << ebits[q];
        psi[gi] = outv[r];
    }
}


inline float4 to_cff(double re, double im) {
    float4 v;
    split_d(re, v.x, v.y);
    split_d(im, v.z, v.w);
    return v;
}

}  // namespace

namespace {

bool plain_cz(const HostGate& h) {
    return h.kind == 1 && h.k == 1 && h.mat.size() == 4 && h.mat[0] == 1.0 && h.mat[1] == 0.0 && h.mat[2] == -1.0 &&
           h.mat[3] == 0.0 && __builtin_popcountll(h.cmask) == 1 && h.cval == h.cmask;
}

uint64_t gate_bits(const HostGate& h) {
    uint64_t m = h.cmask;
    if (h.kind == 5) return ~0ULL;
    for (int q = 0; q < h.k; q++) m |= 1ULL << h.ebit[q];
    return m;
}

// Diagonal gates (other than CZ, which merge into parity phases when packed) are folded into one
// diagonal table over the union of their bits, up to kMaxMergedDiag bits.  The open table floats
// forward past gates it commutes with (diagonal ones, and any gate on other bits), and is emitted
// before the first non-diagonal gate that touches one of its bits.  One pass over the tile then
// replaces a pass per gate.
constexpr int kMaxMergedDiag = BS_TILE_MAXK;

struct DiagTable {
    uint64_t bits = 0;                 // endian bits, ascending in ebit order
    std::vector<int> eb;
    std::vector<std::complex<double>> d;
};

void diag_absorb(DiagTable& t, const HostGate& h) {
    const uint64_t nb = t.bits | gate_bits(h);
    std::vector<int> eb;
    for (int e = 0; e < 64; e++) if ((nb >> e) & 1ULL) eb.push_back(e);
    const int k = (int)eb.size();
    std::vector<std::complex<double>> d((size_t)1 << k);
    for (int x = 0; x < (1 << k); x++) {
        uint64_t g = 0;   // the assignment x on the endian bits
        for (int q = 0; q < k; q++) if ((x >> q) & 1) g |= 1ULL << eb[(size_t)q];
        std::complex<double> v(1.0, 0.0);
        if (!t.eb.empty() || t.bits == 0) {
            int xi = 0;
            for (size_t q = 0; q < t.eb.size(); q++) xi |= (int)((g >> t.eb[q]) & 1ULL) << q;
            if (!t.d.empty()) v = t.d[(size_t)xi];
        }
        if ((g & h.cmask) == h.cval) {
            int hi = 0;
            for (int q = 0; q < h.k; q++) hi |= (int)((g >> h.ebit[q]) & 1ULL) << q;
            v *= std::complex<double>(h.mat[2 * hi], h.mat[2 * hi + 1]);
        }
        d[(size_t)x] = v;
    }
    t.bits = nb;
    t.eb = eb;
    t.d = d;
}

void merge_diagonals(const std::vector<HostGate>& in, std::vector<HostGate>& out) {
    out.clear();
    DiagTable open;
    int n_open = 0;
    const HostGate* first = nullptr;
    // CZ gates float forward the same way and are emitted together sorted by the distance of their
    // two bits, so that the packer folds each distance into one parity-phase term
    std::vector<const HostGate*> czs;
    uint64_t cz_bits = 0;
    auto cz_dist = [](const HostGate* h) {
        const int c = 63 - __builtin_clzll(h->cmask), t = h->ebit[0];
        return c > t ? c - t : t - c;
    };
    auto flush_cz = [&]() {
        std::stable_sort(czs.begin(), czs.end(), [&](const HostGate* a, const HostGate* b) { return cz_dist(a) < cz_dist(b); });
        for (const HostGate* h : czs) out.push_back(*h);
        czs.clear();
        cz_bits = 0;
    };
    auto flush = [&]() {
        if (n_open == 1) {
            out.push_back(*first);   // a single gate keeps its own form
        } else if (n_open > 1) {
            HostGate m;
            m.kind = 1;
            m.k = (int)open.eb.size();
            for (int q = 0; q < m.k; q++) m.ebit[q] = open.eb[(size_t)q];
            m.mat.resize(2 * open.d.size());
            for (size_t x = 0; x < open.d.size(); x++) {
                m.mat[2 * x] = open.d[x].real();
                m.mat[2 * x + 1] = open.d[x].imag();
            }
            out.push_back(std::move(m));
        }
        open = DiagTable{};
        n_open = 0;
        first = nullptr;
    };
    for (const HostGate& h : in) {
        if (plain_cz(h)) {
            czs.push_back(&h);
            cz_bits |= gate_bits(h);
            continue;
        }
        const bool mergeable = h.kind == 1 && __builtin_popcountll(gate_bits(h)) <= kMaxMergedDiag;
        if (mergeable) {
            if (n_open && __builtin_popcountll(open.bits | gate_bits(h)) > kMaxMergedDiag) flush();
            if (n_open == 0) first = &h;
            diag_absorb(open, h);
            n_open++;
            continue;
        }
        if (h.kind != 1) {
            if (n_open && (gate_bits(h) & open.bits)) flush();
            if (!czs.empty() && (gate_bits(h) & cz_bits)) flush_cz();
        }
        out.push_back(h);
    }
    flush();
    flush_cz();
}

}  // namespace

namespace {
// The tensor-core sweep's offsets of a fused gate on tile bits tb[0..4], in its bank-swizzled tile
// (tc::sw, restated here for the host): 56 uint16 packed two per int32 — sw of the deposit of a
// column index's bits 0..3 and 4..6 into the 7 other tile bits (ascending), then sw of each of the 32
// target patterns.  The swizzle is linear over XOR, so sw(column) = table[m & 15] ^ table[16 + (m >> 4)].
int host_sw(int j) { return j ^ (((j >> 3) ^ (j >> 6) ^ (j >> 9)) & 7); }
void tc_offset_tables(const int32_t* tb, std::vector<int32_t>& out) {
    uint32_t tmask = 0;
    for (int q = 0; q < 5; q++) tmask |= 1u << tb[q];
    int nb[7], k = 0;
    for (int b = 0; b < 12; b++)
        if (!((tmask >> b) & 1u)) nb[k++] = b;
    uint16_t v[56];
    for (int i = 0; i < 16; i++) {
        int p = 0;
        for (int j = 0; j < 4; j++) if ((i >> j) & 1) p |= 1 << nb[j];
        v[i] = (uint16_t)host_sw(p);
    }
    for (int i = 0; i < 8; i++) {
        int p = 0;
        for (int j = 0; j < 3; j++) if ((i >> j) & 1) p |= 1 << nb[4 + j];
        v[16 + i] = (uint16_t)host_sw(p);
    }
    for (int t = 0; t < 32; t++) {
        int p = 0;
        for (int q = 0; q < 5; q++) if ((t >> q) & 1) p |= 1 << tb[q];
        v[24 + t] = (uint16_t)host_sw(p);
    }
    for (int i = 0; i < 28; i++) out.push_back((int32_t)((uint32_t)v[2 * i] | ((uint32_t)v[2 * i + 1] << 16)));
}
}  // namespace

int bs_run_sweeps(bs_sim* s, const std::vector<Sweep>& sweeps) {
    if (sweeps.empty()) return BS_OK;
    const int n_bits = bs_vec_bits(s);
    const int T = std::min(bs_tile_bits(s), n_bits);
    const int L = std::min(BS_TILE_LOW_BITS, T);
    // pack: per sweep [TileGate...], then one float4 pool, then one int pool
    std::vector<TileGate> tg;
    std::vector<float4> mats;
    std::vector<int32_t> perms;
    struct Launch {
        int64_t gate0; int n_gates; std::vector<int> hi; bool big; int big_gate; int kmax = 1;
        int tc_last = -1;          // index (within the sweep) of the last fused tensor-core gate, -1 if none
        int n_tc = 0;
    };
    std::vector<Launch> launches;
    std::vector<int32_t> big_bits;
    std::vector<double> tc_mats, tc_scale;   // fused matrices (complex 32x32 per variant), 2^(7-eu) per variant
    int64_t n_var = 0;
    const bool c64 = s->precision == BS_PREC_C64;
    // fused tensor-core sweeps from bs_tc_min_bits vector bits up (22 by default: measured wins at
    // 24, 26, 28 and 30 bits; small states are dominated by host planning)
    const bool use_tc = bs_tc_enabled(s) && !c64 && T == 12 && L == 5 && n_bits >= bs_tc_min_bits(s);
    const double tc_threshold = bs_tc_cost(s);
    // fusion per sweep (independent, so on a few host threads); a sweep left with unfused 3/4-target
    // gates or with reference-mode channels keeps its plain gate list, since the tensor-core sweep
    // kernel carries float-float paths for 1- and 2-target gates only
    std::vector<std::vector<HostGate>> fused_all(use_tc ? sweeps.size() : 0);
    std::vector<char> fused_ok(fused_all.size(), 0);
    if (use_tc) {
        auto work = [&](size_t first, size_t step) {
            for (size_t i = first; i < sweeps.size(); i += step) {
                const Sweep& sw = sweeps[i];
                if ((int)sw.hi_bits.size() != T - L) continue;
                int local[64];
                for (int b = 0; b < 64; b++) local[b] = -1;
                for (int b = 0; b < L; b++) local[b] = b;
                for (size_t q = 0; q < sw.hi_bits.size(); q++) local[sw.hi_bits[q]] = L + (int)q;
                bs_fuse_tc(sw.gates, local, T, tc_threshold, fused_all[i]);
                bool ok = true;
                for (const HostGate& hg : fused_all[i])
                    if (hg.kind != 1 && hg.kind != 4 && hg.kind != 5 && hg.k >= 3) ok = false;
                fused_ok[i] = ok;
            }
        };
        const unsigned hw = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
        const size_t nth = std::min<size_t>(sweeps.size(), hw);
        if (nth <= 1) {
            work(0, 1);
        } else {
            std::vector<std::thread> th;
            for (size_t t = 0; t < nth; t++) th.emplace_back(work, t, nth);
            for (std::thread& x : th) x.join();
        }
    }
    size_t swi = 0;
    for (const Sweep& sw : sweeps) {
        const size_t si = swi++;
        Launch ln;
        ln.gate0 = (int64_t)tg.size();
        ln.n_gates = 0;
        ln.hi = sw.hi_bits;
        ln.big = false;
        ln.big_gate = -1;
        // tile-local position of each endian bit
        int local[64];
        for (int b = 0; b < 64; b++) local[b] = -1;
        for (int b = 0; b < L; b++) local[b] = b;
        for (size_t i = 0; i < sw.hi_bits.size(); i++) local[sw.hi_bits[i]] = L + (int)i;
        std::vector<HostGate> merged, small;
        if (use_tc && fused_ok[si]) {
            merge_diagonals(fused_all[si], merged);
        } else if (c64) {
            // complex64 sweep: 1- and 2-bit runs fused into dense 2-bit gates where that saves passes (a
            // pass of the complex64 kernel costs about four 1-qubit gates' arithmetic; batch of 512
            // circuits 1.79 -> 1.48 s on the device).  The float-float kernel is bound by its
            // arithmetic: fusing there measured slower (18 qubits: 7.7 -> 9.2 ms)
            bs_fuse_small(sw.gates, local, 4.0, 2, small);
            merge_diagonals(small, merged);
        } else {
            merge_diagonals(sw.gates, merged);
        }
        const std::vector<HostGate>* glist = &merged;
        for (const HostGate& hg : *glist) {
            if (hg.kind == 5) {
                // reference-rule channel: its row and column target bits are tile bits (the planner needs them)
                TileGate t{};
                t.kind = 5;
                t.k = hg.k;
                const int nq = n_bits / 2, D = 1 << hg.k;
                uint64_t rt = 0;
                for (int q = 0; q < 2 * hg.k; q++) t.tbit[q] = local[hg.ebit[q]];
                for (int q = 0; q < hg.k; q++) rt |= 1ULL << hg.ebit[q];
                const uint64_t nt = (((uint64_t)1 << nq) - 1) & ~rt;
                uint64_t unif = 0;
                for (int b = 0; b < nq; b++)
                    if (((nt >> b) & 1ULL) && local[b] < 0 && local[b + nq] < 0) unif |= 1ULL << b;
                t.pmask[0] = nt;
                t.pmask[1] = unif;
                t.npar = (int32_t)(hg.mat.size() / (size_t)(2 * D * D));
                t.mat_off = (int32_t)mats.size();
                for (size_t e = 0; e + 1 < hg.mat.size(); e += 2) mats.push_back(to_cff(hg.mat[e], hg.mat[e + 1]));
                tg.push_back(t);
                ln.n_gates++;
                continue;
            }
            if (hg.kind == 4) {
                TileGate t{};
                t.kind = 4;
                t.k = 5;
                for (int q = 0; q < 5; q++) t.gbit[q] = local[hg.ebit[q]];
                t.perm_off = (int32_t)perms.size();
                tc_offset_tables(t.gbit, perms);
                const int nvar = 1 << hg.ubits.size();
                t.tc_nu = (int32_t)hg.ubits.size();
                for (size_t i = 0; i < hg.ubits.size(); i++) t.tc_ub[i] = hg.ubits[i];
                t.tc_off = (int32_t)n_var;
                int eu = 0;
                if (!bs_tc_exponent(hg.mat.data(), nvar, eu))
                    return bs_fail(s, BS_ERR_INVALID_ARG, "fused gate matrix out of range");
                tc_mats.insert(tc_mats.end(), hg.mat.begin(), hg.mat.begin() + (size_t)nvar * 2048);
                for (int v = 0; v < nvar; v++) tc_scale.push_back(std::ldexp(1.0, 7 - eu));
                n_var += nvar;
                t.tc_eu = eu;
                ln.tc_last = ln.n_gates;
                ln.n_tc++;
                tg.push_back(t);
                ln.n_gates++;
                continue;
            }
            // consecutive CZ gates (Z on one bit, one control at value 1) merge into one parity-phase gate
            if (hg.kind == 1 && hg.k == 1 && hg.mat.size() == 4 && hg.mat[0] == 1.0 && hg.mat[1] == 0.0 &&
                hg.mat[2] == -1.0 && hg.mat[3] == 0.0 && __builtin_popcountll(hg.cmask) == 1 && hg.cval == hg.cmask) {
                const int c = 63 - __builtin_clzll(hg.cmask), t = hg.ebit[0];
                const int lo = std::min(c, t), dd = std::max(c, t) - lo;
                auto add_pair = [&](TileGate& g) {
                    for (int q = 0; q < g.npar; q++)
                        if (g.pshift[q] == dd) { g.pmask[q] ^= 1ULL << lo; return true; }   // CZ twice = identity
                    if (g.npar == 4) return false;
                    g.pshift[g.npar] = dd;
                    g.pmask[g.npar] = 1ULL << lo;
                    g.npar++;
                    return true;
                };
                if (!(ln.n_gates > 0 && tg.back().kind == 3 && add_pair(tg.back()))) {
                    TileGate t3{};
                    t3.kind = 3;
                    add_pair(t3);
                    tg.push_back(t3);
                    ln.n_gates++;
                }
                continue;
            }
            bool big = hg.kind != 1 && hg.k > BS_TILE_MAXK;
            if (!big && hg.kind != 1)
                for (int q = 0; q < hg.k; q++) if (local[hg.ebit[q]] < 0) big = true;
            if (big) {
                // runs alone: sweeps hold a single out-of-tile gate
                ln.big = true;
                ln.big_gate = (int)tg.size();
                TileGate t{};
                t.kind = hg.kind;
                t.k = hg.k;
                t.gc_mask = hg.cmask;
                t.gc_val = hg.cval;
                t.mat_off = (int32_t)mats.size();
                t.perm_off = (int32_t)big_bits.size();
                for (int q = 0; q < hg.k; q++) big_bits.push_back(hg.ebit[q]);
                if (hg.kind == 0) {
                    for (int i = 0; i < (1 << (2 * hg.k)); i++) mats.push_back(to_cff(hg.mat[2 * i], hg.mat[2 * i + 1]));
                } else {
                    // monomial given as dense
                    int D = 1 << hg.k;
                    std::vector<float4> dense((size_t)D * D, make_float4(0, 0, 0, 0));
                    for (int c = 0; c < D; c++) {
                        int r = hg.perm[2 * c], p = hg.perm[2 * c + 1] & 3;
                        double re = (p == 0) ? 1 : (p == 2 ? -1 : 0), im = (p == 1) ? 1 : (p == 3 ? -1 : 0);
                        dense[(size_t)r * D + c] = to_cff(re, im);
                    }
                    t.kind = 0;
                    mats.insert(mats.end(), dense.begin(), dense.end());
                }
                tg.push_back(t);
                ln.n_gates++;
                continue;
            }
            TileGate t{};
            t.kind = hg.kind;
            t.k = hg.k;
            uint64_t gcm = 0, gcv = 0;
            uint32_t lcm = 0, lcv = 0;
            for (int b = 0; b < n_bits; b++) {
                if (!((hg.cmask >> b) & 1ULL)) continue;
                uint64_t v = (hg.cval >> b) & 1ULL;
                if (local[b] >= 0) { lcm |= 1u << local[b]; lcv |= (uint32_t)v << local[b]; }
                else { gcm |= 1ULL << b; gcv |= v << b; }
            }
            t.lc_mask = lcm; t.lc_val = lcv; t.gc_mask = gcm; t.gc_val = gcv;
            for (int q = 0; q < hg.k; q++) {
                t.gbit[q] = hg.ebit[q];
                if (q < BS_TILE_MAXK) t.tbit[q] = local[hg.ebit[q]];
            }
            t.mat_off = (int32_t)mats.size();
            t.perm_off = (int32_t)perms.size();
            if (hg.kind == 0) {
                for (int i = 0; i < (1 << (2 * hg.k)); i++) mats.push_back(to_cff(hg.mat[2 * i], hg.mat[2 * i + 1]));
            } else if (hg.kind == 1) {
                for (int i = 0; i < (1 << hg.k); i++) mats.push_back(to_cff(hg.mat[2 * i], hg.mat[2 * i + 1]));
            } else {
                perms.insert(perms.end(), hg.perm.begin(), hg.perm.end());
            }
            if (hg.kind != 1) ln.kmax = std::max(ln.kmax, hg.k);
            tg.push_back(t);
            ln.n_gates++;
        }
        launches.push_back(std::move(ln));
    }
    // upload
    auto al = [](int64_t x) { return (x + 255) & ~(int64_t)255; };
    int64_t b_tg = al((int64_t)tg.size() * (int64_t)sizeof(TileGate));
    int64_t b_m = al((int64_t)mats.size() * (int64_t)sizeof(float4));
    int64_t b_p = al((int64_t)(perms.size() + big_bits.size() + 1) * (int64_t)sizeof(int32_t));
    int64_t b_tm = al((int64_t)tc_mats.size() * (int64_t)sizeof(double));
    int64_t b_ts = al((int64_t)tc_scale.size() * (int64_t)sizeof(double));
    int64_t b_tc = al(n_var * tc::kPoolBlock * (int64_t)sizeof(uint16_t));   // written on the device
    const int64_t o_tm = b_tg + b_m + b_p, o_ts = o_tm + b_tm, o_tc = o_ts + b_ts;
    int rc = bs_ensure_plan(s, o_tc + b_tc);
    if (rc) return rc;
    char* host = bs_stage(s, (size_t)o_tc);
    if (!host) return bs_fail(s, BS_ERR_ALLOC, "pinned staging allocation");
    std::memset(host, 0, (size_t)o_tc);
    if (!tc_mats.empty()) {
        std::memcpy(host + o_tm, tc_mats.data(), tc_mats.size() * sizeof(double));
        std::memcpy(host + o_ts, tc_scale.data(), tc_scale.size() * sizeof(double));
    }
    if (!tg.empty()) std::memcpy(host, tg.data(), tg.size() * sizeof(TileGate));
    if (!mats.empty()) std::memcpy(host + b_tg, mats.data(), mats.size() * sizeof(float4));
    if (!perms.empty()) std::memcpy(host + b_tg + b_m, perms.data(), perms.size() * sizeof(int32_t));
    if (!big_bits.empty())
        std::memcpy(host + b_tg + b_m + perms.size() * sizeof(int32_t), big_bits.data(), big_bits.size() * sizeof(int32_t));
    char* dev = (char*)s->plan_buf;
    rc = bs_cuda_check(s, cudaMemcpyAsync(dev, host, (size_t)o_tc, cudaMemcpyHostToDevice, s->stream), "plan upload");
    bs_stage_done(s);
    if (rc) return rc;
    const TileGate* d_tg = (const TileGate*)dev;
    const float4* d_m = (const float4*)(dev + b_tg);
    const int32_t* d_p = (const int32_t*)(dev + b_tg + b_m);
    const int32_t* d_big = d_p + perms.size();

    const int H = T - L;
    const size_t smem = ((size_t)1 << T) * sizeof(float4) + ((size_t)1 << H) * sizeof(int64_t);
    static bool attr_set[64] = {false};
    if (!attr_set[s->device & 63]) {
        // largest carveout: three 65 KiB tiles per SM instead of two
        auto attrs = [](const void* f) {
            cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
            cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        };
        attrs((const void*)k_tile_sweep<2, 256>);
        attrs((const void*)k_tile_sweep<4, 256>);
        attrs((const void*)k_tile_sweep<2, 512>);
        attrs((const void*)k_tile_sweep<4, 512>);
        attrs((const void*)k_tile_sweep_c64<2>);
        attrs((const void*)k_tile_sweep_c64<4>);
        cudaFuncSetAttribute(k_dense_big_c64, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
        cudaFuncSetAttribute(k_dense_big, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
        cudaFuncSetAttribute(k_tile_sweep_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
        cudaFuncSetAttribute(k_tile_sweep_tc, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        attr_set[s->device & 63] = true;
    }
    double2* psi = (double2*)s->state;
    uint16_t* d_tc = (uint16_t*)(dev + o_tc);
    if (n_var) {
        k_tc_digits<<<(unsigned)n_var, 256, 0, s->stream>>>((const double*)(dev + o_tm), (const double*)(dev + o_ts), d_tc);
        s->stats.kernel_launches++;
        if (!s->dev_flag) {
            rc = bs_cuda_check(s, cudaMalloc((void**)&s->dev_flag, 256), "flag alloc");
            if (rc) return rc;
        }
        if (!s->flag_armed) {
            rc = bs_cuda_check(s, cudaMemsetAsync(s->dev_flag, 0, sizeof(int), s->stream), "flag reset");
            if (rc) return rc;
            s->flag_armed = true;
        }
    }
    const double esz = c64 ? 8.0 : 16.0;          // bytes per stored amplitude
    const int64_t ntiles = (int64_t)1 << (n_bits - T);
    for (size_t li = 0; li < launches.size(); li++) {
        const Launch& ln = launches[li];
        if (ln.big) {
            const TileGate& t = tg[(size_t)ln.big_gate];
            int64_t groups = (int64_t)1 << (n_bits - t.k);
            size_t bsm = ((size_t)2 << t.k) * sizeof(float4);
            if (bsm > 100 * 1024) return bs_fail(s, BS_ERR_UNSUPPORTED, "gate has too many targets");
            for (int64_t g0 = 0; g0 < groups; g0 += 1LL << 30) {
                int64_t ng = std::min<int64_t>(groups - g0, 1LL << 30);
                if (c64)
                    k_dense_big_c64<<<(unsigned)ng, kThreads, bsm, s->stream>>>((float2*)s->state, n_bits, t.k,
                                                                              d_big + t.perm_off, t.gc_mask, t.gc_val,
                                                                              d_m + t.mat_off, g0);
                else
                    k_dense_big<<<(unsigned)ng, kThreads, bsm, s->stream>>>(psi, n_bits, t.k, d_big + t.perm_off,
                                                                            t.gc_mask, t.gc_val, d_m + t.mat_off, g0);
            }
            s->stats.kernel_launches++;
            s->stats.sweeps++;
            s->stats.gates++;
            s->stats.bytes_moved += 2.0 * esz * (double)s->len;
            continue;
        }
        SweepDesc d{};
        d.n_bits = n_bits;
        d.T = T;
        d.L = L;
        d.n_gates = ln.n_gates;
        uint64_t tm = (L >= 64) ? ~0ULL : ((1ULL << L) - 1);
        for (int i = 0; i < H; i++) { d.hi_bits[i] = ln.hi[(size_t)i]; tm |= 1ULL << ln.hi[(size_t)i]; }
        d.tile_mask = tm;
        d.gates = d_tg + ln.gate0;
        d.mats = d_m;
        d.perms = d_p;
        d.tc_pool = d_tc;
        d.err = s->dev_flag;
        for (int64_t t0 = 0; t0 < ntiles; t0 += (1LL << 30)) {
            int64_t nb = std::min<int64_t>(ntiles - t0, 1LL << 30);
            if (ln.tc_last >= 0 && s->capturing) {
                k_tile_sweep_tc<<<(unsigned)nb, kTcThreads, kTcSmem, s->stream>>>(psi, d, t0, ln.tc_last);
                s->stats.tc_launches++;
            } else if (ln.tc_last >= 0) {
                const size_t pe = 2 * s->tc_events_used;
                while (s->tc_events.size() < pe + 2) {
                    cudaEvent_t e;
                    rc = bs_cuda_check(s, cudaEventCreate(&e), "event");
                    if (rc) return rc;
                    s->tc_events.push_back(e);
                }
                cudaEventRecord(s->tc_events[pe], s->stream);
                k_tile_sweep_tc<<<(unsigned)nb, kTcThreads, kTcSmem, s->stream>>>(psi, d, t0, ln.tc_last);
                cudaEventRecord(s->tc_events[pe + 1], s->stream);
                s->tc_events_used++;
                s->stats.tc_launches++;
            } else if (c64) {
                const size_t sm64 = ((size_t)1 << T) * sizeof(float2) + ((size_t)1 << H) * sizeof(int64_t);
                if (ln.kmax <= 2) k_tile_sweep_c64<2><<<(unsigned)nb, kThreads, sm64, s->stream>>>((float2*)s->state, d, t0);
                else k_tile_sweep_c64<4><<<(unsigned)nb, kThreads, sm64, s->stream>>>((float2*)s->state, d, t0);
            } else if (bs_tile_threads(s) == 512) {
                if (ln.kmax <= 2) k_tile_sweep<2, 512><<<(unsigned)nb, 512, smem, s->stream>>>(psi, d, t0);
                else k_tile_sweep<4, 512><<<(unsigned)nb, 512, smem, s->stream>>>(psi, d, t0);
            } else {
                if (ln.kmax <= 2) k_tile_sweep<2, 256><<<(unsigned)nb, 256, smem, s->stream>>>(psi, d, t0);
                else k_tile_sweep<4, 256><<<(unsigned)nb, 256, smem, s->stream>>>(psi, d, t0);
            }
        }
        s->stats.kernel_launches++;
        s->stats.sweeps++;
        s->stats.gates += ln.n_gates;
        s->stats.tc_gates += ln.n_tc;
        s->stats.bytes_moved += 2.0 * esz * (double)s->len;
    }
    return bs_cuda_check(s, cudaGetLastError(), "tile sweep launch");
}

void bs_collect_tc_time(bs_sim* s) {
    for (size_t i = 0; i < s->tc_events_used; i++) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->tc_events[2 * i], s->tc_events[2 * i + 1]) == cudaSuccess)
            s->stats.tc_ms += ms;
    }
    s->tc_events_used = 0;
}

namespace {
// A wait that nothing completes: one thread waits on a fresh mbarrier (no arrival, no copy and no MMA
// in flight) with the tensor-core sweep's bounded wait, gives up after `limit` cycles and raises the
// device flag, as a sweep whose copy or MMA never landed would.
__global__ void k_wait_selftest(int* __restrict__ err, long long limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) tc::mbar_init(tc::su32(&bar));
    __syncthreads();
    if (threadIdx.x == 0 && !tc::mbar_wait_for(tc::su32(&bar), 0u, limit)) atomicExch(err, 1);
}
}  // namespace

extern "C" int bs_selftest_wait_timeout(bs_sim* s, double seconds) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!(seconds > 0.0) || seconds > 1.0) return bs_fail(s, BS_ERR_INVALID_ARG, "wait limit must be in (0, 1] s");
    if (s->capturing) return bs_fail(s, BS_ERR_STATE, "not during graph capture");
    int rc = BS_OK;
    if (!s->dev_flag) {
        rc = bs_cuda_check(s, cudaMalloc((void**)&s->dev_flag, 256), "flag alloc");
        if (rc) return rc;
    }
    rc = bs_cuda_check(s, cudaMemsetAsync(s->dev_flag, 0, sizeof(int), s->stream), "flag reset");
    if (rc) return rc;
    s->flag_armed = true;
    k_wait_selftest<<<1, 32, 0, s->stream>>>(s->dev_flag, (long long)(seconds * 2.0e9));
    rc = bs_cuda_check(s, cudaGetLastError(), "self-test launch");
    if (rc) return rc;
    rc = bs_check_device_flag(s);
    if (rc == BS_ERR_TIMEOUT) return bs_fail(s, BS_ERR_TIMEOUT, "self-test: the bounded wait gave up and raised the device flag");
    if (rc == BS_OK) return bs_fail(s, BS_ERR_STATE, "self-test: the wait completed");
    return rc;
}

int bs_check_device_flag(bs_sim* s) {
    if (!s->flag_armed) return BS_OK;
    s->flag_armed = false;
    int flag = 0;
    const int rc = bs_copy_out(s, &flag, s->dev_flag, sizeof(int), "flag read");
    if (rc) return rc;
    if (flag) return bs_fail(s, BS_ERR_TIMEOUT, "a tensor-core sweep gave up waiting for its copies or MMAs");
    return BS_OK;
}

// ---------------------------------------------------------------------------
// Whole small state vectors in one CTA (bs_run_small): the reference's simulate of a small circuit
// (src/BraketSimulator.jl:307-322: reinit!, evolve!, then results) as one launch.  The CTA builds
// |0...0> in shared memory, applies every gate of the planned sweeps in order with the tile kernels'
// float-float gates (the whole state is the tile, so sweep boundaries cost nothing), writes the state
// back and the probabilities, computed from the stored complex128 values exactly as bs_probabilities
// computes them.
namespace {

struct NoOff {
    __device__ __forceinline__ int64_t operator[](int) const { return 0; }
};

__device__ __forceinline__ int64_t globaltimer_ns() {
    int64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The end of a small run, for a host that polls instead of synchronising: the kernel's end time, then
// every thread's writes are made visible to the system, then one thread writes the call's ticket into
// the host-mapped word.
__device__ __forceinline__ void small_run_done(volatile int64_t* done, int64_t ticket, int64_t* times) {
    if (!done) return;
    if (times && threadIdx.x == 0) times[1] = globaltimer_ns();
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) *done = ticket;
}

// STAGED: the matrices and permutations are copied into shared memory first (one round trip to the
// plan, which may live in host-mapped memory) instead of being read from the plan at every gate.
template <int KMAX, bool STAGED>
__global__ void __launch_bounds__(512) k_small_run(double2* __restrict__ psi, int n, const TileGate* __restrict__ gates,
                                                   int ng, const float4* __restrict__ mats, int n_mats,
                                                   const int32_t* __restrict__ perms, int n_perms,
                                                   double* __restrict__ probs, int64_t shots, uint64_t seed,
                                                   int64_t* __restrict__ samples, volatile int64_t* done, int64_t ticket,
                                                   int64_t* times) {
    if (times && threadIdx.x == 0) times[0] = globaltimer_ns();
    extern __shared__ float4 smem[];
    __shared__ float s_ch[kCpb], s_cl[kCpb];
    __shared__ double s_cinc[kCpb], s_total;
    __shared__ long long s_ckey[kCpb];
    __shared__ TileGate s_gates[kGateChunk];
    const int nt = 1 << n, nc32 = (nt + kChunk - 1) / kChunk * kChunk;
    // the probabilities, after the tile (or after the sampler's two arrays, which replace the tile),
    // then the staged matrices and permutations
    double* sprob = reinterpret_cast<double*>(reinterpret_cast<char*>(smem) + max(nt * 16, 2 * nc32 * 8));
    const float4* m_op = mats;
    const int32_t* p_op = perms;
    if (STAGED) {
        float4* ms = reinterpret_cast<float4*>(sprob + nt);
        int32_t* ps = reinterpret_cast<int32_t*>(ms + n_mats);
        for (int j = threadIdx.x; j < n_mats; j += blockDim.x) ms[j] = mats[j];
        for (int j = threadIdx.x; j < n_perms; j += blockDim.x) ps[j] = perms[j];
        m_op = ms;
        p_op = ps;   // read after the barrier that opens the first chunk of gates
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) smem[j] = make_float4(j == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
    for (int gi = 0; gi < ng; gi++) {
        if (gi % kGateChunk == 0) stage_gates(s_gates, gates + gi, min(kGateChunk, ng - gi));   // one latency per 32 gates
        const TileGate& g = s_gates[gi % kGateChunk];
        const int kind = g.kind, k = g.k;
        if (kind == 0) {
            if (k == 1) tile_dense<1, false, STAGED>(smem, n, g, m_op);
            else if (k == 2) tile_dense<2, false, STAGED>(smem, n, g, m_op);
            else if (KMAX == 4 && k == 3) tile_dense<3, false, STAGED>(smem, n, g, m_op);
            else if (KMAX == 4) tile_dense<4, false, STAGED>(smem, n, g, m_op);
        } else if (kind == 1) {
            tile_diag<NoOff, false, STAGED>(smem, n, n, g, m_op, 0, NoOff{}, 0);
        } else {
            if (k == 1) tile_monomial<1, false, STAGED>(smem, n, g, p_op);
            else if (k == 2) tile_monomial<2, false, STAGED>(smem, n, g, p_op);
            else if (KMAX == 4 && k == 3) tile_monomial<3, false, STAGED>(smem, n, g, p_op);
            else if (KMAX == 4) tile_monomial<4, false, STAGED>(smem, n, g, p_op);
        }
        __syncthreads();
    }
    for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const double2 v = store_c128(f4c(smem[j]));
        psi[j] = v;
        const cff x = load_c128(v);
        ffacc a;
        acc_first(a, x.rh, x.rl, x.rh, x.rl);
        acc_add(a, x.ih, x.il, x.ih, x.il);
        const ff r = acc_done(a);
        const double pj = ff2d(r.h, r.l);   // prob_at's value for this amplitude
        probs[j] = pj;
        sprob[j] = pj;
    }
    __syncthreads();
    if (shots <= 0) {
        small_run_done(done, ticket, times);
        return;
    }
    // The shots, as bs_sample draws them for a state of one CDF block (k_sample_small): the same
    // chunk sums and chunk prefix sums, the same in-chunk running sums (a warp's shuffle scan, kept
    // here per element), the same uniforms and comparisons, so the same indices; one thread per shot.
    block_chunk_sums_p(sprob, nt, 0, s_ch, s_cl, &s_total, s_cinc);
    double* scan = reinterpret_cast<double*>(smem);   // the tile is no longer needed
    // per element: the largest value, as an integer key, of (chunk base + running sum) over the chunk
    // up to it, so that a binary search finds the first element whose own value reaches the target
    long long* fkey = reinterpret_cast<long long*>(scan + nc32);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int c = warp; c * kChunk < nt; c += nw) {
        const int i = c * kChunk + lane;
        double p = (i < nt) ? sprob[i] : 0.0;
        const double cb = c == 0 ? 0.0 : s_cinc[c - 1];   // 0.0 + cb is cb: the sums are non-negative
        if (__ballot_sync(0xffffffffu, p != 0.0) == 0u) {
            // a chunk of zeros: every running sum is 0, every compared value the chunk base
            scan[i] = 0.0;
            fkey[i] = __double_as_longlong(cb);
            continue;
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double v = __shfl_up_sync(0xffffffffu, p, o);
            if (lane >= o) p += v;
        }
        scan[i] = p;
        long long key = __double_as_longlong(cb + p);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long v = __shfl_up_sync(0xffffffffu, key, o);
            if (lane >= o) key = max(key, v);
        }
        fkey[i] = key;
    }
    for (int c = threadIdx.x; c < kCpb; c += blockDim.x) s_ckey[c] = __double_as_longlong(0.0 + s_cinc[c]);
    __syncthreads();
    // Every value compared below is a sum of probabilities, so non-negative: its order is the order of
    // its bit pattern as an integer, which keeps the comparisons off the FP64 pipe (2 per clock per SM).
    const double total = 0.0 + s_total;
    // u * total with u = (r >> 11) 2^-53: the scaling by 2^-53 is exact on either factor, so
    // (r >> 11) * (total 2^-53) rounds the same real product once, as the samplers' u * total does
    const double tscale = total * 0x1.0p-53;
    for (int64_t sh = threadIdx.x; sh < shots; sh += blockDim.x) {
        const uint64_t r = splitmix64(seed ^ splitmix64((uint64_t)sh));
        const double t = (double)(r >> 11) * tscale;
        const long long tb = __double_as_longlong(t);
        int clo = 0, chi = kCpb - 1;
        while (clo < chi) {
            const int mid = (clo + chi) >> 1;
            if (s_ckey[mid] >= tb) chi = mid; else clo = mid + 1;
        }
        const int c0 = clo * kChunk;
        int lo = 0, hi = kChunk;   // first element of the chunk whose value reaches the target
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (fkey[c0 + mid] >= tb) hi = mid; else lo = mid + 1;
        }
        int64_t out = nt - 1;
        bool found = lo < kChunk && c0 + lo < nt;
        if (found) out = c0 + lo;
        if (!found && c0 < nt) {
            // the chunk's own running sum fell short of its prefix sum by rounding: go on as the
            // one-block sampler does, with the running sum carried from chunk to chunk
            double cw = (0.0 + (clo == 0 ? 0.0 : s_cinc[clo - 1])) + scan[c0 + kChunk - 1];
            for (int c = c0 + kChunk; c < nt && !found; c += kChunk) {
                for (int l = 0; l < kChunk; l++) {
                    const int i = c + l;
                    if (i < nt && cw + scan[i] >= t) { out = i; found = true; break; }
                }
                cw += scan[c + kChunk - 1];
            }
        }
        samples[sh] = out;
    }
    small_run_done(done, ticket, times);
}

}  // namespace

int bs_small_pack(const bs_sim* s, const std::vector<Sweep>& sweeps, SmallPlan& out) {
    const int n = s->n;
    if (s->kind != BS_KIND_SV || s->precision != BS_PREC_C128 || n > 12) return BS_ERR_UNSUPPORTED;
    std::vector<TileGate>& tg = out.tg;
    std::vector<float4>& mats = out.mats;
    std::vector<int32_t>& perms = out.perms;
    tg.clear();
    mats.clear();
    perms.clear();
    int kmax = 1;
    std::vector<HostGate> merged;
    for (const Sweep& sw : sweeps) {
        merge_diagonals(sw.gates, merged);
        for (const HostGate& hg : merged) {
            if (hg.kind != 0 && hg.kind != 1 && hg.kind != 2) return BS_ERR_UNSUPPORTED;
            if (hg.kind != 1 && hg.k > BS_TILE_MAXK) return BS_ERR_UNSUPPORTED;
            TileGate t{};
            t.kind = hg.kind;
            t.k = hg.k;
            t.lc_mask = (uint32_t)hg.cmask;   // every bit is in the tile, at its own position
            t.lc_val = (uint32_t)hg.cval;
            for (int q = 0; q < hg.k; q++) {
                t.gbit[q] = hg.ebit[q];
                if (q < BS_TILE_MAXK) t.tbit[q] = hg.ebit[q];
            }
            t.mat_off = (int32_t)mats.size();
            t.perm_off = (int32_t)perms.size();
            if (hg.kind == 0) {
                for (int i = 0; i < (1 << (2 * hg.k)); i++) mats.push_back(to_cff(hg.mat[2 * i], hg.mat[2 * i + 1]));
                kmax = std::max(kmax, hg.k);
            } else if (hg.kind == 1) {
                for (int i = 0; i < (1 << hg.k); i++) mats.push_back(to_cff(hg.mat[2 * i], hg.mat[2 * i + 1]));
            } else {
                perms.insert(perms.end(), hg.perm.begin(), hg.perm.end());
                kmax = std::max(kmax, hg.k);
            }
            tg.push_back(t);
        }
    }
    out.kmax = kmax;
    return BS_OK;
}

int bs_small_launch(bs_sim* s, const SmallPlan& plan, double* dprobs, int64_t shots, uint64_t seed,
                    int64_t* dsamples, int64_t* done, int64_t ticket, const SmallIO* io) {
    const int n = s->n;
    const std::vector<TileGate>& tg = plan.tg;
    const std::vector<float4>& mats = plan.mats;
    const std::vector<int32_t>& perms = plan.perms;
    const int kmax = plan.kmax;
    auto al = [](int64_t x) { return (x + 255) & ~(int64_t)255; };
    const int64_t b_tg = al((int64_t)(tg.size() + 1) * (int64_t)sizeof(TileGate));
    const int64_t b_m = al((int64_t)(mats.size() + 1) * (int64_t)sizeof(float4));
    const int64_t b_p = al((int64_t)(perms.size() + 1) * (int64_t)sizeof(int32_t));
    const int64_t b_all = b_tg + b_m + b_p;
    char* dev;
    int rc;
    if (io && b_all <= (int64_t)io->plan_cap) {
        // the plan goes straight into host-mapped memory, which the kernel reads (the previous run on
        // this thread has completed, so nothing reads it any more); the launch orders these writes
        // before the kernel's reads
        char* host = io->hplan;
        if (!tg.empty()) std::memcpy(host, tg.data(), tg.size() * sizeof(TileGate));
        if (!mats.empty()) std::memcpy(host + b_tg, mats.data(), mats.size() * sizeof(float4));
        if (!perms.empty()) std::memcpy(host + b_tg + b_m, perms.data(), perms.size() * sizeof(int32_t));
        std::atomic_thread_fence(std::memory_order_release);
        dev = io->dplan;
    } else {
        rc = bs_ensure_plan(s, b_all);
        if (rc) return rc;
        char* host = bs_stage(s, (size_t)b_all);
        if (!host) return bs_fail(s, BS_ERR_ALLOC, "pinned staging allocation");
        if (!tg.empty()) std::memcpy(host, tg.data(), tg.size() * sizeof(TileGate));
        if (!mats.empty()) std::memcpy(host + b_tg, mats.data(), mats.size() * sizeof(float4));
        if (!perms.empty()) std::memcpy(host + b_tg + b_m, perms.data(), perms.size() * sizeof(int32_t));
        dev = (char*)s->plan_buf;
        rc = bs_cuda_check(s, cudaMemcpyAsync(dev, host, (size_t)b_all, cudaMemcpyHostToDevice, s->stream), "plan upload");
        bs_stage_done(s);
        if (rc) return rc;
    }
    // the tile (afterwards two arrays of the sampler, whole 32-element chunks), then the probabilities,
    // then (staged) the matrices and permutations
    const size_t base = std::max(((size_t)1 << n) * sizeof(float4), (size_t)2 * (((1 << n) + 31) / 32 * 32) * sizeof(double)) +
                        ((size_t)1 << n) * sizeof(double);
    const size_t stage = mats.size() * sizeof(float4) + perms.size() * sizeof(int32_t);
    constexpr size_t kSmemCap = 160 * 1024;
    const bool staged = base + stage <= kSmemCap;
    const size_t smem = staged ? base + stage : base;
    const TileGate* d_tg = (const TileGate*)dev;
    const float4* d_m = (const float4*)(dev + b_tg);
    const int32_t* d_p = (const int32_t*)(dev + b_tg + b_m);
    static bool attr_set[64] = {false};
    if (!attr_set[s->device & 63]) {
        cudaFuncSetAttribute(k_small_run<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap);
        cudaFuncSetAttribute(k_small_run<4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap);
        cudaFuncSetAttribute(k_small_run<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap);
        cudaFuncSetAttribute(k_small_run<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemCap);
        attr_set[s->device & 63] = true;
    }
    const int threads = std::min(512, std::max(128, (1 << n) / 2));
    auto kern = kmax <= 2 ? (staged ? k_small_run<2, true> : k_small_run<2, false>)
                          : (staged ? k_small_run<4, true> : k_small_run<4, false>);
    kern<<<1, threads, smem, s->stream>>>((double2*)s->state, n, d_tg, (int)tg.size(), d_m, (int)mats.size(), d_p,
                                          (int)perms.size(), dprobs, shots, seed, dsamples, done, ticket,
                                          io ? io->dtimes : nullptr);
    s->stats.kernel_launches++;
    s->stats.sweeps++;
    s->stats.gates += (int64_t)tg.size();
    s->stats.bytes_moved += 16.0 * (double)((int64_t)1 << n);
    return bs_cuda_check(s, cudaGetLastError(), "small run");
}
