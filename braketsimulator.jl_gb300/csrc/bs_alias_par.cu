// Parallel alias-table construction (BS_ALIAS_PARALLEL).
//
// The reference builds its table serially (make_alias_table!, src/result_types.jl:8-54): light
// and heavy items on two stacks, popped in pairs.  That order is what BS_ALIAS_EXACT keeps, on one
// GPU thread, for bit-exact draws.  This builder gives a table for the same distribution in
// O(n) parallel work, following the sweeping construction of Hübschle-Schneider & Sanders
// ("Parallel weighted random sampling", ACM TOMS 2022): heavy items, in index order, fill the
// buckets of the light items, in index order; a heavy item serves lights while it still has
// weight above 1, and once it drops to 1 or below its own bucket is topped up by the next heavy.
//
// With normalised weights w_i = p_i n / W (mean 1), light deficits d_i = 1 - w_i and heavy
// surpluses s_j = w_j - 1, and exclusive prefix sums D(i) over the lights and S(j) over the
// heavies, the sweep is closed-form:
//   light i is served by the heavy j with S(j) <= D(i) < S(j+1):  ap = w_i, alias = heavy j;
//   heavy j ends with deficit e_j = D(i_end) - S(j+1), i_end = first light with D >= S(j+1):
//   e_j > 0: ap = 1 - e_j, alias = heavy j+1;  otherwise ap = 1 (its bucket is its own).
// (Summing the sweep's per-heavy balance 1 + s_j - served lights - e_(j-1) = 1 - e_j telescopes
// to that e_j; every e_j < 1 because one light's deficit is at most 1.)
//
// The sums are exact: weights are fixed point with 64 fraction bits in unsigned 128-bit integers,
// so the prefix sums, the searches and e_j carry no rounding; the table represents the fixed-point
// weights exactly, i.e. the distribution to within the quantisation of each weight (2^-65 of the
// mean weight) and the FP64 rounding of ap.  Weight that rounding leaves unbalanced at the very end
// (at most n 2^-65 of the mean) stays with the last bucket.
#include <algorithm>
#include "bs_internal.h"

namespace {

typedef unsigned __int128 u128;
constexpr int kT = 256;          // threads per block
constexpr int kPer = 8;          // items per thread
constexpr int kItems = kT * kPer;
const u128 kOne = (u128)1 << 64; // weight 1 in fixed point

// round(w * 2^64) for w >= 0 (w below 2^-64 rounds to 0 or 1 unit)
__device__ __forceinline__ u128 to_fixed(double w) {
    if (!(w > 0.0)) return 0;
    int e;
    const double f = frexp(w, &e);                      // w = f 2^e, f in [0.5, 1)
    const uint64_t m = (uint64_t)ldexp(f, 53);           // exact 53-bit integer
    const int sh = e - 53 + 64;                          // w 2^64 = m 2^sh
    if (sh >= 0) return (u128)m << sh;
    if (sh <= -64) return 0;
    return (u128)((m >> (-sh)) + ((m >> (-sh - 1)) & 1ULL));
}

__device__ __forceinline__ u128 shfl_up128(u128 v, int o) {
    const uint64_t lo = __shfl_up_sync(0xffffffffu, (uint64_t)v, o);
    const uint64_t hi = __shfl_up_sync(0xffffffffu, (uint64_t)(v >> 64), o);
    return ((u128)hi << 64) | lo;
}

struct Tot {          // per-block totals: light count, heavy count, light deficits, heavy surpluses
    int64_t nl, nh;
    u128 d, s;
};

// class of item i: 1 light (w < 1), 2 heavy (w > 1), 0 exactly 1; its deficit or surplus
__device__ __forceinline__ int classify(const double* p, int64_t n, double ac, int64_t i, u128& amount) {
    // ac = n / W: the weights normalised to mean 1
    if (i >= n) { amount = 0; return 3; }
    const u128 q = to_fixed(p[i] * ac);
    if (q < kOne) { amount = kOne - q; return 1; }
    if (q > kOne) { amount = q - kOne; return 2; }
    amount = 0;
    return 0;
}

__global__ void __launch_bounds__(kT) k_alias_count(const double* __restrict__ p, int64_t n, const double* __restrict__ acp,
                                                    Tot* __restrict__ tot) {
    __shared__ Tot red[kT / 32];
    const double ac = *acp;
    const int64_t b0 = (int64_t)blockIdx.x * kItems;
    Tot t{0, 0, 0, 0};
    for (int k = 0; k < kPer; k++) {
        u128 a;
        const int c = classify(p, n, ac, b0 + (int64_t)k * kT + threadIdx.x, a);
        if (c == 1) { t.nl++; t.d += a; }
        else if (c == 2) { t.nh++; t.s += a; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        t.nl += __shfl_down_sync(0xffffffffu, t.nl, o);
        t.nh += __shfl_down_sync(0xffffffffu, t.nh, o);
        const uint64_t dl = __shfl_down_sync(0xffffffffu, (uint64_t)t.d, o), dh = __shfl_down_sync(0xffffffffu, (uint64_t)(t.d >> 64), o);
        const uint64_t sl = __shfl_down_sync(0xffffffffu, (uint64_t)t.s, o), shh = __shfl_down_sync(0xffffffffu, (uint64_t)(t.s >> 64), o);
        t.d += ((u128)dh << 64) | dl;
        t.s += ((u128)shh << 64) | sl;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        Tot a{0, 0, 0, 0};
        for (int w = 0; w < kT / 32; w++) { a.nl += red[w].nl; a.nh += red[w].nh; a.d += red[w].d; a.s += red[w].s; }
        tot[blockIdx.x] = a;
    }
}

// Exact weight total: per block the sum of the probabilities in 64-fraction-bit fixed point
// (tot[b].d), then one CTA adds the blocks and rounds once: *ac = n / W with W correctly rounded, so
// that the normalised weights sum to n within their own FP64 roundings.
__global__ void __launch_bounds__(kT) k_alias_wsum(const double* __restrict__ p, int64_t n, Tot* __restrict__ tot) {
    __shared__ u128 red[kT / 32];
    const int64_t b0 = (int64_t)blockIdx.x * kItems;
    u128 t = 0;
    for (int k = 0; k < kPer; k++) {
        const int64_t i = b0 + (int64_t)k * kT + threadIdx.x;
        if (i < n) t += to_fixed(p[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t lo = __shfl_down_sync(0xffffffffu, (uint64_t)t, o), hi = __shfl_down_sync(0xffffffffu, (uint64_t)(t >> 64), o);
        t += ((u128)hi << 64) | lo;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        u128 a = 0;
        for (int w = 0; w < kT / 32; w++) a += red[w];
        tot[blockIdx.x].d = a;
    }
}
__global__ void __launch_bounds__(512) k_alias_wsum_final(const Tot* __restrict__ tot, int64_t nb, int64_t n,
                                                          double* __restrict__ ac) {
    __shared__ u128 part[512];
    u128 t = 0;
    for (int64_t b = threadIdx.x; b < nb; b += blockDim.x) t += tot[b].d;
    part[threadIdx.x] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        u128 a = 0;
        for (int w = 0; w < (int)blockDim.x; w++) a += part[w];
        // W = a 2^-64: its top 64 bits converted once (the bits below them only decide exact ties)
        int sh = 0;
        while ((a >> sh) >> 64) sh++;
        const double W = ldexp((double)(uint64_t)(a >> sh), sh - 64);
        *ac = (W > 0.0) ? (double)n / W : 0.0;
    }
}

__global__ void k_alias_set_scale(double* ac, double v) { *ac = v; }

// exclusive scan of the block totals in place (one CTA; a serial run per thread, then a scan of the
// run totals); tot[nb] receives the grand totals
__global__ void __launch_bounds__(512) k_alias_scan_blocks(Tot* __restrict__ tot, int64_t nb) {
    __shared__ Tot part[512];
    const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const int64_t b0 = threadIdx.x * per, b1 = std::min<int64_t>(nb, b0 + per);
    Tot s{0, 0, 0, 0};
    for (int64_t b = b0; b < b1; b++) { s.nl += tot[b].nl; s.nh += tot[b].nh; s.d += tot[b].d; s.s += tot[b].s; }
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        Tot run{0, 0, 0, 0};
        for (int w = 0; w < (int)blockDim.x; w++) {
            const Tot v = part[w];
            part[w] = run;
            run.nl += v.nl; run.nh += v.nh; run.d += v.d; run.s += v.s;
        }
        tot[nb] = run;
    }
    __syncthreads();
    Tot run = part[threadIdx.x];
    for (int64_t b = b0; b < b1; b++) {
        const Tot v = tot[b];
        tot[b] = run;
        run.nl += v.nl; run.nh += v.nh; run.d += v.d; run.s += v.s;
    }
}

// Block-local exclusive scans, then the lights' (index, D) at [0, NL) and the heavies' (index, S)
// at [NL, NL + NH) of idx / pref.  Items of weight exactly 1 get their final entry here.
__global__ void __launch_bounds__(kT) k_alias_scatter(const double* __restrict__ p, int64_t n, const double* __restrict__ acp,
                                                      const Tot* __restrict__ tot, int64_t nb, int64_t* __restrict__ idx,
                                                      u128* __restrict__ pref, double* __restrict__ ap,
                                                      int64_t* __restrict__ alias) {
    __shared__ Tot wsum[kT / 32];
    const double ac = *acp;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const Tot base = tot[blockIdx.x];
    const int64_t NL = tot[nb].nl;
    // each thread takes kPer consecutive items so that the block order is the index order
    const int64_t i0 = (int64_t)blockIdx.x * kItems + (int64_t)threadIdx.x * kPer;
    int cls[kPer];
    u128 amt[kPer];
    Tot mine{0, 0, 0, 0};
    for (int k = 0; k < kPer; k++) {
        cls[k] = classify(p, n, ac, i0 + k, amt[k]);
        if (cls[k] == 1) { mine.nl++; mine.d += amt[k]; }
        else if (cls[k] == 2) { mine.nh++; mine.s += amt[k]; }
    }
    // inclusive warp scan of the thread totals
    Tot inc = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t a = __shfl_up_sync(0xffffffffu, inc.nl, o), b = __shfl_up_sync(0xffffffffu, inc.nh, o);
        const u128 c = shfl_up128(inc.d, o), d = shfl_up128(inc.s, o);
        if (lane >= o) { inc.nl += a; inc.nh += b; inc.d += c; inc.s += d; }
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    Tot off = base;
    for (int w = 0; w < warp; w++) { off.nl += wsum[w].nl; off.nh += wsum[w].nh; off.d += wsum[w].d; off.s += wsum[w].s; }
    off.nl += inc.nl - mine.nl;
    off.nh += inc.nh - mine.nh;
    off.d += inc.d - mine.d;
    off.s += inc.s - mine.s;
    for (int k = 0; k < kPer; k++) {
        const int64_t i = i0 + k;
        if (cls[k] == 1) {
            idx[off.nl] = i;
            pref[off.nl] = off.d;
            off.nl++;
            off.d += amt[k];
        } else if (cls[k] == 2) {
            idx[NL + off.nh] = i;
            pref[NL + off.nh] = off.s;
            off.nh++;
            off.s += amt[k];
        } else if (cls[k] == 0) {
            ap[i] = 1.0;
            alias[i] = -1;
        }
    }
}

// last position in [0, m) with a[pos] <= v (a ascending, a[0] = 0 <= v): the donor of a light
__device__ __forceinline__ int64_t last_le(const u128* a, int64_t m, u128 v) {
    int64_t lo = 0, hi = m - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (a[mid] <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}
// first position in [0, m) with a[pos] >= v, m if none
__device__ __forceinline__ int64_t first_ge(const u128* a, int64_t m, u128 v) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] >= v) hi = mid; else lo = mid + 1;
    }
    return lo;
}

__global__ void k_alias_pair(const double* __restrict__ p, const double* __restrict__ acp, const Tot* __restrict__ tot,
                             int64_t nb, const int64_t* __restrict__ idx, const u128* __restrict__ pref,
                             double* __restrict__ ap, int64_t* __restrict__ alias) {
    const double ac = *acp;
    const int64_t NL = tot[nb].nl, NH = tot[nb].nh;
    const u128 DT = tot[nb].d, ST = tot[nb].s;
    const u128* D = pref;
    const u128* S = pref + NL;
    const int64_t* hidx = idx + NL;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < NL + NH; t += stride) {
        if (t < NL) {
            // light: served by the heavy j with S(j) <= D(t) < S(j+1)
            const int64_t i = idx[t];
            const u128 q = to_fixed(p[i] * ac);
            ap[i] = (double)(uint64_t)q * 0x1.0p-64;
            if (NH > 0 && D[t] < ST) {
                alias[i] = hidx[last_le(S, NH, D[t])];
            } else {
                ap[i] = 1.0;        // no weight left to fill it: the rounding residue
                alias[i] = -1;
            }
        } else {
            const int64_t j = t - NL;
            const int64_t i = hidx[j];
            const u128 snext = (j + 1 < NH) ? S[j + 1] : ST;
            const int64_t iend = first_ge(D, NL, snext);
            const u128 dend = (iend < NL) ? D[iend] : DT;
            if (dend > snext && j + 1 < NH) {
                const u128 e = dend - snext;                   // < 2^64 (one light's deficit at most)
                const uint64_t e64 = (e >> 64) ? ~0ULL : (uint64_t)e;
                ap[i] = 1.0 - (double)e64 * 0x1.0p-64;
                alias[i] = hidx[j + 1];
            } else {
                ap[i] = 1.0;
                alias[i] = -1;
            }
        }
    }
}

}  // namespace

// Scratch needed by bs_alias_parallel for n items, beyond the probabilities.
int64_t bs_alias_parallel_scratch(int64_t n) {
    const int64_t nb = (n + kItems - 1) / kItems;
    return n * 16 + n * 8 + (nb + 1) * (int64_t)sizeof(Tot) + 256;
}

// ap/alias (device, n entries) from device probabilities dprobs.  wsum > 0: the weights' total as the
// caller gives it (the reference normalises by its own sum); otherwise the exact total, rounded once.
// work: bs_alias_parallel_scratch(n) bytes of device memory, 16-byte aligned, not overlapping dprobs.
int bs_alias_parallel(bs_sim* s, const double* dprobs, int64_t n, double wsum, double* ap, int64_t* alias, void* work) {
    const int64_t nb = (n + kItems - 1) / kItems;
    if (nb > ((int64_t)1 << 31) - 2) return bs_fail(s, BS_ERR_UNSUPPORTED, "alias table too large");
    char* w = static_cast<char*>(work);
    u128* pref = reinterpret_cast<u128*>(w);
    int64_t* idx = reinterpret_cast<int64_t*>(w + n * 16);
    const int64_t toff = (n * 24 + 15) & ~(int64_t)15;
    Tot* tot = reinterpret_cast<Tot*>(w + toff);
    double* acp = reinterpret_cast<double*>(w + toff + (nb + 1) * (int64_t)sizeof(Tot));
    if (wsum > 0.0) {
        k_alias_set_scale<<<1, 1, 0, s->stream>>>(acp, (double)n / wsum);
    } else {
        k_alias_wsum<<<(unsigned)nb, kT, 0, s->stream>>>(dprobs, n, tot);
        k_alias_wsum_final<<<1, 512, 0, s->stream>>>(tot, nb, n, acp);
    }
    k_alias_count<<<(unsigned)nb, kT, 0, s->stream>>>(dprobs, n, acp, tot);
    k_alias_scan_blocks<<<1, 512, 0, s->stream>>>(tot, nb);
    k_alias_scatter<<<(unsigned)nb, kT, 0, s->stream>>>(dprobs, n, acp, tot, nb, idx, pref, ap, alias);
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    k_alias_pair<<<(unsigned)g, 256, 0, s->stream>>>(dprobs, acp, tot, nb, idx, pref, ap, alias);
    return bs_cuda_check(s, cudaGetLastError(), "parallel alias build");
}
