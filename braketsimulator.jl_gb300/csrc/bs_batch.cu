// Batched simulation of many independent circuits of uneven size.
//
// Reference: the batch simulate(sim, ::Vector, shots; max_parallel)
// (src/BraketSimulator.jl:347-395) runs up to 32 Julia tasks, each a full
// simulate on its own simulator copy.  Here:
//  - circuits with at most BS_BATCH_SMALL_QUBITS qubits run whole inside one CTA:
//    one persistent launch whose CTAs pull circuit indices from an atomic queue
//    (largest first); the complex64 state, every gate, the Pauli expectations and
//    the shots (inverse CDF over a float-float prefix sum) stay in shared memory;
//  - larger circuits run as ordinary tile sweeps on a pool of handles, one CUDA
//    stream each, driven by host worker threads so their kernels overlap.
// Arithmetic of the small path: complex64 state, FP32 gate math, FP64-accurate
// (float-float) expectations and CDF.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>
#include "bs_internal.h"
#include "bs_ff.cuh"

#define BS_BATCH_SMALL_QUBITS 12

namespace {

struct BGate {            // one gate of a small circuit (canonical endian bits)
    int32_t type;         // 0: 2x2 matrix on t0 with controls; 1: swap t0 <-> t1 with controls
    int32_t t0, t1;
    uint32_t cmask, cval;
    float2 m[4];
};

struct BCirc {            // one small circuit
    int32_t n;
    int32_t g0, ng;       // gate range
    int32_t out;          // output slot (circuit index)
};

constexpr int kBT = 256;

__global__ void __launch_bounds__(kBT) k_batch_small(const BCirc* __restrict__ circs, int nc, const BGate* __restrict__ gates,
                                                      int n_terms, const uint64_t* __restrict__ xme,
                                                      const uint64_t* __restrict__ zme, const int* __restrict__ phs,
                                                      int64_t shots, uint64_t seed, double* __restrict__ exp_out,
                                                      int64_t* __restrict__ samp_out, int* __restrict__ queue) {
    extern __shared__ double sm_d[];
    double* cdf = sm_d;                                           // 2^12 doubles
    float2* st = reinterpret_cast<float2*>(sm_d + (1 << BS_BATCH_SMALL_QUBITS));   // 2^12 float2
    __shared__ int s_ci;
    __shared__ double red[kBT / 32];
    __shared__ double s_part[kBT];
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_ci = atomicAdd(queue, 1);
        __syncthreads();
        const int ci = s_ci;
        if (ci >= nc) return;
        const BCirc c = circs[ci];
        const int dim = 1 << c.n;
        for (int i = threadIdx.x; i < dim; i += blockDim.x) st[i] = make_float2(i == 0 ? 1.f : 0.f, 0.f);
        __syncthreads();
        for (int gi = c.g0; gi < c.g0 + c.ng; gi++) {
            const BGate g = gates[gi];
            if (g.type == 0) {
                for (int p = threadIdx.x; p < dim / 2; p += blockDim.x) {
                    const int lo = ((p >> g.t0) << (g.t0 + 1)) | (p & ((1 << g.t0) - 1));
                    if (((uint32_t)lo & g.cmask) != g.cval) continue;
                    const int hi = lo | (1 << g.t0);
                    const float2 a = st[lo], b = st[hi];
                    st[lo] = make_float2(g.m[0].x * a.x - g.m[0].y * a.y + g.m[1].x * b.x - g.m[1].y * b.y,
                                         g.m[0].x * a.y + g.m[0].y * a.x + g.m[1].x * b.y + g.m[1].y * b.x);
                    st[hi] = make_float2(g.m[2].x * a.x - g.m[2].y * a.y + g.m[3].x * b.x - g.m[3].y * b.y,
                                         g.m[2].x * a.y + g.m[2].y * a.x + g.m[3].x * b.y + g.m[3].y * b.x);
                }
            } else {
                for (int i = threadIdx.x; i < dim; i += blockDim.x) {
                    const int b0 = (i >> g.t0) & 1, b1 = (i >> g.t1) & 1;
                    if (b0 == 1 || b1 == 0) continue;              // visit each swapped pair once
                    if (((uint32_t)i & g.cmask) != g.cval) continue;
                    const int j = i ^ (1 << g.t0) ^ (1 << g.t1);
                    const float2 v = st[i];
                    st[i] = st[j];
                    st[j] = v;
                }
            }
            __syncthreads();
        }
        // Pauli expectations, FP64-accurate sums over the complex64 values
        for (int t = 0; t < n_terms; t++) {
            const uint64_t xm = xme[(int64_t)c.out * n_terms + t], zm = zme[(int64_t)c.out * n_terms + t];
            const int ph = phs[(int64_t)c.out * n_terms + t];
            ffsum acc{0.f, 0.f};
            for (int i = threadIdx.x; i < dim; i += blockDim.x) {
                const float2 a = st[i], b = st[i ^ (int)xm];
                ffacc r, m;
                acc_first(r, a.x, 0.f, b.x, 0.f);
                acc_add(r, a.y, 0.f, b.y, 0.f);
                acc_first(m, a.x, 0.f, b.y, 0.f);
                acc_add(m, -a.y, 0.f, b.x, 0.f);
                const ff rr = acc_done(r), mm = acc_done(m);
                float vh, vl;
                switch (ph) {
                    case 0: vh = rr.h; vl = rr.l; break;
                    case 1: vh = mm.h; vl = mm.l; break;
                    case 2: vh = -rr.h; vl = -rr.l; break;
                    default: vh = -mm.h; vl = -mm.l; break;
                }
                if (__popcll((unsigned long long)i & zm) & 1) { vh = -vh; vl = -vl; }
                fsum_add(acc, vh, vl);
            }
            double v = ff2d(acc.h, acc.l);
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                double s = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
                exp_out[(int64_t)c.out * n_terms + t] = s;
            }
            __syncthreads();
        }
        if (shots <= 0) continue;
        // CDF: each thread a contiguous chunk, then an exclusive scan of the chunk sums
        const int per = (dim + blockDim.x - 1) / blockDim.x;
        const int i0 = threadIdx.x * per, i1 = min(dim, i0 + per);
        ffsum run{0.f, 0.f};
        for (int i = i0; i < i1; i++) {
            const float2 a = st[i];
            ffacc r;
            acc_first(r, a.x, 0.f, a.x, 0.f);
            acc_add(r, a.y, 0.f, a.y, 0.f);
            const ff p = acc_done(r);
            fsum_add(run, p.h, p.l);
            cdf[i] = ff2d(run.h, run.l);
        }
        s_part[threadIdx.x] = ff2d(run.h, run.l);
        __syncthreads();
        if (threadIdx.x == 0) {
            double acc = 0.0;
            for (int w = 0; w < (int)blockDim.x; w++) { const double v = s_part[w]; s_part[w] = acc; acc += v; }
        }
        __syncthreads();
        const double off = s_part[threadIdx.x];
        for (int i = i0; i < i1; i++) cdf[i] += off;
        __syncthreads();
        const double total = cdf[dim - 1];
        for (int64_t s = threadIdx.x; s < shots; s += blockDim.x) {
            uint64_t x = seed ^ ((uint64_t)c.out * 0x9E3779B97F4A7C15ULL) ^ ((uint64_t)s * 0xD1B54A32D192ED03ULL);
            x += 0x9e3779b97f4a7c15ULL;
            x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
            x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
            x ^= x >> 31;
            const double tt = (double)(x >> 11) * 0x1.0p-53 * total;
            int lo = 0, hi = dim - 1;
            while (lo < hi) { const int mid = (lo + hi) >> 1; if (cdf[mid] >= tt) hi = mid; else lo = mid + 1; }
            samp_out[(int64_t)c.out * shots + s] = lo;
        }
    }
}

}  // namespace

extern "C" int bs_run_batch(int n_circuits, const int* n_qubits, const bs_op* const* ops, const int64_t* n_ops,
                            int n_terms, const uint64_t* xmask, const uint64_t* zmask, int64_t shots, uint64_t seed,
                            int precision, double* expectations_out, int64_t* samples_out, bs_stats* stats_out) {
    if (n_circuits < 0 || (n_circuits > 0 && (!n_qubits || !ops || !n_ops)) || n_terms < 0 || n_terms > 64 || shots < 0)
        return BS_ERR_INVALID_ARG;
    if ((n_terms > 0 && (!xmask || !zmask || !expectations_out)) || (shots > 0 && !samples_out)) return BS_ERR_INVALID_ARG;
    if (precision != BS_PREC_C64 && precision != BS_PREC_C128) return BS_ERR_INVALID_ARG;
    for (int c = 0; c < n_circuits; c++)
        if (n_qubits[c] < 1 || n_qubits[c] > 30) return BS_ERR_INVALID_ARG;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // ---- split by size; small circuits only in the complex64 batch kernel
    std::vector<int> small, large;
    for (int c = 0; c < n_circuits; c++) {
        bool ok_small = precision == BS_PREC_C64 && n_qubits[c] <= BS_BATCH_SMALL_QUBITS;
        // the small kernel takes 1-target gates (any controls) and swaps
        for (int64_t i = 0; ok_small && i < n_ops[c]; i++) {
            const bs_op& o = ops[c][i];
            if (o.kind == 2) continue;
            if (o.kind != 0 || o.n_targets > 2) ok_small = false;
            else if (o.n_targets == 2 && !(o.flags & BS_GATE_DIAGONAL)) {
                // only the SWAP permutation qualifies
                const double* m = o.matrix;
                const double sw[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0};
                for (int e = 0; e < 32; e++) if (m[e] != sw[e]) { ok_small = false; break; }
            } else if (o.n_targets == 2) ok_small = false;
        }
        (ok_small ? small : large).push_back(c);
    }
    // endian Pauli masks per circuit
    std::vector<uint64_t> xme((size_t)n_circuits * n_terms), zme((size_t)n_circuits * n_terms);
    std::vector<int> phs((size_t)n_circuits * n_terms);
    for (int c = 0; c < n_circuits; c++)
        for (int t = 0; t < n_terms; t++) {
            const size_t k = (size_t)c * n_terms + t;
            uint64_t x = 0, z = 0;
            for (int q = 0; q < n_qubits[c]; q++) {
                if ((xmask[k] >> q) & 1ULL) x |= 1ULL << (n_qubits[c] - 1 - q);
                if ((zmask[k] >> q) & 1ULL) z |= 1ULL << (n_qubits[c] - 1 - q);
            }
            xme[k] = x;
            zme[k] = z;
            phs[k] = __builtin_popcountll(xmask[k] & zmask[k]) & 3;
            if ((xmask[k] | zmask[k]) >> n_qubits[c]) return BS_ERR_INVALID_ARG;
        }
    int rc = BS_OK;
    bs_stats tot{};
    cudaStream_t sstream = nullptr;
    cudaStreamCreateWithFlags(&sstream, cudaStreamNonBlocking);
    cudaEventRecord(e0, sstream);
    void* dbuf = nullptr;
    if (!small.empty()) {
        // lower small circuits with the ordinary gate lowering, then pack
        bs_sim tmp;
        tmp.kind = BS_KIND_SV;
        std::vector<BCirc> bc;
        std::vector<BGate> bg;
        std::sort(small.begin(), small.end(), [&](int a, int b) { return n_qubits[a] > n_qubits[b]; });
        for (int c : small) {
            tmp.n = n_qubits[c];
            BCirc cc{};
            cc.n = n_qubits[c];
            cc.g0 = (int32_t)bg.size();
            cc.out = c;
            std::vector<HostGate> hg;
            for (int64_t i = 0; i < n_ops[c]; i++) {
                const bs_op& o = ops[c][i];
                if (o.kind == 2) continue;
                rc = bs_lower_gate(&tmp, o.matrix, o.n_targets, o.targets, o.n_controls, o.controls, o.control_values,
                                   o.flags, false, hg);
                if (rc) break;
            }
            if (rc) break;
            for (const HostGate& h : hg) {
                BGate g{};
                g.cmask = (uint32_t)h.cmask;
                g.cval = (uint32_t)h.cval;
                if (h.k == 2) {               // swap
                    g.type = 1;
                    g.t0 = h.ebit[0];
                    g.t1 = h.ebit[1];
                } else {
                    g.type = 0;
                    g.t0 = h.ebit[0];
                    double m[8] = {0};
                    if (h.kind == 0) { for (int e = 0; e < 8; e++) m[e] = h.mat[(size_t)e]; }
                    else if (h.kind == 1) { m[0] = h.mat[0]; m[1] = h.mat[1]; m[6] = h.mat[2]; m[7] = h.mat[3]; }
                    else {
                        for (int col = 0; col < 2; col++) {
                            const int row = h.perm[2 * col], p = h.perm[2 * col + 1] & 3;
                            m[2 * (row * 2 + col)] = (p == 0) ? 1 : (p == 2 ? -1 : 0);
                            m[2 * (row * 2 + col) + 1] = (p == 1) ? 1 : (p == 3 ? -1 : 0);
                        }
                    }
                    for (int e = 0; e < 4; e++) g.m[e] = make_float2((float)m[2 * e], (float)m[2 * e + 1]);
                }
                bg.push_back(g);
            }
            cc.ng = (int32_t)bg.size() - cc.g0;
            bc.push_back(cc);
        }
        if (!rc) {
            const size_t b_c = bc.size() * sizeof(BCirc), b_g = (bg.size() + 1) * sizeof(BGate);
            const size_t b_t = xme.size() * 8 + 8, b_p = phs.size() * 4 + 4;
            const size_t b_e = (size_t)n_circuits * n_terms * 8 + 8, b_s = (size_t)n_circuits * shots * 8 + 8;
            auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
            const size_t total = al(b_c) + al(b_g) + 2 * al(b_t) + al(b_p) + al(b_e) + al(b_s) + 256;
            if (cudaMalloc(&dbuf, total) != cudaSuccess) rc = BS_ERR_ALLOC;
            if (!rc) {
                char* p = (char*)dbuf;
                BCirc* d_c = (BCirc*)p; p += al(b_c);
                BGate* d_g = (BGate*)p; p += al(b_g);
                uint64_t* d_x = (uint64_t*)p; p += al(b_t);
                uint64_t* d_z = (uint64_t*)p; p += al(b_t);
                int* d_ph = (int*)p; p += al(b_p);
                double* d_e = (double*)p; p += al(b_e);
                int64_t* d_s = (int64_t*)p; p += al(b_s);
                int* d_q = (int*)p;
                cudaMemcpyAsync(d_c, bc.data(), b_c, cudaMemcpyHostToDevice, sstream);
                if (!bg.empty()) cudaMemcpyAsync(d_g, bg.data(), bg.size() * sizeof(BGate), cudaMemcpyHostToDevice, sstream);
                if (!xme.empty()) {
                    cudaMemcpyAsync(d_x, xme.data(), xme.size() * 8, cudaMemcpyHostToDevice, sstream);
                    cudaMemcpyAsync(d_z, zme.data(), zme.size() * 8, cudaMemcpyHostToDevice, sstream);
                    cudaMemcpyAsync(d_ph, phs.data(), phs.size() * 4, cudaMemcpyHostToDevice, sstream);
                }
                cudaMemsetAsync(d_q, 0, 4, sstream);
                const size_t smem = (size_t)(1 << BS_BATCH_SMALL_QUBITS) * (8 + 8);
                cudaFuncSetAttribute(k_batch_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                const int grid = (int)std::min<size_t>(bc.size(), 152 * 3);
                k_batch_small<<<grid, kBT, smem, sstream>>>(d_c, (int)bc.size(), d_g, n_terms, d_x, d_z, d_ph, shots, seed,
                                                             d_e, d_s, d_q);
                tot.kernel_launches += 1;
                // copy back only the small circuits' rows
                for (const BCirc& cc : bc) {
                    if (n_terms)
                        cudaMemcpyAsync(expectations_out + (size_t)cc.out * n_terms, d_e + (size_t)cc.out * n_terms,
                                        (size_t)n_terms * 8, cudaMemcpyDeviceToHost, sstream);
                    if (shots)
                        cudaMemcpyAsync(samples_out + (size_t)cc.out * shots, d_s + (size_t)cc.out * shots,
                                        (size_t)shots * 8, cudaMemcpyDeviceToHost, sstream);
                }
            }
        }
    }
    // ---- large circuits: a pool of handles, one stream each, host worker threads
    std::atomic<int> next{0};
    std::atomic<int> err{0};
    std::sort(large.begin(), large.end(), [&](int a, int b) { return n_qubits[a] > n_qubits[b]; });
    const int workers = (int)std::min<size_t>(large.size(), 4);
    std::vector<bs_stats> wst((size_t)std::max(workers, 1));
    int dev = 0;
    cudaGetDevice(&dev);
    auto work = [&](int w) {
        cudaSetDevice(dev);
        bs_sim* h = nullptr;
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= (int)large.size() || err.load()) break;
            const int c = large[(size_t)i];
            int r = h ? bs_reinit(h, n_qubits[c]) : bs_create(BS_KIND_SV, n_qubits[c], precision, &h);
            if (!r) r = bs_evolve(h, ops[c], n_ops[c], 0);
            if (!r) {
                wst[(size_t)w].sweeps += h->stats.sweeps;
                wst[(size_t)w].kernel_launches += h->stats.kernel_launches;
                wst[(size_t)w].gates += h->stats.gates;
                wst[(size_t)w].bytes_moved += h->stats.bytes_moved;
                wst[(size_t)w].tc_gates += h->stats.tc_gates;
                wst[(size_t)w].tc_launches += h->stats.tc_launches;
                wst[(size_t)w].tc_ms += h->stats.tc_ms;
            }
            if (!r && n_terms)
                r = bs_expectation_pauli(h, n_terms, xmask + (size_t)c * n_terms, zmask + (size_t)c * n_terms, nullptr,
                                         expectations_out + (size_t)c * n_terms);
            if (!r && shots) r = bs_sample(h, seed ^ ((uint64_t)c * 0x9E3779B97F4A7C15ULL), shots, samples_out + (size_t)c * shots);
            if (r) { err.store(r); break; }
        }
        if (h) bs_destroy(h);
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < workers; w++) pool.emplace_back(work, w);
    for (auto& t : pool) t.join();
    cudaEventRecord(e1, sstream);
    cudaStreamSynchronize(sstream);
    if (dbuf) cudaFree(dbuf);
    cudaStreamDestroy(sstream);
    if (!rc) rc = err.load();
    for (const bs_stats& x : wst) {
        tot.sweeps += x.sweeps;
        tot.kernel_launches += x.kernel_launches;
        tot.gates += x.gates;
        tot.bytes_moved += x.bytes_moved;
        tot.tc_gates += x.tc_gates;
        tot.tc_launches += x.tc_launches;
        tot.tc_ms += x.tc_ms;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    tot.gpu_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats_out) *stats_out = tot;
    return rc;
}
