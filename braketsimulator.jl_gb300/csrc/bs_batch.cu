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
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
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

namespace {

// Whether circuit c runs whole inside one CTA of k_batch_small: complex64, at most
// BS_BATCH_SMALL_QUBITS qubits, 1-target gates (any controls) and swaps only.
bool small_ok(int precision, int nq, const bs_op* ops, int64_t n_ops) {
    if (precision != BS_PREC_C64 || nq > BS_BATCH_SMALL_QUBITS) return false;
    for (int64_t i = 0; i < n_ops; i++) {
        const bs_op& o = ops[i];
        if (o.kind == 2) continue;
        if (o.kind != 0 || o.n_targets > 2) return false;
        if (o.n_targets == 2) {
            if (o.flags & BS_GATE_DIAGONAL) return false;
            // only the SWAP permutation qualifies
            const double* m = o.matrix;
            const double sw[32] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0};
            for (int e = 0; e < 32; e++) if (m[e] != sw[e]) return false;
        }
    }
    return true;
}

// Lower the small circuits (largest first) into the packed BCirc/BGate form of k_batch_small.
int pack_small(std::vector<int> small, const int* n_qubits, const bs_op* const* ops, const int64_t* n_ops,
               std::vector<BCirc>& bc, std::vector<BGate>& bg) {
    bs_sim tmp;
    tmp.kind = BS_KIND_SV;
    bc.clear();
    bg.clear();
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
            int rc = bs_lower_gate(&tmp, o.matrix, o.n_targets, o.targets, o.n_controls, o.controls, o.control_values,
                                   o.flags, false, hg);
            if (rc) return rc;
        }
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
    return BS_OK;
}

// Endian Pauli masks (bit n-1-q) and Y-phase counts per (circuit, term); false on a mask outside the register.
bool endian_terms(int n_circuits, const int* n_qubits, int n_terms, const uint64_t* xmask, const uint64_t* zmask,
                  std::vector<uint64_t>& xme, std::vector<uint64_t>& zme, std::vector<int>& phs) {
    xme.assign((size_t)n_circuits * n_terms, 0);
    zme.assign((size_t)n_circuits * n_terms, 0);
    phs.assign((size_t)n_circuits * n_terms, 0);
    for (int c = 0; c < n_circuits; c++)
        for (int t = 0; t < n_terms; t++) {
            const size_t k = (size_t)c * n_terms + t;
            if ((xmask[k] | zmask[k]) >> n_qubits[c]) return false;
            uint64_t x = 0, z = 0;
            for (int q = 0; q < n_qubits[c]; q++) {
                if ((xmask[k] >> q) & 1ULL) x |= 1ULL << (n_qubits[c] - 1 - q);
                if ((zmask[k] >> q) & 1ULL) z |= 1ULL << (n_qubits[c] - 1 - q);
            }
            xme[k] = x;
            zme[k] = z;
            phs[k] = __builtin_popcountll(xmask[k] & zmask[k]) & 3;
        }
    return true;
}

// Device layout of the small-circuit batch: circuits | gates | x masks | z masks | phases |
// expectations | samples | queue counter.
struct SmallLayout {
    size_t o_c = 0, o_g = 0, o_x = 0, o_z = 0, o_ph = 0, o_e = 0, o_s = 0, o_q = 0, total = 0;
    size_t b_c = 0, b_g = 0, b_t = 0, b_p = 0;
};
SmallLayout small_layout(size_t n_bc, size_t n_bg, int n_circuits, int n_terms, int64_t shots) {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    SmallLayout L;
    L.b_c = n_bc * sizeof(BCirc);
    L.b_g = (n_bg + 1) * sizeof(BGate);
    L.b_t = (size_t)n_circuits * n_terms * 8 + 8;
    L.b_p = (size_t)n_circuits * n_terms * 4 + 4;
    const size_t b_e = (size_t)n_circuits * n_terms * 8 + 8, b_s = (size_t)n_circuits * shots * 8 + 8;
    L.o_c = 0;
    L.o_g = L.o_c + al(L.b_c);
    L.o_x = L.o_g + al(L.b_g);
    L.o_z = L.o_x + al(L.b_t);
    L.o_ph = L.o_z + al(L.b_t);
    L.o_e = L.o_ph + al(L.b_p);
    L.o_s = L.o_e + al(b_e);
    L.o_q = L.o_s + al(b_s);
    L.total = L.o_q + 256;
    return L;
}

// Queue the small-circuit batch on stream st: uploads from the host image `img` (small-layout bytes
// up to o_e), the persistent kernel, and the copies of the small circuits' result rows into
// exp_out / samp_out.
void enqueue_small(cudaStream_t st, char* dbuf, const SmallLayout& L, const char* img, const std::vector<BCirc>& bc,
                   int n_terms, int64_t shots, uint64_t seed, double* exp_out, int64_t* samp_out) {
    cudaMemcpyAsync(dbuf, img, L.o_e, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(dbuf + L.o_q, 0, 4, st);
    const size_t smem = (size_t)(1 << BS_BATCH_SMALL_QUBITS) * (8 + 8);
    cudaFuncSetAttribute(k_batch_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int grid = (int)std::min<size_t>(bc.size(), 152 * 3);
    double* d_e = (double*)(dbuf + L.o_e);
    int64_t* d_s = (int64_t*)(dbuf + L.o_s);
    k_batch_small<<<grid, kBT, smem, st>>>((const BCirc*)(dbuf + L.o_c), (int)bc.size(), (const BGate*)(dbuf + L.o_g),
                                           n_terms, (const uint64_t*)(dbuf + L.o_x), (const uint64_t*)(dbuf + L.o_z),
                                           (const int*)(dbuf + L.o_ph), shots, seed, d_e, d_s, (int*)(dbuf + L.o_q));
    for (const BCirc& cc : bc) {
        if (n_terms)
            cudaMemcpyAsync(exp_out + (size_t)cc.out * n_terms, d_e + (size_t)cc.out * n_terms, (size_t)n_terms * 8,
                            cudaMemcpyDeviceToHost, st);
        if (shots)
            cudaMemcpyAsync(samp_out + (size_t)cc.out * shots, d_s + (size_t)cc.out * shots, (size_t)shots * 8,
                            cudaMemcpyDeviceToHost, st);
    }
}

// Host image of the small-layout inputs (up to o_e).
void small_image(char* img, const SmallLayout& L, const std::vector<BCirc>& bc, const std::vector<BGate>& bg,
                 const std::vector<uint64_t>& xme, const std::vector<uint64_t>& zme, const std::vector<int>& phs) {
    std::memset(img, 0, L.o_e);
    if (!bc.empty()) std::memcpy(img + L.o_c, bc.data(), bc.size() * sizeof(BCirc));
    if (!bg.empty()) std::memcpy(img + L.o_g, bg.data(), bg.size() * sizeof(BGate));
    if (!xme.empty()) {
        std::memcpy(img + L.o_x, xme.data(), xme.size() * 8);
        std::memcpy(img + L.o_z, zme.data(), zme.size() * 8);
        std::memcpy(img + L.o_ph, phs.data(), phs.size() * 4);
    }
}

uint64_t circuit_seed(uint64_t seed, int c) { return seed ^ ((uint64_t)c * 0x9E3779B97F4A7C15ULL); }

// Handles (one stream each) that run the larger circuits side by side (BS_BATCH_STREAMS, default 4, at
// most 64).  On the 512-circuit benchmark batch 4, 16 and 32 streams replay in the same 1.30-1.31 s:
// the largest circuits' sweeps, which fill the GPU on their own, set the time.
int batch_pool_size(size_t n_large) {
    static const int cap = [] {
        const char* v = getenv("BS_BATCH_STREAMS");
        const int x = v ? atoi(v) : 4;
        return std::max(1, std::min(64, x));
    }();
    return (int)std::min<size_t>(n_large, (size_t)cap);
}

void add_stats(bs_stats& a, const bs_stats& b) {
    a.sweeps += b.sweeps;
    a.kernel_launches += b.kernel_launches;
    a.gates += b.gates;
    a.bytes_moved += b.bytes_moved;
    a.tc_gates += b.tc_gates;
    a.tc_launches += b.tc_launches;
    a.tc_ms += b.tc_ms;
}

// One large circuit on handle h (reinit, evolve, Pauli expectations, shots).
int run_large(bs_sim* h, int c, int nq, const bs_op* ops, int64_t n_ops, int n_terms, const uint64_t* xmask,
              const uint64_t* zmask, int64_t shots, uint64_t seed, double* exp_out, int64_t* samp_out, bs_stats* acc) {
    int r = bs_reinit(h, nq);
    if (!r) r = bs_evolve(h, ops, n_ops, 0);
    if (!r && acc) add_stats(*acc, h->stats);
    if (!r && n_terms)
        r = bs_expectation_pauli(h, n_terms, xmask + (size_t)c * n_terms, zmask + (size_t)c * n_terms, nullptr,
                                 exp_out + (size_t)c * n_terms);
    if (!r && shots) r = bs_sample(h, circuit_seed(seed, c), shots, samp_out + (size_t)c * shots);
    return r;
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
    std::vector<uint64_t> xme, zme;
    std::vector<int> phs;
    if (!endian_terms(n_circuits, n_qubits, n_terms, xmask, zmask, xme, zme, phs)) return BS_ERR_INVALID_ARG;
    std::vector<int> small, large;
    for (int c = 0; c < n_circuits; c++) (small_ok(precision, n_qubits[c], ops[c], n_ops[c]) ? small : large).push_back(c);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int rc = BS_OK;
    bs_stats tot{};
    cudaStream_t sstream = nullptr;
    cudaStreamCreateWithFlags(&sstream, cudaStreamNonBlocking);
    cudaEventRecord(e0, sstream);
    void* dbuf = nullptr;
    std::vector<char> img;
    if (!small.empty()) {
        std::vector<BCirc> bc;
        std::vector<BGate> bg;
        rc = pack_small(small, n_qubits, ops, n_ops, bc, bg);
        if (!rc) {
            const SmallLayout L = small_layout(bc.size(), bg.size(), n_circuits, n_terms, shots);
            if (cudaMalloc(&dbuf, L.total) != cudaSuccess) rc = BS_ERR_ALLOC;
            if (!rc) {
                img.resize(L.o_e);
                small_image(img.data(), L, bc, bg, xme, zme, phs);
                enqueue_small(sstream, (char*)dbuf, L, img.data(), bc, n_terms, shots, seed, expectations_out, samples_out);
                tot.kernel_launches += 1;
            }
        }
    }
    // ---- large circuits: a pool of handles, one stream each, host worker threads
    std::atomic<int> next{0};
    std::atomic<int> err{0};
    std::sort(large.begin(), large.end(), [&](int a, int b) { return n_qubits[a] > n_qubits[b]; });
    const int workers = batch_pool_size(large.size());
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
            int r = h ? BS_OK : bs_create(BS_KIND_SV, n_qubits[c], precision, &h);
            if (!r) r = run_large(h, c, n_qubits[c], ops[c], n_ops[c], n_terms, xmask, zmask, shots, seed, expectations_out,
                                  samples_out, &wst[(size_t)w]);
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
    for (const bs_stats& x : wst) add_stats(tot, x);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    tot.gpu_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (stats_out) *stats_out = tot;
    return rc;
}

// ------------------------------------------------------------------ captured batches
// A batch whose whole execution (small circuits in one persistent launch, large circuits on a pool
// of handles and streams) is captured once into a CUDA graph and replayed by bs_batch_launch.
// Handles are sized by an eager run before the capture; every upload of the graph reads a pinned
// host image owned by the batch or by a handle's capture arena, and every result lands in the
// batch's pinned output arrays, so a replay needs no host work but the final copies.
struct bs_batch {
    int nc = 0, n_terms = 0, precision = BS_PREC_C64;
    int64_t shots = 0;
    uint64_t seed = 0;
    std::vector<int> nq;
    std::vector<uint64_t> xmask, zmask, xme, zme;
    std::vector<int> phs;
    std::vector<int> small, large;
    std::vector<int> owner;                      // large circuit -> handle (LPT by 2^n)
    std::vector<bs_sim*> h;
    cudaStream_t origin = nullptr, sstream = nullptr;
    cudaEvent_t fork = nullptr, e0 = nullptr, e1 = nullptr;
    std::vector<cudaEvent_t> join;
    // small circuits
    std::vector<BCirc> bc;
    std::vector<BGate> bg;
    SmallLayout L;
    char* dsmall = nullptr;
    size_t dsmall_bytes = 0;
    char* img = nullptr;                         // pinned host image read by the graph
    char* img_old = nullptr;
    // results, filled by every replay
    double* exp_pin = nullptr;
    int64_t* samp_pin = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bs_stats st{};
    std::vector<std::vector<std::pair<char*, size_t>>> arena_old;
    // a copy of the current ops (and their matrices), for rebuilds after a tuning change
    std::vector<std::vector<bs_op>> ops;
    std::vector<std::vector<double>> mats;
    std::vector<const bs_op*> op_ptrs;
    std::vector<int64_t> n_ops;
};

namespace {

void free_pinned(char*& p) {
    if (p) cudaFreeHost(p);
    p = nullptr;
}

// Keep a deep copy of the circuits' ops (matrix data included).
void batch_store_ops(bs_batch* b, const bs_op* const* ops, const int64_t* n_ops) {
    b->ops.assign((size_t)b->nc, {});
    b->mats.assign((size_t)b->nc, {});
    b->op_ptrs.assign((size_t)b->nc, nullptr);
    b->n_ops.assign(n_ops, n_ops + b->nc);
    for (int c = 0; c < b->nc; c++) {
        std::vector<size_t> off;
        for (int64_t i = 0; i < n_ops[c]; i++) {
            const bs_op& o = ops[c][i];
            off.push_back(b->mats[(size_t)c].size());
            if (o.kind == 2 || !o.matrix) continue;
            const int d = 1 << o.n_targets;
            size_t len;
            if (o.kind == 1) len = (size_t)std::max(o.n_matrices, 1) * d * d * 2;
            else len = (o.flags & BS_GATE_DIAGONAL) ? (size_t)d * 2 : (size_t)d * d * 2;
            b->mats[(size_t)c].insert(b->mats[(size_t)c].end(), o.matrix, o.matrix + len);
        }
        b->ops[(size_t)c].assign(ops[c], ops[c] + n_ops[c]);
        for (int64_t i = 0; i < n_ops[c]; i++) {
            bs_op& o = b->ops[(size_t)c][(size_t)i];
            if (o.kind != 2 && o.matrix) o.matrix = b->mats[(size_t)c].data() + off[(size_t)i];
        }
        b->op_ptrs[(size_t)c] = b->ops[(size_t)c].data();
    }
}

// Pack the small circuits of ops into a fresh pinned image (the previous one stays alive in
// img_old until the graph that reads it is gone); grow the device buffer if needed.
int batch_pack_small(bs_batch* b, const bs_op* const* ops, const int64_t* n_ops) {
    if (b->small.empty()) return BS_OK;
    int rc = pack_small(b->small, b->nq.data(), ops, n_ops, b->bc, b->bg);
    if (rc) return rc;
    b->L = small_layout(b->bc.size(), b->bg.size(), b->nc, b->n_terms, b->shots);
    if (b->L.total > b->dsmall_bytes) {
        if (b->dsmall) cudaFree(b->dsmall);
        b->dsmall = nullptr;
        b->dsmall_bytes = 0;
        if (cudaMalloc(&b->dsmall, b->L.total) != cudaSuccess) return BS_ERR_ALLOC;
        b->dsmall_bytes = b->L.total;
    }
    free_pinned(b->img_old);
    b->img_old = b->img;
    b->img = nullptr;
    if (cudaMallocHost(&b->img, b->L.o_e) != cudaSuccess) return BS_ERR_ALLOC;
    small_image(b->img, b->L, b->bc, b->bg, b->xme, b->zme, b->phs);
    return BS_OK;
}

// Eager run (sizes every handle buffer; results into the pinned outputs).
int batch_eager(bs_batch* b, const bs_op* const* ops, const int64_t* n_ops) {
    if (!b->small.empty())
        enqueue_small(b->sstream, b->dsmall, b->L, b->img, b->bc, b->n_terms, b->shots, b->seed, b->exp_pin, b->samp_pin);
    std::vector<int> rcs(b->h.size(), BS_OK);
    std::vector<bs_stats> ws(b->h.size());
    int dev = 0;
    cudaGetDevice(&dev);
    std::vector<std::thread> pool;
    for (size_t w = 0; w < b->h.size(); w++)
        pool.emplace_back([&, w]() {
            cudaSetDevice(dev);
            for (int c : b->large) {
                if (b->owner[(size_t)c] != (int)w) continue;
                int r = run_large(b->h[w], c, b->nq[(size_t)c], ops[c], n_ops[c], b->n_terms, b->xmask.data(), b->zmask.data(),
                                  b->shots, b->seed, b->exp_pin, b->samp_pin, &ws[w]);
                if (r) { rcs[w] = r; break; }
            }
        });
    for (auto& t : pool) t.join();
    cudaStreamSynchronize(b->sstream);
    b->st = bs_stats{};
    b->st.kernel_launches = b->small.empty() ? 0 : 1;
    for (size_t w = 0; w < ws.size(); w++) {
        add_stats(b->st, ws[w]);
        if (rcs[w]) return rcs[w];
    }
    return BS_OK;
}

// Capture the whole batch into a graph (on success *g owns it).
int batch_capture(bs_batch* b, const bs_op* const* ops, const int64_t* n_ops, cudaGraph_t* g) {
    *g = nullptr;
    if (cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed) != cudaSuccess) return BS_ERR_CUDA;
    cudaEventRecord(b->fork, b->origin);
    std::vector<cudaStream_t> ss;
    ss.push_back(b->sstream);
    for (bs_sim* s : b->h) ss.push_back(s->stream);
    for (cudaStream_t x : ss) cudaStreamWaitEvent(x, b->fork, 0);
    int rc = BS_OK;
    if (!b->small.empty())
        enqueue_small(b->sstream, b->dsmall, b->L, b->img, b->bc, b->n_terms, b->shots, b->seed, b->exp_pin, b->samp_pin);
    for (bs_sim* s : b->h) s->capturing = true;
    for (int c : b->large) {
        bs_sim* s = b->h[(size_t)b->owner[(size_t)c]];
        rc = run_large(s, c, b->nq[(size_t)c], ops[c], n_ops[c], b->n_terms, b->xmask.data(), b->zmask.data(), b->shots,
                       b->seed, b->exp_pin, b->samp_pin, nullptr);
        if (rc) break;
    }
    for (bs_sim* s : b->h) s->capturing = false;
    for (size_t i = 0; i < ss.size(); i++) {
        cudaEventRecord(b->join[i], ss[i]);
        cudaStreamWaitEvent(b->origin, b->join[i], 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->origin, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return rc ? rc : BS_ERR_CUDA;
    }
    *g = graph;
    return BS_OK;
}

// (Re)build the executable graph for ops: capture, and if a handle would have to grow a buffer,
// run eagerly once to size it and capture again.  An existing executable graph is updated in place
// when the topology allows it, otherwise replaced.
int batch_build(bs_batch* b, const bs_op* const* ops, const int64_t* n_ops, bool eager_first) {
    int rc = batch_pack_small(b, ops, n_ops);
    if (rc) return rc;
    // the arenas read by the current graph stay alive until it has been replaced
    for (bs_sim* s : b->h) {
        if (!s->arena.empty()) b->arena_old.push_back(s->arena);
        s->arena.clear();
        s->arena_used = 0;
    }
    if (eager_first) {
        rc = batch_eager(b, ops, n_ops);
        if (rc) return rc;
    }
    cudaGraph_t g = nullptr;
    rc = batch_capture(b, ops, n_ops, &g);
    if (rc == BS_ERR_STATE && !eager_first) {
        for (bs_sim* s : b->h) bs_arena_release(s);
        rc = batch_eager(b, ops, n_ops);
        if (!rc) rc = batch_capture(b, ops, n_ops, &g);
    }
    if (rc) {
        for (bs_sim* s : b->h) bs_arena_release(s);   // read by no graph
        return rc;
    }
    bool updated = false;
    if (b->exec) {
        cudaGraphExecUpdateResultInfo info{};
        updated = cudaGraphExecUpdate(b->exec, g, &info) == cudaSuccess;
        cudaGetLastError();
        if (!updated) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
    }
    if (!updated && cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
        cudaGraphDestroy(g);
        return BS_ERR_CUDA;
    }
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph = g;
    // nothing reads the previous images any more
    cudaStreamSynchronize(b->origin);
    for (auto& chunks : b->arena_old)
        for (auto& c : chunks) cudaFreeHost(c.first);
    b->arena_old.clear();
    free_pinned(b->img_old);
    return BS_OK;
}

}  // namespace

extern "C" {

int bs_batch_destroy(bs_batch* b) {
    if (!b) return BS_OK;
    if (b->origin) cudaStreamSynchronize(b->origin);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (bs_sim* s : b->h) bs_destroy(s);
    for (auto& chunks : b->arena_old)
        for (auto& c : chunks) cudaFreeHost(c.first);
    if (b->dsmall) cudaFree(b->dsmall);
    free_pinned(b->img);
    free_pinned(b->img_old);
    if (b->exp_pin) cudaFreeHost(b->exp_pin);
    if (b->samp_pin) cudaFreeHost(b->samp_pin);
    for (cudaEvent_t e : b->join) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->sstream) cudaStreamDestroy(b->sstream);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
    return BS_OK;
}

int bs_batch_create(int n_circuits, const int* n_qubits, const bs_op* const* ops, const int64_t* n_ops, int n_terms,
                    const uint64_t* xmask, const uint64_t* zmask, int64_t shots, uint64_t seed, int precision,
                    bs_batch** out) {
    if (!out) return BS_ERR_INVALID_ARG;
    *out = nullptr;
    if (n_circuits < 1 || !n_qubits || !ops || !n_ops || n_terms < 0 || n_terms > 64 || shots < 0) return BS_ERR_INVALID_ARG;
    if (n_terms > 0 && (!xmask || !zmask)) return BS_ERR_INVALID_ARG;
    if (precision != BS_PREC_C64 && precision != BS_PREC_C128) return BS_ERR_INVALID_ARG;
    for (int c = 0; c < n_circuits; c++)
        if (n_qubits[c] < 1 || n_qubits[c] > 30 || n_ops[c] < 0 || (n_ops[c] > 0 && !ops[c])) return BS_ERR_INVALID_ARG;
    bs_batch* b = new (std::nothrow) bs_batch();
    if (!b) return BS_ERR_ALLOC;
    b->nc = n_circuits;
    b->n_terms = n_terms;
    b->shots = shots;
    b->seed = seed;
    b->precision = precision;
    b->nq.assign(n_qubits, n_qubits + n_circuits);
    if (n_terms) {
        b->xmask.assign(xmask, xmask + (size_t)n_circuits * n_terms);
        b->zmask.assign(zmask, zmask + (size_t)n_circuits * n_terms);
    }
    if (!endian_terms(n_circuits, n_qubits, n_terms, b->xmask.data(), b->zmask.data(), b->xme, b->zme, b->phs)) {
        bs_batch_destroy(b);
        return BS_ERR_INVALID_ARG;
    }
    for (int c = 0; c < n_circuits; c++) (small_ok(precision, n_qubits[c], ops[c], n_ops[c]) ? b->small : b->large).push_back(c);
    // largest first onto the handle with the least work so far (work ~ 2^n)
    std::sort(b->large.begin(), b->large.end(), [&](int x, int y) { return n_qubits[x] > n_qubits[y] || (n_qubits[x] == n_qubits[y] && x < y); });
    const int workers = batch_pool_size(b->large.size());
    std::vector<double> load((size_t)workers, 0.0);
    std::vector<int> wmax((size_t)workers, 1);
    b->owner.assign((size_t)n_circuits, -1);
    for (int c : b->large) {
        const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        b->owner[(size_t)c] = w;
        load[(size_t)w] += std::ldexp(1.0, n_qubits[c]);
        wmax[(size_t)w] = std::max(wmax[(size_t)w], n_qubits[c]);
    }
    int rc = BS_OK;
    if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->sstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess || cudaEventCreate(&b->e0) != cudaSuccess ||
        cudaEventCreate(&b->e1) != cudaSuccess)
        rc = BS_ERR_CUDA;
    for (int w = 0; !rc && w < workers; w++) {
        bs_sim* s = nullptr;
        rc = bs_create(BS_KIND_SV, wmax[(size_t)w], precision, &s);
        if (!rc) b->h.push_back(s);
    }
    for (size_t i = 0; !rc && i < b->h.size() + 1; i++) {
        cudaEvent_t e;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) rc = BS_ERR_CUDA;
        else b->join.push_back(e);
    }
    if (!rc && n_terms && cudaMallocHost(&b->exp_pin, (size_t)n_circuits * n_terms * 8) != cudaSuccess) rc = BS_ERR_ALLOC;
    if (!rc && shots && cudaMallocHost(&b->samp_pin, (size_t)n_circuits * shots * 8) != cudaSuccess) rc = BS_ERR_ALLOC;
    if (!rc) {
        batch_store_ops(b, ops, n_ops);
        rc = batch_build(b, b->op_ptrs.data(), b->n_ops.data(), true);
    }
    if (rc) {
        bs_batch_destroy(b);
        return rc;
    }
    *out = b;
    return BS_OK;
}

int bs_batch_set_ops(bs_batch* b, const bs_op* const* ops, const int64_t* n_ops) {
    if (!b || !ops || !n_ops) return BS_ERR_INVALID_ARG;
    for (int c = 0; c < b->nc; c++) {
        if (n_ops[c] < 0 || (n_ops[c] > 0 && !ops[c])) return BS_ERR_INVALID_ARG;
        // a circuit may not move between the small and the large path
        const bool sm = small_ok(b->precision, b->nq[(size_t)c], ops[c], n_ops[c]);
        if (sm != (b->owner[(size_t)c] < 0)) return BS_ERR_INVALID_ARG;
    }
    batch_store_ops(b, ops, n_ops);
    return batch_build(b, b->op_ptrs.data(), b->n_ops.data(), false);
}

int bs_batch_set_tuning(bs_batch* b, int n, const int* params, const double* values) {
    if (!b || n < 0 || (n > 0 && (!params || !values))) return BS_ERR_INVALID_ARG;
    for (bs_sim* s : b->h)
        for (int i = 0; i < n; i++) {
            const int rc = bs_set_tuning(s, params[i], values[i]);
            if (rc) return rc;
        }
    return batch_build(b, b->op_ptrs.data(), b->n_ops.data(), false);
}

int bs_batch_launch(bs_batch* b, double* expectations_out, int64_t* samples_out, bs_stats* stats_out) {
    if (!b || !b->exec) return BS_ERR_INVALID_ARG;
    if ((b->n_terms > 0 && !expectations_out) || (b->shots > 0 && !samples_out)) return BS_ERR_INVALID_ARG;
    cudaEventRecord(b->e0, b->origin);
    if (cudaGraphLaunch(b->exec, b->origin) != cudaSuccess) return BS_ERR_CUDA;
    cudaEventRecord(b->e1, b->origin);
    if (cudaStreamSynchronize(b->origin) != cudaSuccess) return BS_ERR_CUDA;
    for (bs_sim* s : b->h) {
        if (s->dev_flag) s->flag_armed = true;   // the graph resets the flag at the start of each replay
        const int r = bs_check_device_flag(s);
        if (r) return r;
    }
    if (b->n_terms) std::memcpy(expectations_out, b->exp_pin, (size_t)b->nc * b->n_terms * 8);
    if (b->shots) std::memcpy(samples_out, b->samp_pin, (size_t)b->nc * b->shots * 8);
    if (stats_out) {
        *stats_out = b->st;
        float ms = 0;
        cudaEventElapsedTime(&ms, b->e0, b->e1);
        stats_out->gpu_ms = ms;
        stats_out->tc_ms = 0;
    }
    return BS_OK;
}

}  // extern "C"
