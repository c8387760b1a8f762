// Pauli-string expectations of a caller-owned state without allocating anything.
//
// Some callers cannot allocate device memory when they need an expectation value:
// a host runtime that has handed all of HBM to its own pool (a 33-qubit state
// alone is 128 GiB), a real-time loop in which the implicit device-wide
// synchronisation of cudaMalloc/cudaFree would stall unrelated work, or a thread
// that must not touch the allocator while another library owns it.  This entry
// point reads the state through the pointer they pass, keeps every partial sum in
// one library-owned static device array, and calls no cudaMalloc, cudaFree or
// other allocating routine (no host heap either: term grouping uses fixed arrays).
//
// The array (BS_NOALLOC_SCRATCH_DOUBLES doubles = 256 KiB) exists on every GPU that
// loads the library and stays there until the process exits.  All calls share it,
// so calls that may overlap on the GPU (unordered streams, several host threads)
// race on it and must be serialised by the caller.  Each call clears the part it
// accumulates into before using it.
#include <cstring>
#include "bs_internal.h"
#include "bs_ff.cuh"

#define BS_NOALLOC_MAX_TERMS 32
#define BS_NOALLOC_SCRATCH_DOUBLES 32768      // 256 KiB
#define BS_NOALLOC_MAX_BLOCKS 512             // 512 * 32 partials + 32 results < 32768

static __device__ __align__(256) double g_noalloc_scratch[BS_NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int kNThreads = 256;
constexpr int kNTermsPerPass = 8;

struct NaTermSet {
    int nt;
    uint64_t zm[kNTermsPerPass];
    int ph[kNTermsPerPass];
    int slot[kNTermsPerPass];
};

__device__ void na_block_store(double v, double* partial, int64_t idx) {
    __shared__ double red[kNThreads / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) partial[idx] = v;
    }
}

// terms sharing flip mask xm; dm != 0 reads the (a, a^xm) elements of the stored matrix
__global__ void __launch_bounds__(kNThreads) k_pauli_noalloc(const double2* __restrict__ st, int dm, int64_t dim,
                                                             uint64_t xm, NaTermSet ts, double* __restrict__ partial,
                                                             int n_slots) {
    ffsum acc[kNTermsPerPass];
    for (int t = 0; t < kNTermsPerPass; t++) acc[t] = {0.f, 0.f};
    const int64_t nwork = (!dm && xm) ? dim / 2 : dim;
    const int hb = xm ? 63 - __clzll((long long)xm) : 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nwork; p += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = p;
        float wrh, wrl, wih, wil;
        if (dm) {
            cff v = load_c128(st[i + (i ^ (int64_t)xm) * dim]);
            wrh = v.rh; wrl = v.rl; wih = v.ih; wil = v.il;
        } else if (xm) {
            const int64_t low = p & ((1LL << hb) - 1);
            i = ((p >> hb) << (hb + 1)) | low;
            cff a = load_c128(st[i]), b = load_c128(st[i ^ (int64_t)xm]);
            ffacc r, m;
            acc_first(r, a.rh, a.rl, b.rh, b.rl);
            acc_add(r, a.ih, a.il, b.ih, b.il);
            acc_first(m, a.rh, a.rl, b.ih, b.il);
            acc_add(m, -a.ih, -a.il, b.rh, b.rl);
            ff rr = acc_done(r), mm = acc_done(m);
            wrh = 2.f * rr.h; wrl = 2.f * rr.l; wih = 2.f * mm.h; wil = 2.f * mm.l;
        } else {
            cff a = load_c128(st[i]);
            ffacc r;
            acc_first(r, a.rh, a.rl, a.rh, a.rl);
            acc_add(r, a.ih, a.il, a.ih, a.il);
            ff rr = acc_done(r);
            wrh = rr.h; wrl = rr.l; wih = 0.f; wil = 0.f;
        }
        for (int t = 0; t < ts.nt; t++) {
            const bool neg = __popcll((unsigned long long)i & ts.zm[t]) & 1;
            float vh, vl;
            switch (ts.ph[t]) {
                case 0: vh = wrh; vl = wrl; break;
                case 1: vh = wih; vl = wil; break;
                case 2: vh = -wrh; vl = -wrl; break;
                default: vh = -wih; vl = -wil; break;
            }
            if (neg) { vh = -vh; vl = -vl; }
            fsum_add(acc[t], vh, vl);
        }
    }
    for (int t = 0; t < ts.nt; t++)
        na_block_store(ff2d(acc[t].h, acc[t].l), partial, (int64_t)blockIdx.x * n_slots + ts.slot[t]);
}

__global__ void k_noalloc_finish(const double* __restrict__ partial, int nblocks, int n_slots, double* __restrict__ out) {
    const int slot = blockIdx.x;
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

// Device address of the static array in the current device's context.  Looked up on every
// call rather than cached: the lookup allocates nothing, and a cached address would go stale
// once a caller resets the device (cudaDeviceReset) and the library's module is loaded again
// into the new context.  The first lookup on a device loads the library's device code.
int scratch_for_current_device(double** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return BS_ERR_CUDA;
    *out = static_cast<double*>(p);
    return BS_OK;
}

}  // namespace

extern "C" int bs_expectation_pauli_noalloc(const void* state_dev, int kind, int n_qubits, int n_terms,
                                            const uint64_t* xmask, const uint64_t* zmask, const double* coeffs,
                                            double* out, void* stream) {
    if (!state_dev || !xmask || !zmask || !out) return BS_ERR_INVALID_ARG;
    if (kind != BS_KIND_SV && kind != BS_KIND_DM) return BS_ERR_INVALID_ARG;
    if (n_terms < 1 || n_qubits < 0) return BS_ERR_INVALID_ARG;
    // beyond the static array's capacity: rejected, never truncated
    if (n_terms > BS_NOALLOC_MAX_TERMS || n_qubits > (kind == BS_KIND_SV ? 34 : 17)) return BS_ERR_UNSUPPORTED;
    const int n = n_qubits;
    const uint64_t qmask = (n >= 64) ? ~0ULL : ((1ULL << n) - 1);
    // endian masks and Y phases, grouped by flip mask with fixed-size arrays
    uint64_t xe[BS_NOALLOC_MAX_TERMS], ze[BS_NOALLOC_MAX_TERMS];
    int ph[BS_NOALLOC_MAX_TERMS];
    bool done[BS_NOALLOC_MAX_TERMS];
    for (int t = 0; t < n_terms; t++) {
        if ((xmask[t] | zmask[t]) & ~qmask) return BS_ERR_INVALID_ARG;
        uint64_t x = 0, z = 0;
        for (int q = 0; q < n; q++) {
            if ((xmask[t] >> q) & 1ULL) x |= 1ULL << (n - 1 - q);
            if ((zmask[t] >> q) & 1ULL) z |= 1ULL << (n - 1 - q);
        }
        xe[t] = x;
        ze[t] = z;
        ph[t] = __builtin_popcountll(xmask[t] & zmask[t]) & 3;
        done[t] = false;
    }
    double* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t dim = (int64_t)1 << n;
    int nb = (int)((dim + kNThreads - 1) / kNThreads);
    if (nb > BS_NOALLOC_MAX_BLOCKS) nb = BS_NOALLOC_MAX_BLOCKS;
    if (nb < 1) nb = 1;
    double* partial = scratch;
    double* res = scratch + (int64_t)nb * n_terms;
    if (cudaMemsetAsync(partial, 0, (size_t)nb * n_terms * sizeof(double), st) != cudaSuccess) return BS_ERR_CUDA;
    const double2* state = static_cast<const double2*>(state_dev);
    for (int t0 = 0; t0 < n_terms; t0++) {
        if (done[t0]) continue;
        NaTermSet set{};
        for (int t = t0; t < n_terms; t++) {
            if (done[t] || xe[t] != xe[t0]) continue;
            set.zm[set.nt] = ze[t];
            set.ph[set.nt] = ph[t];
            set.slot[set.nt] = t;
            set.nt++;
            done[t] = true;
            if (set.nt == kNTermsPerPass) {
                k_pauli_noalloc<<<nb, kNThreads, 0, st>>>(state, kind == BS_KIND_DM, dim, xe[t0], set, partial, n_terms);
                set.nt = 0;
            }
        }
        if (set.nt > 0)
            k_pauli_noalloc<<<nb, kNThreads, 0, st>>>(state, kind == BS_KIND_DM, dim, xe[t0], set, partial, n_terms);
    }
    k_noalloc_finish<<<n_terms, 256, 0, st>>>(partial, nb, n_terms, res);
    if (cudaGetLastError() != cudaSuccess) return BS_ERR_CUDA;
    if (cudaMemcpyAsync(out, res, (size_t)n_terms * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return BS_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return BS_ERR_CUDA;
    if (coeffs)
        for (int t = 0; t < n_terms; t++) out[t] *= coeffs[t];
    return BS_OK;
}
