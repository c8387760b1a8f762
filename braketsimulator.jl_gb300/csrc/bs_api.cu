// C ABI entry points: handle lifecycle, state transfer, gate / channel / evolve.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <iterator>
#include <cstring>
#include <new>
#include "bs_internal.h"

int bs_fail(bs_sim* s, int code, const std::string& msg) {
    if (s) s->err = msg;
    return code;
}
int bs_cuda_check(bs_sim* s, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return BS_OK;
    return bs_fail(s, e == cudaErrorMemoryAllocation ? BS_ERR_ALLOC : BS_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}
int bs_vec_bits(const bs_sim* s) { return s->kind == BS_KIND_DM ? 2 * s->n : s->n; }

char* bs_stage(bs_sim* s, size_t bytes) {
    bytes = (bytes + 255) & ~(size_t)255;
    if (s->capturing) {
        if (s->arena.empty() || s->arena_used + bytes > s->arena.back().second) {
            const size_t cap = std::max(bytes, (size_t)4 << 20);
            char* p = nullptr;
            if (cudaMallocHost(&p, cap) != cudaSuccess) return nullptr;
            s->arena.push_back({p, cap});
            s->arena_used = 0;
        }
        char* p = s->arena.back().first + s->arena_used;
        s->arena_used += bytes;
        return p;
    }
    if (s->hstage_pending) {
        cudaEventSynchronize(s->hstage_ev);
        s->hstage_pending = false;
    }
    if (bytes > s->hstage_cap) {
        if (s->hstage) cudaFreeHost(s->hstage);
        s->hstage = nullptr;
        s->hstage_cap = 0;
        if (cudaMallocHost(&s->hstage, bytes) != cudaSuccess) return nullptr;
        s->hstage_cap = bytes;
    }
    return s->hstage;
}
void bs_stage_done(bs_sim* s) {
    if (s->capturing) return;
    cudaEventRecord(s->hstage_ev, s->stream);
    s->hstage_pending = true;
}
void bs_arena_release(bs_sim* s) {
    for (auto& c : s->arena) cudaFreeHost(c.first);
    s->arena.clear();
    s->arena_used = 0;
}

namespace {
// Pinned landing buffer for small device-to-host results, one per host thread (handles are used
// from one thread at a time; several handles on one thread copy one after another).
constexpr size_t kOutStage = (size_t)1 << 20;
struct OutStage {
    void* p = nullptr;
    ~OutStage() {
        if (p) cudaFreeHost(p);
    }
};
thread_local OutStage t_out;
// Pinned host memory mapped into the device's address space, one per host thread: bs_run_small's
// kernel writes the probabilities and the shots straight into it (no copy call), the host reads them
// after the one synchronisation.
struct MapStage {
    char* h = nullptr;
    char* d = nullptr;
    bool tried = false;
    int64_t ticket = 0;   // bs_run_small calls of this thread: the kernel writes the call's ticket when done
    ~MapStage() {
        if (h) cudaFreeHost(h);
    }
};
thread_local MapStage t_map;
bool map_stage() {
    if (t_map.h) return true;
    if (t_map.tried) return false;
    t_map.tried = true;
    void* h = nullptr;
    void* d = nullptr;
    if (cudaHostAlloc(&h, kOutStage, cudaHostAllocMapped) != cudaSuccess) { cudaGetLastError(); return false; }
    if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) { cudaGetLastError(); cudaFreeHost(h); return false; }
    t_map.h = (char*)h;
    t_map.d = (char*)d;
    return true;
}
}  // namespace

int bs_copy_out(bs_sim* s, void* host, const void* dev, size_t bytes, const char* what) {
    if (s->capturing)   // the graph owner's buffer: enqueue only
        return bs_cuda_check(s, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s->stream), what);
    if (bytes <= kOutStage && !t_out.p && cudaMallocHost(&t_out.p, kOutStage) != cudaSuccess) {
        cudaGetLastError();
        t_out.p = nullptr;
    }
    if (bytes <= kOutStage && t_out.p) {
        int rc = bs_cuda_check(s, cudaMemcpyAsync(t_out.p, dev, bytes, cudaMemcpyDeviceToHost, s->stream), what);
        if (!rc) rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), what);
        if (!rc) std::memcpy(host, t_out.p, bytes);
        return rc;
    }
    int rc = bs_cuda_check(s, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s->stream), what);
    if (!rc) rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), what);
    return rc;
}

int bs_ensure_scratch(bs_sim* s, int64_t bytes) {
    if (s->scratch_bytes >= bytes) return BS_OK;
    if (s->capturing) return bs_fail(s, BS_ERR_STATE, "scratch growth during graph capture");
    if (s->scratch) cudaFree(s->scratch);
    s->scratch = nullptr;
    s->scratch_bytes = 0;
    int rc = bs_cuda_check(s, cudaMalloc(&s->scratch, (size_t)bytes), "scratch allocation");
    if (rc) return rc;
    s->scratch_bytes = bytes;
    return BS_OK;
}
int bs_ensure_plan(bs_sim* s, int64_t bytes) {
    if (s->plan_bytes >= bytes) return BS_OK;
    if (s->capturing) return bs_fail(s, BS_ERR_STATE, "plan buffer growth during graph capture");
    // the previous plan may still be read by queued kernels
    cudaStreamSynchronize(s->stream);
    if (s->plan_buf) cudaFree(s->plan_buf);
    s->plan_buf = nullptr;
    s->plan_bytes = 0;
    int64_t b = std::max<int64_t>(bytes, 1 << 16);
    int rc = bs_cuda_check(s, cudaMalloc(&s->plan_buf, (size_t)b), "plan allocation");
    if (rc) return rc;
    s->plan_bytes = b;
    return BS_OK;
}

namespace {

__global__ void k_basis0(double2* psi) { psi[0] = make_double2(1.0, 0.0); }
__global__ void k_basis0_c64(float2* psi) { psi[0] = make_float2(1.0f, 0.0f); }

// complex128 <-> complex64 element conversion (round to nearest)
__global__ void k_to_c64(const double2* __restrict__ in, float2* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_float2(__double2float_rn(in[i].x), __double2float_rn(in[i].y));
}
__global__ void k_to_c128(const float2* __restrict__ in, double2* __restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = make_double2((double)in[i].x, (double)in[i].y);
}

int elem_bytes(const bs_sim* s) { return s->precision == BS_PREC_C64 ? 8 : 16; }

// complex128 host buffer <-> complex64 state, through a bounded device staging buffer
int transfer_c64(bs_sim* s, double* host, int64_t n, bool to_device) {
    const int64_t chunk = std::min<int64_t>(n, (int64_t)1 << 22);   // 64 MiB of complex128
    int rc = bs_ensure_scratch(s, chunk * 16);
    if (rc) return rc;
    double2* stage = (double2*)s->scratch;
    float2* st = (float2*)s->state;
    for (int64_t off = 0; off < n; off += chunk) {
        const int64_t m = std::min<int64_t>(chunk, n - off);
        const int blocks = (int)std::min<int64_t>((m + 255) / 256, 152 * 8);
        if (to_device) {
            rc = bs_cuda_check(s, cudaMemcpyAsync(stage, host + 2 * off, (size_t)m * 16, cudaMemcpyHostToDevice, s->stream), "set_state");
            if (rc) return rc;
            k_to_c64<<<blocks, 256, 0, s->stream>>>(stage, st + off, m);
        } else {
            k_to_c128<<<blocks, 256, 0, s->stream>>>(st + off, stage, m);
            rc = bs_cuda_check(s, cudaMemcpyAsync(host + 2 * off, stage, (size_t)m * 16, cudaMemcpyDeviceToHost, s->stream), "get_state");
            if (rc) return rc;
        }
        rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), "state transfer");
        if (rc) return rc;
    }
    return BS_OK;
}

int alloc_state(bs_sim* s, int n) {
    const int bits = (s->kind == BS_KIND_DM) ? 2 * n : n;
    if (n < 0 || bits > 34) return bs_fail(s, BS_ERR_INVALID_ARG, "qubit count out of range");
    const int64_t len = (int64_t)1 << bits;
    const int64_t bytes = len * elem_bytes(s);
    if (bytes > s->cap_bytes) {
        if (s->capturing) return bs_fail(s, BS_ERR_STATE, "state growth during graph capture");
        if (s->state) cudaFree(s->state);
        s->state = nullptr;
        s->cap_bytes = 0;
        int rc = bs_cuda_check(s, cudaMalloc(&s->state, (size_t)bytes), "state allocation");
        if (rc) return rc;
        s->cap_bytes = bytes;
    }
    s->n = n;
    s->len = len;
    s->alias_valid = false;
    int rc = bs_cuda_check(s, cudaMemsetAsync(s->state, 0, (size_t)bytes, s->stream), "state clear");
    if (rc) return rc;
    if (s->precision == BS_PREC_C64) k_basis0_c64<<<1, 1, 0, s->stream>>>((float2*)s->state);
    else k_basis0<<<1, 1, 0, s->stream>>>((double2*)s->state);
    return bs_cuda_check(s, cudaGetLastError(), "state init");
}

bool ok_handle(bs_sim* s) { return s != nullptr; }

}  // namespace

extern "C" {

const char* bs_version(void) { return "braket_gb300 0.1 (sm_103a, float-float complex128)"; }

int bs_create(int kind, int n_qubits, int precision, bs_sim** out) {
    if (!out) return BS_ERR_INVALID_ARG;
    *out = nullptr;
    if (kind != BS_KIND_SV && kind != BS_KIND_DM) return BS_ERR_INVALID_ARG;
    if (precision != BS_PREC_C128 && precision != BS_PREC_C64) return BS_ERR_INVALID_ARG;
    bs_sim* s = new (std::nothrow) bs_sim();
    if (!s) return BS_ERR_ALLOC;
    s->kind = kind;
    s->precision = precision;
    cudaGetDevice(&s->device);
    int rc = bs_cuda_check(s, cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream");
    if (!rc) rc = bs_cuda_check(s, cudaEventCreate(&s->ev0), "event");
    if (!rc) rc = bs_cuda_check(s, cudaEventCreate(&s->ev1), "event");
    if (!rc) rc = bs_cuda_check(s, cudaEventCreateWithFlags(&s->hstage_ev, cudaEventDisableTiming), "event");
    if (!rc) rc = alloc_state(s, n_qubits);
    if (rc) { bs_destroy(s); return rc; }
    *out = s;
    return BS_OK;
}

int bs_destroy(bs_sim* s) {
    if (!s) return BS_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->state) cudaFree(s->state);
    if (s->scratch) cudaFree(s->scratch);
    if (s->plan_buf) cudaFree(s->plan_buf);
    if (s->dev_flag) cudaFree(s->dev_flag);
    if (s->alias_ap) cudaFree(s->alias_ap);
    if (s->alias_ix) cudaFree(s->alias_ix);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    for (cudaEvent_t e : s->tc_events) cudaEventDestroy(e);
    if (s->hstage_ev) cudaEventDestroy(s->hstage_ev);
    if (s->hstage) cudaFreeHost(s->hstage);
    bs_arena_release(s);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return BS_OK;
}

int bs_set_tuning(bs_sim* s, int param, double value) {
    if (!s) return BS_ERR_INVALID_ARG;
    const bool reset = value < 0;
    const int iv = (int)value;
    switch (param) {
        case BS_TUNE_TILE_BITS:
            if (!reset && (iv < 10 || iv > BS_TILE_MAX_BITS || iv != value)) break;
            s->tune.tile_bits = reset ? -1 : iv;
            return BS_OK;
        case BS_TUNE_TILE_THREADS:
            if (!reset && iv != 256 && iv != 512) break;
            s->tune.tile_threads = reset ? -1 : iv;
            return BS_OK;
        case BS_TUNE_TC:
            if (!reset && iv != 0 && iv != 1) break;
            s->tune.tc = reset ? -1 : iv;
            return BS_OK;
        case BS_TUNE_TC_MIN_BITS:
            if (!reset && (iv > 64 || iv != value)) break;
            s->tune.tc_min_bits = reset ? -1 : iv;
            return BS_OK;
        case BS_TUNE_TC_COST:
            if (!reset && !(value < 1e9)) break;
            s->tune.tc_cost = reset ? -1.0 : value;
            return BS_OK;
        case BS_TUNE_ADJ_SEGMENTS:
            if (!reset && (iv < 1 || iv > 1024 || iv != value)) break;
            s->tune.adj_segments = reset ? -1 : iv;
            return BS_OK;
        default:
            return bs_fail(s, BS_ERR_INVALID_ARG, "unknown tuning parameter");
    }
    return bs_fail(s, BS_ERR_INVALID_ARG, "tuning value out of range");
}

int bs_get_tuning(bs_sim* s, int param, double* value) {
    if (!s || !value) return BS_ERR_INVALID_ARG;
    switch (param) {
        case BS_TUNE_TILE_BITS: *value = bs_tile_bits(s); return BS_OK;
        case BS_TUNE_TILE_THREADS: *value = bs_tile_threads(s); return BS_OK;
        case BS_TUNE_TC: *value = bs_tc_enabled(s) ? 1.0 : 0.0; return BS_OK;
        case BS_TUNE_TC_MIN_BITS: *value = bs_tc_min_bits(s); return BS_OK;
        case BS_TUNE_TC_COST: *value = bs_tc_cost(s); return BS_OK;
        case BS_TUNE_ADJ_SEGMENTS: *value = s->tune.adj_segments; return BS_OK;
        default: return bs_fail(s, BS_ERR_INVALID_ARG, "unknown tuning parameter");
    }
}

int bs_reinit(bs_sim* s, int n_qubits) {
    if (!ok_handle(s)) return BS_ERR_INVALID_ARG;
    return alloc_state(s, n_qubits);
}

int bs_qubit_count(const bs_sim* s, int* out) {
    if (!s || !out) return BS_ERR_INVALID_ARG;
    *out = s->n;
    return BS_OK;
}

const char* bs_last_error(const bs_sim* s) { return s ? s->err.c_str() : "null handle"; }

int bs_set_state(bs_sim* s, const double* host, int64_t n) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!host || n != s->len) return bs_fail(s, BS_ERR_INVALID_ARG, "state length mismatch");
    s->alias_valid = false;
    if (s->precision == BS_PREC_C64) return transfer_c64(s, const_cast<double*>(host), n, true);
    int rc = bs_cuda_check(s, cudaMemcpyAsync(s->state, host, (size_t)n * 16, cudaMemcpyHostToDevice, s->stream), "set_state");
    if (rc) return rc;
    return bs_cuda_check(s, cudaStreamSynchronize(s->stream), "set_state sync");
}

int bs_get_state(bs_sim* s, double* host, int64_t n) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!host || n != s->len) return bs_fail(s, BS_ERR_INVALID_ARG, "state length mismatch");
    if (s->precision == BS_PREC_C64) return transfer_c64(s, host, n, false);
    int rc = bs_cuda_check(s, cudaMemcpyAsync(host, s->state, (size_t)n * 16, cudaMemcpyDeviceToHost, s->stream), "get_state");
    if (rc) return rc;
    return bs_cuda_check(s, cudaStreamSynchronize(s->stream), "get_state sync");
}

int bs_set_state_device(bs_sim* s, const void* dev, int64_t n) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!dev || n != s->len) return bs_fail(s, BS_ERR_INVALID_ARG, "state length mismatch");
    s->alias_valid = false;
    return bs_cuda_check(s, cudaMemcpyAsync(s->state, dev, (size_t)n * elem_bytes(s), cudaMemcpyDeviceToDevice, s->stream), "set_state_device");
}

int bs_get_state_device(bs_sim* s, void* dev, int64_t n) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (!dev || n != s->len) return bs_fail(s, BS_ERR_INVALID_ARG, "state length mismatch");
    return bs_cuda_check(s, cudaMemcpyAsync(dev, s->state, (size_t)n * elem_bytes(s), cudaMemcpyDeviceToDevice, s->stream), "get_state_device");
}

int bs_copy_state(bs_sim* dst, const bs_sim* src) {
    if (!dst || !src) return BS_ERR_INVALID_ARG;
    if (dst->kind != src->kind || dst->len != src->len || dst->precision != src->precision)
        return bs_fail(dst, BS_ERR_INVALID_ARG, "simulators differ in kind, size or precision");
    cudaStreamSynchronize(src->stream);
    dst->alias_valid = false;
    return bs_cuda_check(dst, cudaMemcpyAsync(dst->state, src->state, (size_t)dst->len * elem_bytes(dst),
                                              cudaMemcpyDeviceToDevice, dst->stream), "copy_state");
}

int bs_synchronize(bs_sim* s) {
    if (!s) return BS_ERR_INVALID_ARG;
    int rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), "synchronize");
    if (!rc) bs_collect_tc_time(s);
    return rc ? rc : bs_check_device_flag(s);
}

int bs_state_device_ptr(bs_sim* s, void** out) {
    if (!s || !out) return BS_ERR_INVALID_ARG;
    *out = s->state;
    return BS_OK;
}

int bs_last_stats(const bs_sim* s, bs_stats* out) {
    if (!s || !out) return BS_ERR_INVALID_ARG;
    *out = s->stats;
    if (s->stats_pending) {   // an evolve that returned without waiting: its device time
        float ms = 0.f;
        if (cudaEventSynchronize(s->ev1) == cudaSuccess && cudaEventElapsedTime(&ms, s->ev0, s->ev1) == cudaSuccess)
            out->gpu_ms = ms;
    }
    return BS_OK;
}

int bs_apply_gate(bs_sim* s, const double* matrix, int k, const int* targets, int nc, const int* controls,
                  const int* cvals, unsigned flags) {
    if (!s) return BS_ERR_INVALID_ARG;
    std::vector<HostGate> hg;
    int rc = bs_lower_gate(s, matrix, k, targets, nc, controls, cvals, flags, s->kind == BS_KIND_DM, hg);
    if (rc) return rc;
    std::vector<Sweep> sw;
    bs_plan_sweeps(hg, bs_vec_bits(s), bs_tile_bits(s), sw);
    s->alias_valid = false;
    return bs_run_sweeps(s, sw);
}

int bs_dm_apply_vec_gate(bs_sim* s, const double* matrix, int k, const int* targets, int nc, const int* controls,
                         const int* cvals, unsigned flags) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (s->kind != BS_KIND_DM) return bs_fail(s, BS_ERR_STATE, "vec gate needs a density-matrix simulator");
    std::vector<HostGate> hg;
    int rc = bs_lower_gate(s, matrix, k, targets, nc, controls, cvals, flags, false, hg);
    if (rc) return rc;
    std::vector<Sweep> sw;
    bs_plan_sweeps(hg, bs_vec_bits(s), bs_tile_bits(s), sw);
    s->alias_valid = false;
    return bs_run_sweeps(s, sw);
}

int bs_apply_kraus(bs_sim* s, const double* kraus, int nk, int k, const int* targets, unsigned flags) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (s->kind != BS_KIND_DM) return bs_fail(s, BS_ERR_STATE, "noise needs a density-matrix simulator");
    if (!kraus || !targets) return bs_fail(s, BS_ERR_INVALID_ARG, "null argument");
    s->alias_valid = false;
    if (flags & BS_NOISE_PHYSICAL) {
        std::vector<HostGate> hg;
        int rc = bs_lower_kraus_physical(s, kraus, nk, k, targets, flags, hg);
        if (rc) return rc;
        std::vector<Sweep> sw;
        bs_plan_sweeps(hg, bs_vec_bits(s), bs_tile_bits(s), sw);
        return bs_run_sweeps(s, sw);
    }
    return bs_kraus_reference(s, kraus, nk, k, targets, flags);
}

// A SWAP of two qubits (no controls, no phases) moves no data here: the evolve keeps a map from
// logical to physical endian bits, relabels every later gate through it, and restores the order
// once at the end (or before a direct kernel call) with as few physical swaps as the map needs.
static bool is_plain_swap(const HostGate& g) {
    return g.kind == 2 && g.k == 2 && g.cmask == 0 && g.perm.size() == 8 && g.perm[0] == 0 && g.perm[1] == 0 &&
           g.perm[2] == 2 && g.perm[3] == 0 && g.perm[4] == 1 && g.perm[5] == 0 && g.perm[6] == 3 && g.perm[7] == 0;
}

int bs_evolve(bs_sim* s, const bs_op* ops, int64_t n_ops, unsigned noise_mode) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (n_ops < 0 || (n_ops > 0 && !ops)) return bs_fail(s, BS_ERR_INVALID_ARG, "bad op list");
    s->stats = bs_stats{};
    s->stats_pending = false;
    if (!s->defer_sync) s->tc_events_used = 0;   // deferred evolves keep their launch events for the caller
    s->alias_valid = false;
    if (!s->capturing && !s->collect) cudaEventRecord(s->ev0, s->stream);   // a plan-only call times nothing
    std::vector<HostGate> pending, lowered;
    const int nb = bs_vec_bits(s);
    int phys[64];   // physical endian bit of each logical one
    for (int e = 0; e < 64; e++) phys[e] = e;
    bool permuted = false;
    auto relabel = [&](std::vector<HostGate>& gs) {
        for (HostGate& g : gs) {
            if (is_plain_swap(g)) {
                std::swap(phys[g.ebit[0]], phys[g.ebit[1]]);
                permuted = true;
                continue;
            }
            if (permuted) {
                const int nbits = g.kind == 5 ? 2 * g.k : g.k;
                for (int q = 0; q < nbits; q++) g.ebit[q] = phys[g.ebit[q]];
                uint64_t cm = 0, cv = 0;
                for (int e = 0; e < 64; e++)
                    if ((g.cmask >> e) & 1ULL) {
                        cm |= 1ULL << phys[e];
                        cv |= ((g.cval >> e) & 1ULL) << phys[e];
                    }
                g.cmask = cm;
                g.cval = cv;
            }
            pending.push_back(std::move(g));
        }
        gs.clear();
    };
    auto restore = [&]() {
        // physical swaps until logical bit l lives at physical bit l
        if (!permuted) return;
        for (int l = 0; l < nb; l++) {
            if (phys[l] == l) continue;
            const int p = phys[l];
            int m = 0;
            while (phys[m] != l) m++;
            HostGate g;
            g.kind = 2;
            g.k = 2;
            g.ebit[0] = l;
            g.ebit[1] = p;
            g.perm = {0, 0, 2, 0, 1, 0, 3, 0};
            pending.push_back(std::move(g));
            phys[l] = l;
            phys[m] = p;
        }
        permuted = false;
    };
    auto flush = [&]() -> int {
        if (pending.empty()) return BS_OK;
        std::vector<Sweep> sw;
        bs_plan_sweeps(pending, bs_vec_bits(s), bs_tile_bits(s), sw);
        pending.clear();
        if (s->collect) {   // bs_run_small: plan only
            s->collect->insert(s->collect->end(), std::make_move_iterator(sw.begin()), std::make_move_iterator(sw.end()));
            return BS_OK;
        }
        return bs_run_sweeps(s, sw);
    };
    const bool dm = s->kind == BS_KIND_DM;
    for (int64_t i = 0; i < n_ops; i++) {
        const bs_op& op = ops[i];
        int rc = BS_OK;
        if (op.kind == 2) continue;
        if (op.kind == 0) {
            rc = bs_lower_gate(s, op.matrix, op.n_targets, op.targets, op.n_controls, op.controls,
                               op.control_values, op.flags, dm, lowered);
        } else if (op.kind == 1) {
            if (!dm) return bs_fail(s, BS_ERR_STATE, "noise instruction on a state-vector simulator");
            unsigned mode = (op.flags & BS_NOISE_PHYSICAL) ? BS_NOISE_PHYSICAL : noise_mode;
            if (mode & BS_NOISE_PHYSICAL) {
                rc = bs_lower_kraus_physical(s, op.matrix, op.n_matrices, op.n_targets, op.targets, op.flags, lowered);
            } else if (s->precision == BS_PREC_C128 && op.n_targets <= 2) {
                // inside the sweeps (complex128 tile kernels)
                rc = bs_lower_kraus_reference(s, op.matrix, op.n_matrices, op.n_targets, op.targets, op.flags,
                                              lowered);
            } else {
                restore();
                rc = flush();
                if (!rc) rc = bs_kraus_reference(s, op.matrix, op.n_matrices, op.n_targets, op.targets, op.flags);
            }
        } else {
            return bs_fail(s, BS_ERR_INVALID_ARG, "unknown op kind");
        }
        if (rc) return rc;
        relabel(lowered);
    }
    restore();
    int rc = flush();
    if (rc) return rc;
    if (s->capturing || s->defer_sync) return BS_OK;   // the graph's launcher / the caller synchronises and checks
    cudaEventRecord(s->ev1, s->stream);
    if (!s->flag_armed && s->tc_events_used == 0) {
        // nothing to check on the device: return without waiting (the next result read synchronises;
        // bs_last_stats waits for the end event when asked for the time)
        s->stats_pending = true;
        return bs_cuda_check(s, cudaGetLastError(), "evolve");
    }
    rc = bs_cuda_check(s, cudaEventSynchronize(s->ev1), "evolve");
    if (rc) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->stats.gpu_ms = ms;
    bs_collect_tc_time(s);
    return bs_check_device_flag(s);
}

// simulate (src/BraketSimulator.jl:307-322: reinit!, evolve!, probabilities, samples) of one small
// state-vector circuit as one upload, one launch and one synchronisation: the kernel evolves the
// state in one CTA, writes it back, and writes the probabilities and the shots into mapped pinned
// host memory.
int bs_run_small(bs_sim* s, const bs_op* ops, int64_t n_ops, int64_t shots, uint64_t seed, double* probs_out,
                 int64_t* samples_out) {
    if (!s) return BS_ERR_INVALID_ARG;
    if (s->kind != BS_KIND_SV || s->n > 12) return bs_fail(s, BS_ERR_UNSUPPORTED, "bs_run_small: state vectors of at most 12 qubits");
    if (s->capturing) return bs_fail(s, BS_ERR_STATE, "bs_run_small: not during graph capture");
    if (shots < 0 || (shots > 0 && !samples_out)) return bs_fail(s, BS_ERR_INVALID_ARG, "bad shot buffer");
    const int64_t dim = (int64_t)1 << s->n;
    // The list's exact bytes: the qubit count and tile setting, every op struct without its matrix
    // pointer, every matrix's values.  The same bytes as the last call reuse its plan.  Lists with
    // a malformed op or more than 1 MiB of matrices are planned every time (bs_evolve reports errors).
    std::vector<char> key;
    bool keyed = n_ops >= 0 && (n_ops == 0 || ops);
    if (keyed) {
        const int head[2] = {s->n, bs_tile_bits(s)};
        key.insert(key.end(), (const char*)head, (const char*)head + sizeof(head));
        size_t mat_bytes = 0;
        for (int64_t i = 0; i < n_ops && keyed; i++) {
            bs_op o = ops[i];
            const double* m = o.matrix;
            o.matrix = nullptr;
            key.insert(key.end(), (const char*)&o, (const char*)&o + sizeof(o));
            if (o.kind == 2) continue;
            if (o.kind != 0 || !m || o.n_targets < 1 || o.n_targets > BS_MAX_TARGETS) { keyed = false; break; }
            const size_t d = (size_t)1 << o.n_targets;
            const size_t nd = 2 * ((o.flags & BS_GATE_DIAGONAL) ? d : d * d);
            mat_bytes += nd * sizeof(double);
            if (mat_bytes > ((size_t)1 << 20)) { keyed = false; break; }
            key.insert(key.end(), (const char*)m, (const char*)(m + nd));
        }
    }
    int rc = BS_OK;
    bool in_tile = true;   // the plan has an in-tile kernel for every gate (else the usual path runs)
    if (!(keyed && s->small_valid && key == s->small_key)) {
        std::vector<Sweep> sweeps;
        // plan the instruction list as bs_evolve does (lowering, SWAP relabelling, diagonal folding),
        // launching nothing
        s->small_valid = false;
        s->collect = &sweeps;
        const bool defer = s->defer_sync;
        s->defer_sync = true;
        rc = bs_evolve(s, ops, n_ops, BS_NOISE_REFERENCE);
        s->defer_sync = defer;
        s->collect = nullptr;
        if (rc) return rc;
        rc = bs_small_pack(s, sweeps, s->small_plan);
        if (rc && rc != BS_ERR_UNSUPPORTED) return rc;
        in_tile = rc == BS_OK;
        if (in_tile && keyed) {
            s->small_key.swap(key);
            s->small_valid = true;
        }
    } else {
        s->stats = bs_stats{};
        s->stats_pending = false;
    }
    // mapped layout: the completion word and the kernel's start and end times (256 bytes), the
    // probabilities, the shots, then room for the plan
    const size_t pb = ((size_t)dim * 8 + 255) & ~(size_t)255, sb = ((size_t)shots * 8 + 255) & ~(size_t)255;
    const bool mapped = 256 + pb + sb <= kOutStage && map_stage();
    double* dprobs;
    int64_t* dsamp;
    int64_t* ddone = nullptr;
    int64_t ticket = 0;
    SmallIO io{};
    if (mapped) {
        ddone = (int64_t*)t_map.d;
        ticket = ++t_map.ticket;
        dprobs = (double*)(t_map.d + 256);
        dsamp = (int64_t*)(t_map.d + 256 + pb);
        io.hplan = t_map.h + 256 + pb + sb;
        io.dplan = t_map.d + 256 + pb + sb;
        io.plan_cap = kOutStage - (256 + pb + sb);
        io.dtimes = (int64_t*)(t_map.d + 8);
    } else {
        rc = bs_ensure_scratch(s, (int64_t)(pb + sb) + 256);
        if (rc) return rc;
        dprobs = (double*)s->scratch;
        dsamp = (int64_t*)((char*)s->scratch + pb);
        cudaEventRecord(s->ev0, s->stream);
    }
    rc = in_tile ? bs_small_launch(s, s->small_plan, dprobs, shots, seed, dsamp, ddone, ticket, mapped ? &io : nullptr)
                 : BS_ERR_UNSUPPORTED;
    if (rc == BS_ERR_UNSUPPORTED) {
        // a gate without an in-tile kernel (dense on more than 4 qubits) or a complex64 state: the usual
        // path, with the same results
        rc = bs_reinit(s, s->n);
        if (!rc) rc = bs_evolve(s, ops, n_ops, BS_NOISE_REFERENCE);
        if (!rc && probs_out) rc = bs_probabilities(s, probs_out, dim);
        if (!rc && shots > 0) rc = bs_sample(s, seed, shots, samples_out);
        return rc;
    }
    if (rc) return rc;
    s->alias_valid = false;
    if (!mapped) {
        cudaEventRecord(s->ev1, s->stream);
        if (probs_out) cudaMemcpyAsync(probs_out, dprobs, (size_t)dim * 8, cudaMemcpyDeviceToHost, s->stream);
        if (sb) cudaMemcpyAsync(samples_out, dsamp, sb, cudaMemcpyDeviceToHost, s->stream);
        rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), "small run");
        if (rc) return rc;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->ev0, s->ev1);
        s->stats.gpu_ms = ms;
        s->stats_pending = false;
        return BS_OK;
    }
    // Wait for the kernel's completion word rather than synchronising the stream (a round trip through
    // the driver that costs more than the kernel): the kernel writes the ticket after every result is
    // visible to the host.  A ticket that has not arrived after 2 s (a failed kernel) falls back to the
    // stream synchronisation, which reports the error.
    volatile int64_t* word = reinterpret_cast<volatile int64_t*>(t_map.h);
    const auto t0 = std::chrono::steady_clock::now();
    bool seen = false;
    for (uint32_t it = 0;; it++) {
        if (*word == ticket) { seen = true; break; }
        if ((it & 1023u) == 1023u && std::chrono::steady_clock::now() - t0 > std::chrono::seconds(2)) break;
    }
    std::atomic_thread_fence(std::memory_order_acquire);
    if (!seen) {
        rc = bs_cuda_check(s, cudaStreamSynchronize(s->stream), "small run");
        if (rc) return rc;
    }
    if (probs_out) std::memcpy(probs_out, t_map.h + 256, (size_t)dim * 8);
    if (shots > 0) std::memcpy(samples_out, t_map.h + 256 + pb, (size_t)shots * 8);
    // device time: the kernel's own start and end stamps (no events on this path)
    const volatile int64_t* times = reinterpret_cast<const volatile int64_t*>(t_map.h + 8);
    s->stats.gpu_ms = (double)(times[1] - times[0]) * 1e-6;
    s->stats_pending = false;
    return BS_OK;
}

}  // extern "C"
