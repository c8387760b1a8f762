// Internal structures shared by the translation units of libbraket_gb300.so.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/braket_gb300.h"

#define BS_TILE_MAX_BITS 12      // 2^12 complex float-float values = 64 KiB of shared memory
#define BS_TILE_LOW_BITS 5       // low endian bits always in a tile: 32 contiguous amplitudes
#define BS_TILE_MAXK 4           // dense targets per tile gate (16x16 superoperators for 2q noise)

// One gate inside a tile sweep.
//   kind 0: dense 2^k x 2^k on tile-local bits tbit[0..k-1] (matrix bit j <-> tbit[j])
//   kind 1: diagonal 2^k entries selected by global bits gbit[0..k-1]
//   kind 2: monomial (one unit-modulus phase i^p per column) on tile-local bits
//   kind 3: a run of CZ gates applied as one parity phase (npar, pshift, pmask)
//   kind 4: fused dense unitary on 5 tile-local bits gbit[0..4] (matrix bit j <-> gbit[j]),
//           applied on the tensor cores from the bf16 digit slices at tc_off (48 KiB blocks)
//   kind 5: Kraus channel on k <= 2 targets in the reference's block-diagonal update rule
//           (density matrix): tbit[0..2k-1] row then column target bits, pmask[0..1], npar = nk
// Controls: (tile_index & lc_mask) == lc_val for in-tile controls,
//           (global_base & gc_mask) == gc_val for controls outside the tile.
struct TileGate {
    int32_t kind;
    int32_t k;
    int32_t tbit[BS_TILE_MAXK];
    int32_t gbit[BS_MAX_TARGETS];
    uint32_t lc_mask, lc_val;
    uint64_t gc_mask, gc_val;
    int32_t mat_off;            // offset (in cff units) into the sweep's matrix pool
    int32_t perm_off;           // monomial: offset into the permutation pool (int32 pairs)
    // kind 3: a run of CZ gates as one phase (-1)^(sum_q popc(i & (i >> pshift[q]) & pmask[q]))
    int32_t npar;
    int32_t pshift[4];
    uint64_t pmask[4];
    int32_t tc_off;             // kind 4: index of the digit-slice block in the sweep's pool
    int32_t tc_eu;              // kind 4: matrix entries are below 2^tc_eu
    int32_t tc_nu;              // kind 4: the CTA's base bits tc_ub[0..tc_nu-1] select the variant block
    int32_t tc_ub[3];
};

struct SweepDesc {
    int32_t n_bits;             // endian bits of the vector (n for SV, 2n for DM)
    int32_t T;                  // tile bits
    int32_t L;                  // low contiguous bits
    int32_t n_gates;
    int32_t hi_bits[BS_TILE_MAX_BITS];
    uint64_t tile_mask;
    const TileGate* gates;      // device
    const float4* mats;         // device, complex float-float entries (rh, rl, ih, il)
    const int32_t* perms;       // device
    const uint16_t* tc_pool;    // device, kind-4 digit slices (24576 bf16 per gate)
    int* err;                   // device flag: a bounded tensor-core wait gave up
};

struct HostGate {                // a gate after lowering to the canonical convention
    int kind;                    // 0 dense, 1 diagonal, 2 monomial, 4 fused 5-bit unitary,
                                 // 5 reference-rule Kraus channel (ebit: k row bits, then k column bits)
    int k;
    int ebit[BS_MAX_TARGETS];    // endian bit of target j (matrix bit j)
    std::vector<double> mat;     // interleaved complex; dense 4^k*2, diag 2^k*2
    uint64_t cmask = 0, cval = 0;// controls on endian bits
    std::vector<int> perm;       // monomial: column c -> (row, i-power)
    std::vector<int> ubits;      // kind 4: out-of-tile bits the fused matrix depends on; mat holds
                                 // 2^|ubits| matrices, variant v for bit values v_i at ubits[i]
};

struct Sweep {
    std::vector<int> hi_bits;    // tile bits above the low contiguous block
    std::vector<HostGate> gates;
};

// Per-handle tuning (bs_set_tuning); a negative value means "environment variable, else the
// built-in default" (BS_TILE_BITS 12, BS_TILE_THREADS 256, BS_TC 1, BS_TC_MIN_BITS 22, BS_TC_COST 2).
struct BsTuning {
    int tile_bits = -1;      // tile bits of the sweep kernels, 10..12
    int tile_threads = -1;   // threads per CTA of the float-float sweep kernel, 256 or 512
    int tc = -1;             // fused tensor-core sweeps on (1) or off (0)
    int tc_min_bits = -1;    // vector bits from which fused tensor-core sweeps are used
    double tc_cost = -1;     // float-float cost (dense 1-qubit gates) above which a block is fused
    int adj_segments = -1;   // adjoint gradients: forward segments (checkpoints + 1); -1 = from memory
};

// The packed plan of one small-circuit run (bs_run_small): the whole state is one tile, so the plan is
// the gate table, its matrices and permutations, and the largest dense or monomial target count.
struct SmallPlan {
    std::vector<TileGate> tg;
    std::vector<float4> mats;
    std::vector<int32_t> perms;
    int kmax = 1;
};

struct bs_sim {
    int kind = BS_KIND_SV;
    int n = 0;                    // qubits
    int precision = BS_PREC_C128;
    int device = 0;
    cudaStream_t stream = nullptr;
    void* state = nullptr;        // complex128: double2[len]
    int64_t len = 0;              // elements of the state vector / vec(S)
    int64_t cap_bytes = 0;
    // scratch for reductions and sampling
    void* scratch = nullptr;
    int64_t scratch_bytes = 0;
    double* alias_ap = nullptr;
    int64_t* alias_ix = nullptr;
    int64_t alias_len = 0;
    bool alias_valid = false;
    // plan upload buffer
    void* plan_buf = nullptr;
    int64_t plan_bytes = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int* dev_flag = nullptr;      // device error flag of the tensor-core sweeps
    bool flag_armed = false;
    std::vector<cudaEvent_t> tc_events;   // pool: an event pair around each tensor-core launch
    size_t tc_events_used = 0;            // pairs recorded since the last bs_collect_tc_time
    bs_stats stats{};
    BsTuning tune{};
    std::string err;
    // Host staging of uploads: pinned, reused once the previous upload has landed (hstage_ev).
    char* hstage = nullptr;
    size_t hstage_cap = 0;
    cudaEvent_t hstage_ev = nullptr;
    bool hstage_pending = false;
    // While the handle's stream is captured into a CUDA graph: no host synchronisation, no device
    // buffer growth, and staging comes from an append-only pinned arena that lives as long as the
    // graph (the graph's copy nodes read it on every replay).
    bool capturing = false;
    bool defer_sync = false;   // bs_evolve returns without synchronising (an internal caller syncs later)
    bool stats_pending = false;   // an evolve returned before its end event (ev1) completed
    std::vector<std::pair<char*, size_t>> arena;   // chunks (pointer, capacity)
    size_t arena_used = 0;                          // bytes used in the last chunk
    std::vector<Sweep>* collect = nullptr;          // bs_evolve plans into this list instead of launching
    // bs_run_small: the plan of the last instruction list, kept with the list's exact bytes (op structs
    // without their matrix pointers, the matrix values, the qubit count and tile setting) so that the
    // same list again skips the planning
    std::vector<char> small_key;
    SmallPlan small_plan;
    bool small_valid = false;
};

// ---- helpers implemented in bs_api.cu
int bs_fail(bs_sim* s, int code, const std::string& msg);
int bs_cuda_check(bs_sim* s, cudaError_t e, const char* what);
// Device-to-host copy of a result, stream synchronised; small ones land in a pinned per-thread
// buffer first (a pageable copy takes a staged driver path).  During graph capture: enqueue only.
int bs_copy_out(bs_sim* s, void* host, const void* dev, size_t bytes, const char* what);
int bs_ensure_scratch(bs_sim* s, int64_t bytes);
int bs_ensure_plan(bs_sim* s, int64_t bytes);
// Pinned host region for one upload of `bytes`; call bs_stage_done after queuing the copy.
char* bs_stage(bs_sim* s, size_t bytes);
void bs_stage_done(bs_sim* s);
// Release the capture arena (the graph that read it is gone).
void bs_arena_release(bs_sim* s);
int bs_vec_bits(const bs_sim* s);

// ---- lowering (bs_plan.cpp)
// Convert a gate (reference convention flags) into canonical HostGate(s) on the
// vector's endian bits.  For DM, returns the column-side U and row-side conj(U).
int bs_lower_gate(bs_sim* s, const double* matrix, int k, const int* targets, int nc,
                  const int* controls, const int* cvals, unsigned flags, bool dm_superop,
                  std::vector<HostGate>& out);
int bs_lower_kraus_physical(bs_sim* s, const double* kraus, int nk, int k, const int* targets,
                            unsigned flags, std::vector<HostGate>& out);
// The gates are moved into the sweeps (the input is left with moved-from gates).
void bs_plan_sweeps(std::vector<HostGate>& gates, int n_bits, int tile_bits, std::vector<Sweep>& out);
// Tuned values of a handle (its setting, else the environment, else the default)
int bs_tile_bits(const bs_sim* s);
int bs_tile_threads(const bs_sim* s);
bool bs_tc_enabled(const bs_sim* s);
int bs_tc_min_bits(const bs_sim* s);
double bs_tc_cost(const bs_sim* s);

// ---- tensor-core fusion (bs_fuse.cpp)
// Fold runs of in-tile gates into kind-4 HostGates (5 endian bits, 32x32 matrix) where that is cheaper
// (float-float cost above `threshold`).  local[e]: tile position of endian bit e or -1.
void bs_fuse_tc(const std::vector<HostGate>& in, const int* local, int T, double threshold, std::vector<HostGate>& out);
void bs_fuse_small(const std::vector<HostGate>& in, const int* local, double pass, int maxk, std::vector<HostGate>& out);
// Smallest eu with every entry of the n_mat 32x32 matrices below 2^eu; false if not finite or above 2^12.
bool bs_tc_exponent(const double* mat, int n_mat, int& eu);

// ---- execution (bs_tile.cu)
int bs_run_sweeps(bs_sim* s, const std::vector<Sweep>& sweeps);
// BS_ERR_TIMEOUT if a tensor-core sweep since the last check gave up on a bounded wait
int bs_check_device_flag(bs_sim* s);
// After the stream has synchronised: add the device time of the recorded tensor-core launches to stats.tc_ms
void bs_collect_tc_time(bs_sim* s);

// ---- reference-compat Kraus (bs_dm.cu)
int bs_kraus_reference(bs_sim* s, const double* kraus, int nk, int k, const int* targets,
                       unsigned flags);
// The same channel (1 or 2 targets) as a kind-5 HostGate applied inside a sweep.
int bs_lower_kraus_reference(bs_sim* s, const double* kraus, int nk, int k, const int* targets, unsigned flags,
                             std::vector<HostGate>& out);

// ---- parallel alias table (bs_alias_par.cu)
int64_t bs_alias_parallel_scratch(int64_t n);
int bs_alias_parallel(bs_sim* s, const double* dprobs, int64_t n, double wsum, double* ap, int64_t* alias, void* work);

// ---- small state vectors in one CTA (bs_tile.cu, bs_sample.cu)
// bs_small_launch: |0...0>, the packed plan's gates, the state written back, its probabilities into
// dprobs and `shots` draws of bs_sample's generator with `seed` into dsamples, in one launch (dprobs
// and dsamples: device addresses, mapped host memory included); at its end the kernel writes `ticket`
// into *done (a host-mapped word, may be null) once every result is visible to the host.  io (may be
// null): host-mapped memory for the plan (written at hplan, read by the kernel at dplan, when it fits
// in plan_cap bytes; otherwise the plan is uploaded) and for the kernel's start and end times
// (globaltimer nanoseconds, at dtimes[0] and dtimes[1]).
struct SmallIO {
    char* hplan;
    char* dplan;
    size_t plan_cap;
    int64_t* dtimes;
};
// Pack the planned sweeps of a small run; BS_ERR_UNSUPPORTED (nothing packed) when a gate has no in-tile
// kernel or the state is not a complex128 state vector of at most 12 qubits.
int bs_small_pack(const bs_sim* s, const std::vector<Sweep>& sweeps, SmallPlan& out);
int bs_small_launch(bs_sim* s, const SmallPlan& plan, double* dprobs, int64_t shots, uint64_t seed,
                    int64_t* dsamples, int64_t* done, int64_t ticket, const SmallIO* io);
