/*
 * braket_gb300.h — C ABI of the GB300 state-vector / density-matrix engine.
 *
 * One handle (bs_sim) owns one quantum state resident in GPU memory: a state
 * vector psi of 2^n complex amplitudes, or a density matrix stored column-major
 * as the reference stores it (element S[r, c] at r + c*2^n).  Basis index bit
 * (n-1-q) belongs to qubit q, so qubit 0 is the most significant bit.
 *
 * Each entry point names the reference function it replaces (file:line inside
 * the BraketSimulator.jl project).  All calls return a status code (BS_OK == 0);
 * on failure bs_last_error() describes the cause.  Host buffers are borrowed for
 * the duration of a call; nothing is kept.  A handle is not re-entrant, distinct
 * handles may be used from distinct host threads (each handle owns its stream).
 */
#ifndef BRAKET_GB300_H
#define BRAKET_GB300_H
#include <stdint.h>
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BS_OK                0
#define BS_ERR_INVALID_ARG   1
#define BS_ERR_CUDA          2
#define BS_ERR_ALLOC         3
#define BS_ERR_STATE         4
#define BS_ERR_UNSUPPORTED   5
#define BS_ERR_TIMEOUT       6
#define BS_ERR_IO            7

/* handle kinds and state precision */
#define BS_KIND_SV           0   /* StateVectorSimulator   (src/sv_simulator.jl:6-42) */
#define BS_KIND_DM           1   /* DensityMatrixSimulator (src/dm_simulator.jl:6-40) */
#define BS_PREC_C128         0   /* complex128 state, float-float arithmetic (~2^-46 per op) */
#define BS_PREC_C64          1   /* complex64 state, FP32 arithmetic, FP64-accurate reductions */

/* gate flags */
#define BS_GATE_DIAGONAL        0x01u /* matrix holds the 2^k diagonal entries only */
#define BS_GATE_CONJ            0x02u /* apply conj(U) instead of U (reference Val{true} path) */
#define BS_GATE_SORTED_TARGETS  0x04u /* matrix bit j <-> j-th largest target qubit (reference >=3-target kernels) */
#define BS_GATE_MSB_FIRST       0x08u /* matrix bit (k-1-j) <-> targets[j] (big-endian) */
/* default (no convention flag): matrix index bit j <-> targets[j] */

/* noise modes */
#define BS_NOISE_REFERENCE      0x00u /* reproduce the reference's block-diagonal Kraus update */
#define BS_NOISE_PHYSICAL       0x10u /* full channel S <- sum conj(K) S K^T on every element */

/* sampling flags */
#define BS_ALIAS_EXACT          0x0u  /* bit-exact restatement of the reference's serial table */
#define BS_ALIAS_PARALLEL       0x1u  /* parallel construction: same distribution, different table */

#define BS_MAX_TARGETS   10
#define BS_MAX_CONTROLS  16

typedef struct bs_sim bs_sim;

/* One instruction of an operation list.
 *  kind 0 = gate: matrix is 2^k x 2^k row-major (or 2^k diagonal), interleaved (re, im).
 *  kind 1 = Kraus channel: n_matrices matrices of 2^k x 2^k, back to back.
 *  kind 2 = no-op (Measure / Barrier / Reset / Delay, src/dm_simulator.jl:154-157). */
typedef struct bs_op {
    int32_t kind;
    uint32_t flags;
    int32_t n_targets;
    int32_t n_controls;
    int32_t targets[BS_MAX_TARGETS];
    int32_t controls[BS_MAX_CONTROLS];
    int32_t control_values[BS_MAX_CONTROLS];
    int32_t n_matrices;
    int32_t reserved;
    const double* matrix;
} bs_op;

/* Per-handle counters for the last evolve call. */
typedef struct bs_stats {
    int64_t sweeps;            /* full passes over the state */
    int64_t kernel_launches;   /* kernels launched */
    int64_t gates;             /* gates applied */
    double  bytes_moved;       /* algorithmic HBM bytes of the executed sweeps */
    double  gpu_ms;            /* device time of the call (CUDA events) */
    int64_t tc_gates;          /* fused unitaries applied on the tensor cores (each replacing a run of gates) */
    int64_t tc_launches;       /* tensor-core sweep kernel launches */
    double  tc_ms;             /* their device time (CUDA events around each launch, same stream) */
} bs_stats;

/* ---- lifecycle: StateVectorSimulator(T, n, shots) / DensityMatrixSimulator(T, n, shots)
 *      (src/sv_simulator.jl:53-68, src/dm_simulator.jl:50-65), reinit! (src/sv_simulator.jl:96-127,
 *      src/dm_simulator.jl:96-128).  The state starts as |0...0> (psi[0] = 1 / S[0,0] = 1). */
int bs_create(int kind, int n_qubits, int precision, bs_sim** out);
int bs_destroy(bs_sim* sim);
int bs_reinit(bs_sim* sim, int n_qubits);
int bs_qubit_count(const bs_sim* sim, int* out);
const char* bs_last_error(const bs_sim* sim);
const char* bs_version(void);

/* ---- state transfer: state_vector / density_matrix / setters
 *      (src/sv_simulator.jl:150-152, src/dm_simulator.jl:261).
 *      n_elems = 2^n (SV) or 4^n (DM) complex elements, interleaved doubles. */
int bs_set_state(bs_sim* sim, const double* host, int64_t n_elems);
int bs_get_state(bs_sim* sim, double* host, int64_t n_elems);
/* device-resident variants (pointer to interleaved complex128 on the handle's GPU) */
int bs_set_state_device(bs_sim* sim, const void* dev, int64_t n_elems);
int bs_get_state_device(bs_sim* sim, void* dev, int64_t n_elems);
int bs_copy_state(bs_sim* dst, const bs_sim* src);       /* copyto! (src/sv_simulator.jl:88-94) */

/* ---- gates: apply_gate!(g, psi, targets...) and the dispatch that picks a kernel
 *      (src/gate_kernels.jl:489-775, src/custom_gates.jl:364-416).
 *      SV: psi <- C(U) psi, where C(U) applies U on the targets when every control
 *      qubit c_i has value control_values[i].
 *      DM: S <- conj(C(U)) S C(U)^T, the two sweeps of _evolve_op! fused into one
 *      (src/dm_simulator.jl:130-140). */
int bs_apply_gate(bs_sim* sim, const double* matrix, int n_targets, const int* targets,
                  int n_controls, const int* controls, const int* control_values, unsigned flags);

/* DM only: one reference apply_gate! call on vec(S) viewed as a 2n-qubit vector
 * (targets in 0..2n-1).  Used to mirror apply_gate!(Val{conj}, op, vec(S), t...) exactly. */
int bs_dm_apply_vec_gate(bs_sim* sim, const double* matrix, int n_targets, const int* targets,
                         int n_controls, const int* controls, const int* control_values, unsigned flags);

/* ---- noise: apply_noise!(kraus, rho, targets...) (src/noise_kernels.jl:102-196).
 *      flags: BS_NOISE_REFERENCE or BS_NOISE_PHYSICAL plus a target convention flag. */
int bs_apply_kraus(bs_sim* sim, const double* kraus, int n_kraus, int n_targets, const int* targets,
                   unsigned flags);

/* ---- evolve!: apply an instruction list (src/sv_simulator.jl:140-148,
 *      src/dm_simulator.jl:170-179).  Gates are fused into shared-memory tiles. */
int bs_evolve(bs_sim* sim, const bs_op* ops, int64_t n_ops, unsigned noise_mode);
int bs_last_stats(const bs_sim* sim, bs_stats* out);

/* ---- simulate of one small circuit (src/BraketSimulator.jl:307-322: reinit!, evolve!, then the
 *      results) in one round trip: the state is reset to |0...0>, the ops are applied, and
 *      probs_out (2^n doubles, may be null) and samples_out (shots basis indices, bs_sample's
 *      generator with this seed) are filled.  The handle keeps the final state, as after
 *      bs_reinit + bs_evolve.  State vectors of at most 12 qubits (complex128 runs in one CTA that
 *      reads the plan from and writes the results into host-mapped memory, and the host polls a
 *      completion word instead of synchronising; other cases take the usual kernels with the same
 *      results).  bs_last_stats then reports the kernel's own device time. */
int bs_run_small(bs_sim* sim, const bs_op* ops, int64_t n_ops, int64_t shots, uint64_t seed, double* probs_out,
                 int64_t* samples_out);

/* ---- probabilities (src/sv_simulator.jl:271, src/dm_simulator.jl:262) */
int bs_probabilities(bs_sim* sim, double* host_out, int64_t n);
/* marginal_probability (src/result_types.jl:96-113): sum over the qubits not in targets,
 * output index bit (k-1-j) <-> targets[j] after the reference's sort of targets. */
int bs_marginal_probabilities(bs_sim* sim, int n_targets, const int* targets, double* host_out);

/* ---- expectations (src/sv_simulator.jl:240-248, src/dm_simulator.jl:253-260,
 *      src/result_types.jl:161-167,196-221).
 * Pauli strings: term t is coeffs[t] * prod_q P_q with P_q = X where x bit set and z unset,
 * Z where z set and x unset, Y where both set (bit q <-> qubit q).  out[t] = real expectation
 * of the whole term (coefficient included); one fused read of the state for all terms. */
int bs_expectation_pauli(bs_sim* sim, int n_terms, const uint64_t* xmask, const uint64_t* zmask,
                         const double* coeffs, double* out);
/* Hermitian matrix observable on k targets (reference convention flags as for gates). */
int bs_expectation_matrix(bs_sim* sim, const double* matrix, int n_targets, const int* targets,
                          unsigned flags, double* out);

/* ---- sampling (src/result_types.jl:8-80).
 * bs_alias_build: build the alias table from the current probabilities.  wsum <= 0 lets the
 * library compute sum(p); pass the reference's wsum for a bit-exact table.
 * bs_sample_alias: out[s] = u[s] < ap[j[s]] ? j[s] : alias[j[s]] on a supplied stream.
 * bs_sample_direct: StatsBase inverse-CDF draw used by the reference at >= 30 qubits.
 * bs_sample: draws with the library's own counter-based generator (seeded). */
int bs_alias_build(bs_sim* sim, double wsum, unsigned flags);
/* same table from a supplied probability vector (the reference's own weights) */
int bs_alias_build_from(bs_sim* sim, const double* probs, int64_t n, double wsum);
int bs_alias_table(bs_sim* sim, double* ap_out, int64_t* alias_out, int64_t n);
int bs_sample_alias(bs_sim* sim, const int64_t* j, const double* u, int64_t shots, int64_t* out);
int bs_sample_direct(bs_sim* sim, const double* u, int64_t shots, double wsum, int64_t* out);
int bs_sample(bs_sim* sim, uint64_t seed, int64_t shots, int64_t* out);

/* ---- adjoint differentiation (no reference counterpart: the reference declares
 * AdjointGradient in src/results.jl:90-159 but rejects it, src/pragmas.jl:67-68).
 * ops: a parameterised circuit; param_index[i] >= 0 marks op i as exp(-i theta G/2) with
 * generator given by gen_xmask/gen_zmask (Pauli string, Rx/Ry/Rz/XX/YY/ZZ) or as a
 * PhaseShift when gen_kind[i] == 1.  H = sum_t coeffs[t] P_t.  Writes <H> and dE/dtheta_p. */
int bs_adjoint_gradient(bs_sim* sim, const bs_op* ops, int64_t n_ops, const int32_t* param_index,
                        const int32_t* gen_kind, const uint64_t* gen_xmask, const uint64_t* gen_zmask,
                        int n_params, int n_terms, const uint64_t* xmask, const uint64_t* zmask,
                        const double* coeffs, double* energy_out, double* grad_out);

/* ---- allocation-free Pauli expectations.  No counterpart in the reference: it serves
 * callers that cannot allocate device memory when they need an expectation value (a runtime
 * that owns all of HBM through its own pool, a real-time loop that cannot afford the device
 * synchronisation of cudaMalloc/cudaFree).  Same terms and result as bs_expectation_pauli,
 * computed from a complex128 state the caller holds at state_dev (kind BS_KIND_SV: 2^n
 * amplitudes; BS_KIND_DM: the stored matrix, column-major 4^n elements), on `stream`
 * (a cudaStream_t, NULL for the default stream); `out` is host memory.
 * Scratch: one static 256 KiB device array inside the library, present on every GPU that
 * loads it until the process exits; no cudaMalloc/cudaFree or other allocation is made.
 * Limits: n_terms <= 32 and n_qubits <= 34 (SV) / 17 (DM); larger requests return
 * BS_ERR_UNSUPPORTED.  Every call looks up the array's device address on the current device
 * (cudaGetSymbolAddress, which allocates nothing, so the address stays right after a caller's
 * cudaDeviceReset); the first call on each device also loads the library's device code and
 * should come before any stream capture.  Every call reuses the same array, so calls that can
 * overlap on the GPU race and must be serialised by the caller. */
int bs_expectation_pauli_noalloc(const void* state_dev, int kind, int n_qubits, int n_terms,
                                 const uint64_t* xmask, const uint64_t* zmask, const double* coeffs,
                                 double* out, void* stream);

/* ---- reduced density matrix: partial_trace (src/sv_simulator.jl:273-318, src/dm_simulator.jl:280-323)
 * for the DensityMatrix result type (src/result_types.jl:239-246), computed on the device.
 * Keeps the n_keep (1..12) given qubits, traces out the rest; out = 2^k x 2^k complex128,
 * row-major, interleaved, with output index bit r <-> the r-th smallest kept endian bit (the
 * reference's loop order before its own final permutation of unsorted targets). */
int bs_reduced_density_matrix(bs_sim* sim, int n_keep, const int* qubits, double* out);

/* Large results written from the device straight to a file, in the reference's byte layout for
 * its memory-mapped result values (_mmap_large_result_values, src/BraketSimulator.jl:410-428:
 * `write(io, value)` of a Vector{ComplexF64} state vector or a Vector{Float64} probability
 * vector).  what = BS_FILE_STATE (state-vector simulators: 2^n complex128, interleaved) or
 * BS_FILE_PROBABILITIES (2^n float64; the diagonal for a density matrix).  Streams through two
 * 32 MiB pinned buffers; bytes_out (may be null) gets the file size.  BS_ERR_IO when the file
 * cannot be opened or written. */
#define BS_FILE_STATE          0
#define BS_FILE_PROBABILITIES  1
int bs_write_result_file(bs_sim* sim, int what, const char* path, int64_t* bytes_out);

/* ---- batched simulate (src/BraketSimulator.jl:347-395): n_circuits independent circuits, each
 * from |0...0> on n_qubits[c] qubits with ops[c][0..n_ops[c]).  Returns per circuit n_terms Pauli
 * expectations (term t of circuit c at xmask/zmask[c*n_terms + t], bit q <-> qubit q) and `shots`
 * basis-index samples.  Circuits of <= 12 qubits (complex64) run whole in one CTA each inside one
 * persistent launch; larger ones run as tile sweeps on a pool of streams.  No handle needed. */
int bs_run_batch(int n_circuits, const int* n_qubits, const bs_op* const* ops, const int64_t* n_ops,
                 int n_terms, const uint64_t* xmask, const uint64_t* zmask, int64_t shots, uint64_t seed,
                 int precision, double* expectations_out, int64_t* samples_out, bs_stats* stats_out);

/* ---- captured batches.  The same work as bs_run_batch (same results, same per-circuit shot
 * seeds), captured once into a CUDA graph and replayed: bs_batch_create runs the batch eagerly once
 * (sizing a pool of handles, 4 by default (BS_BATCH_STREAMS), circuits assigned largest-first), then captures every
 * upload, kernel and result copy of the batch into one graph; bs_batch_launch replays it and
 * copies the results out (host work per replay: one graph launch and two memcpy).
 * bs_batch_set_ops replaces every circuit's ops (same qubit counts; a circuit may not move
 * between the small-circuit kernel and the tile path), recaptures, and updates the executable
 * graph in place when its topology is unchanged (re-instantiates it otherwise) — the path for
 * parameter sweeps.  A replay repeats the same shot seeds.  No reference counterpart: the
 * reference's batch (src/BraketSimulator.jl:347-395) spawns Julia tasks per call. */
typedef struct bs_batch bs_batch;
int bs_batch_create(int n_circuits, const int* n_qubits, const bs_op* const* ops, const int64_t* n_ops,
                    int n_terms, const uint64_t* xmask, const uint64_t* zmask, int64_t shots, uint64_t seed,
                    int precision, bs_batch** out);
int bs_batch_set_ops(bs_batch* batch, const bs_op* const* ops, const int64_t* n_ops);
int bs_batch_launch(bs_batch* batch, double* expectations_out, int64_t* samples_out, bs_stats* stats_out);
int bs_batch_destroy(bs_batch* batch);

/* ---- per-handle tuning, set by the project's autotuner (braketsimulator_gb300.autotune) or by hand.
 * No reference counterpart (the reference has no tunable kernels).  A negative value restores
 * "environment variable, else built-in default"; bs_get_tuning returns the value in effect.
 *   BS_TUNE_TILE_BITS     10..12  amplitude bits per tile of the sweep kernels (BS_TILE_BITS)
 *   BS_TUNE_TILE_THREADS  256|512 threads per CTA of the float-float sweep (BS_TILE_THREADS)
 *   BS_TUNE_TC            0|1     fused tensor-core sweeps (BS_TC)
 *   BS_TUNE_TC_MIN_BITS   n       vector bits from which they are used (BS_TC_MIN_BITS, 22)
 *   BS_TUNE_TC_COST       x       fuse a block when its float-float cost (dense 1-qubit gates)
 *                                 exceeds x (BS_TC_COST, 2)
 *   BS_TUNE_ADJ_SEGMENTS  S >= 1  bs_adjoint_gradient: forward segments, psi kept after each of the
 *                                 first S-1 (checkpoints); default (-1) from the parameterised gate
 *                                 count and a quarter of the free memory, halved while allocation
 *                                 fails; 1 = pure uncomputation */
#define BS_TUNE_TILE_BITS     0
#define BS_TUNE_TILE_THREADS  1
#define BS_TUNE_TC            2
#define BS_TUNE_TC_MIN_BITS   3
#define BS_TUNE_TC_COST       4
#define BS_TUNE_ADJ_SEGMENTS  5
int bs_set_tuning(bs_sim* sim, int param, double value);
int bs_get_tuning(bs_sim* sim, int param, double* value);
/* n settings (params[i] = values[i]) on every handle of a captured batch, then one rebuild of its
 * graph (the batch keeps a copy of its circuits for this) */
int bs_batch_set_tuning(bs_batch* batch, int n, const int* params, const double* values);

/* synchronise the handle's stream; device pointer of the state (for in-HBM benchmarking) */
int bs_synchronize(bs_sim* sim);
/* Failure-detection self-test (no reference counterpart): one thread waits, with the tensor-core sweep's bounded mbarrier
 * wait, on a barrier that nothing completes, gives up after about `seconds` (0 < seconds <= 1) of
 * clock, and raises the handle's device flag.  Returns BS_ERR_TIMEOUT, as a sweep whose copy or MMA
 * never landed would; the handle stays usable.  Nothing faults or hangs. */
int bs_selftest_wait_timeout(bs_sim* sim, double seconds);
int bs_state_device_ptr(bs_sim* sim, void** out);

#ifdef __cplusplus
}
#endif
#endif
