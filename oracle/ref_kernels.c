/*
 * ORACLE — test infrastructure only.  CPU FP64 restatement of the reference
 * BraketSimulator.jl state-vector / density-matrix kernels, written so that the
 * GPU product can be checked against the reference's exact index conventions.
 * Only tests/, the smoke check and bench.py's CPU-baseline leg may load this.
 *
 * Every kernel below follows one reference function (cited file:line, paths
 * relative to the BraketSimulator.jl project).  Index conventions are kept
 * exactly, including the ones that differ between kernels:
 *   - qubit q <-> bit (n-1-q) of the basis index ("endian_qubits",
 *     src/gate_kernels.jl:193-206);
 *   - 2-target gate matrices: matrix index bit0 <-> t1, bit1 <-> t2
 *     (src/gate_kernels.jl:555-571);
 *   - >=3-target matrices: matrix index bit k <-> k-th smallest endian bit,
 *     whatever the order of the targets (src/gate_kernels.jl:759-767);
 *   - 2-target Kraus on rho: matrix index bit1 <-> t1, bit0 <-> t2
 *     (src/noise_kernels.jl:144-158);
 *   - Kraus kernels touch only the blocks of rho whose row and column share all
 *     non-target bits (src/noise_kernels.jl:111-132,141-167,181-195).
 * Matrices are passed row-major as interleaved complex doubles.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

/* Threads only from 2^17 amplitudes: the reference's sweeps run in chunks of 2^16 pairs
 * (src/gate_kernels.jl:489-537), so a small state is one chunk on one thread. */
#define ORC_PAR_MIN ((int64_t)1 << 17)

/* src/gate_kernels.jl:34-38 */
static inline int64_t pad_bit(int64_t ix, int bit) {
    int64_t left = (ix >> bit) << bit;
    int64_t right = ix - left;
    return (left << 1) ^ right;
}
/* src/gate_kernels.jl:78-84 (bits applied in the order given) */
static inline int64_t pad_bits(int64_t ix, const int* bits, int nb) {
    for (int i = 0; i < nb; i++) ix = pad_bit(ix, bits[i]);
    return ix;
}
/* src/gate_kernels.jl:119-121 */
static inline int64_t flip_bit(int64_t ix, int bit) { return ix ^ ((int64_t)1 << bit); }

static int log2i(int64_t n) { int k = 0; while (((int64_t)1 << k) < n) k++; return k; }

static void sort_ints(int* a, int n) {
    for (int i = 1; i < n; i++) { int v = a[i], j = i - 1; while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; j--; } a[j + 1] = v; }
}

/* 1-target dense/diagonal gate, src/gate_kernels.jl:489-537.
 * new_lo = m00*lo + m01*hi, new_hi = m10*lo + m11*hi. */
void orc_apply_1q(cplx* psi, int64_t n_amps, const cplx* m, int qubit) {
    int nq = log2i(n_amps);
    int e = nq - 1 - qubit;
    int64_t flipper = (int64_t)1 << e;
    cplx g00 = m[0], g01 = m[1], g10 = m[2], g11 = m[3];
#pragma omp parallel for schedule(static) if (n_amps >= ORC_PAR_MIN)
    for (int64_t t = 0; t < n_amps / 2; t++) {
        int64_t lo = pad_bit(t, e), hi = lo + flipper;
        cplx a = psi[lo], b = psi[hi];
        psi[lo] = g00 * a + g01 * b;
        psi[hi] = g10 * a + g11 * b;
    }
}

/* 2-target dense/diagonal gate, src/gate_kernels.jl:540-576. */
void orc_apply_2q(cplx* psi, int64_t n_amps, const cplx* m, int t1, int t2) {
    int nq = log2i(n_amps);
    int e1 = nq - 1 - t1, e2 = nq - 1 - t2;
    int b[2] = { e1 < e2 ? e1 : e2, e1 < e2 ? e2 : e1 };
#pragma omp parallel for schedule(static) if (n_amps >= ORC_PAR_MIN)
    for (int64_t ix = 0; ix < n_amps / 4; ix++) {
        int64_t i00 = pad_bits(ix, b, 2);
        int64_t i10 = flip_bit(i00, e2);
        int64_t i01 = flip_bit(i00, e1);
        int64_t i11 = flip_bit(i10, e1);
        int64_t idx[4] = { i00, i01, i10, i11 };
        cplx a[4], r[4];
        for (int j = 0; j < 4; j++) a[j] = psi[idx[j]];
        for (int i = 0; i < 4; i++) { r[i] = 0; for (int j = 0; j < 4; j++) r[i] += m[4 * i + j] * a[j]; }
        for (int j = 0; j < 4; j++) psi[idx[j]] = r[j];
    }
}

/* 1 control, 1 target, src/gate_kernels.jl:579-606. */
void orc_apply_c1t1(cplx* psi, int64_t n_amps, const cplx* m, int cbit, int control, int target) {
    int nq = log2i(n_amps);
    int ec = nq - 1 - control, et = nq - 1 - target;
    int small = ec < et ? ec : et, big = ec < et ? et : ec;
    cplx g00 = m[0], g01 = m[1], g10 = m[2], g11 = m[3];
#pragma omp parallel for schedule(static) if (n_amps >= ORC_PAR_MIN)
    for (int64_t ix = 0; ix < n_amps / 4; ix++) {
        int64_t i00 = pad_bit(pad_bit(ix, small), big);
        int64_t i10 = flip_bit(i00, ec);
        int64_t i01 = flip_bit(i00, et);
        int64_t i11 = flip_bit(i01, ec);
        int64_t lo = cbit ? i10 : i00, hi = cbit ? i11 : i01;
        cplx a = psi[lo], b = psi[hi];
        psi[lo] = g00 * a + g01 * b;
        psi[hi] = g10 * a + g11 * b;
    }
}

/* 1 control, 2 targets, src/gate_kernels.jl:608-636. */
void orc_apply_c1t2(cplx* psi, int64_t n_amps, const cplx* m, int cbit, int control, int t1, int t2) {
    int nq = log2i(n_amps);
    int ec = nq - 1 - control, e1 = nq - 1 - t1, e2 = nq - 1 - t2;
    int b[3] = { ec, e1, e2 };
    sort_ints(b, 3);
    for (int64_t ix = 0; ix < n_amps / 8; ix++) {
        int64_t i00 = pad_bits(ix, b, 3);
        if (cbit) i00 = flip_bit(i00, ec);
        int64_t i10 = flip_bit(i00, e2);
        int64_t i01 = flip_bit(i00, e1);
        int64_t i11 = flip_bit(i01, e2);
        int64_t idx[4] = { i00, i01, i10, i11 };
        cplx a[4], r[4];
        for (int j = 0; j < 4; j++) a[j] = psi[idx[j]];
        for (int i = 0; i < 4; i++) { r[i] = 0; for (int j = 0; j < 4; j++) r[i] += m[4 * i + j] * a[j]; }
        for (int j = 0; j < 4; j++) psi[idx[j]] = r[j];
    }
}

/* 2 controls, 1 target, src/gate_kernels.jl:638-670. */
void orc_apply_c2t1(cplx* psi, int64_t n_amps, const cplx* m, int c1bit, int c2bit, int c1, int c2, int target) {
    int nq = log2i(n_amps);
    int e1 = nq - 1 - c1, e2 = nq - 1 - c2, et = nq - 1 - target;
    int b[3] = { e1, e2, et };
    sort_ints(b, 3);
    cplx g00 = m[0], g01 = m[1], g10 = m[2], g11 = m[3];
    for (int64_t ix = 0; ix < n_amps / 8; ix++) {
        int64_t lo = pad_bits(ix, b, 3);
        if (c1bit) lo = flip_bit(lo, e1);
        if (c2bit) lo = flip_bit(lo, e2);
        int64_t hi = flip_bit(lo, et);
        cplx a = psi[lo], bb = psi[hi];
        psi[lo] = g00 * a + g01 * bb;
        psi[hi] = g10 * a + g11 * bb;
    }
}

/* Generic k-target gate (k >= 3), src/gate_kernels.jl:753-775.
 * Matrix index bit k <-> k-th smallest endian target bit. */
void orc_apply_nq(cplx* psi, int64_t n_amps, const cplx* m, int k, const int* targets) {
    int nq = log2i(n_amps);
    int ord[32];
    for (int i = 0; i < k; i++) ord[i] = nq - 1 - targets[i];
    sort_ints(ord, k);
    int64_t dim = (int64_t)1 << k;
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * dim);
    cplx* a = (cplx*)malloc(sizeof(cplx) * dim);
    for (int64_t ix = 0; ix < n_amps / dim; ix++) {
        int64_t p = pad_bits(ix, ord, k);
        for (int64_t j = 0; j < dim; j++) {
            int64_t f = p;
            for (int b = 0; b < k; b++) if ((j >> b) & 1) f = flip_bit(f, ord[b]);
            idx[j] = f;
            a[j] = psi[f];
        }
        for (int64_t i = 0; i < dim; i++) {
            cplx s = 0;
            for (int64_t j = 0; j < dim; j++) s += m[i * dim + j] * a[j];
            psi[idx[i]] = s;
        }
    }
    free(idx); free(a);
}

/* DoubleExcitation two-amplitude kernel, src/custom_gates.jl:390-414.
 * half_angle = angle * pow_exponent / 2. */
void orc_apply_double_excitation(cplx* psi, int64_t n_amps, double half_angle, const int* t) {
    int nq = log2i(n_amps);
    int e[4], ord[4];
    for (int i = 0; i < 4; i++) { e[i] = nq - 1 - t[i]; ord[i] = e[i]; }
    sort_ints(ord, 4);
    double s = sin(half_angle), c = cos(half_angle);
    for (int64_t ix = 0; ix < n_amps / 16; ix++) {
        int64_t p = pad_bits(ix, ord, 4);
        int64_t i0011 = flip_bit(flip_bit(p, e[2]), e[3]);
        int64_t i1100 = flip_bit(flip_bit(p, e[0]), e[1]);
        cplx a = psi[i0011], b = psi[i1100];
        psi[i0011] = c * a - s * b;
        psi[i1100] = s * a + c * b;
    }
}

/* ---------------- density matrix (column-major, rho[r + c*dim]) ---------------- */

/* PhaseFlip elementwise kernel, src/noise_kernels.jl:7-23 (updates every element). */
void orc_dm_phase_flip(cplx* rho, int64_t dim, double p, int qubit) {
    int nq = log2i(dim);
    int e = nq - 1 - qubit;
    for (int64_t idx = 0; idx < dim * dim; idx++) {
        int64_t ix = idx % dim, jx = idx / dim;
        double iv = 1.0 - 2.0 * (double)((ix >> e) & 1), jv = 1.0 - 2.0 * (double)((jx >> e) & 1);
        double factor = (1.0 - p) + iv * jv * p;
        rho[ix + jx * dim] *= factor;
    }
}

/* sum_k K rho_blk K^dagger on a dim_k x dim_k block gathered at rows/cols idx[] */
static void kraus_block(cplx* rho, int64_t dim, const int64_t* idx, int64_t dk, const cplx* K, int nk, cplx* blk, cplx* tmp, cplx* acc) {
    for (int64_t i = 0; i < dk; i++) for (int64_t j = 0; j < dk; j++) blk[i * dk + j] = rho[idx[i] + idx[j] * dim];
    for (int64_t x = 0; x < dk * dk; x++) acc[x] = 0;
    for (int q = 0; q < nk; q++) {
        const cplx* Kq = K + (int64_t)q * dk * dk;
        for (int64_t i = 0; i < dk; i++) for (int64_t j = 0; j < dk; j++) {
            cplx s = 0; for (int64_t l = 0; l < dk; l++) s += Kq[i * dk + l] * blk[l * dk + j]; tmp[i * dk + j] = s;
        }
        for (int64_t i = 0; i < dk; i++) for (int64_t j = 0; j < dk; j++) {
            cplx s = 0; for (int64_t l = 0; l < dk; l++) s += tmp[i * dk + l] * conj(Kq[j * dk + l]); acc[i * dk + j] += s;
        }
    }
    for (int64_t i = 0; i < dk; i++) for (int64_t j = 0; j < dk; j++) rho[idx[i] + idx[j] * dim] = acc[i * dk + j];
}

/* 1-target Kraus, src/noise_kernels.jl:105-133 (block-diagonal update). */
void orc_dm_kraus_1q(cplx* rho, int64_t dim, const cplx* K, int nk, int qubit) {
    int nq = log2i(dim);
    int e = nq - 1 - qubit;
    cplx blk[4], tmp[4], acc[4];
    for (int64_t ix = 0; ix < dim / 2; ix++) {
        int64_t lo = pad_bit(ix, e);
        int64_t idx[2] = { lo, flip_bit(lo, e) };
        kraus_block(rho, dim, idx, 2, K, nk, blk, tmp, acc);
    }
}

/* 2-target Kraus, src/noise_kernels.jl:135-168: order (00, t2 flipped, t1 flipped, 11). */
void orc_dm_kraus_2q(cplx* rho, int64_t dim, const cplx* K, int nk, int t1, int t2) {
    int nq = log2i(dim);
    int e1 = nq - 1 - t1, e2 = nq - 1 - t2;
    int b[2] = { e1 < e2 ? e1 : e2, e1 < e2 ? e2 : e1 };
    cplx blk[16], tmp[16], acc[16];
    for (int64_t ix = 0; ix < dim / 4; ix++) {
        int64_t p = pad_bits(ix, b, 2);
        int64_t idx[4] = { p, flip_bit(p, e2), flip_bit(p, e1), flip_bit(flip_bit(p, e1), e2) };
        kraus_block(rho, dim, idx, 4, K, nk, blk, tmp, acc);
    }
}

/* k-target Kraus (k >= 3), src/noise_kernels.jl:170-196. */
void orc_dm_kraus_nq(cplx* rho, int64_t dim, const cplx* K, int nk, int k, const int* targets) {
    int nq = log2i(dim);
    int ord[32];
    for (int i = 0; i < k; i++) ord[i] = nq - 1 - targets[i];
    sort_ints(ord, k);
    int64_t dk = (int64_t)1 << k;
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * dk);
    cplx* blk = (cplx*)malloc(sizeof(cplx) * dk * dk * 3);
    for (int64_t ix = 0; ix < dim / dk; ix++) {
        int64_t p = pad_bits(ix, ord, k);
        for (int64_t j = 0; j < dk; j++) {
            int64_t f = p;
            for (int bb = 0; bb < k; bb++) if ((j >> bb) & 1) f = flip_bit(f, ord[bb]);
            idx[j] = f;
        }
        kraus_block(rho, dim, idx, dk, K, nk, blk, blk + dk * dk, blk + 2 * dk * dk);
    }
    free(idx); free(blk);
}

/* Physically complete channel (not in the reference): S' = sum_k conj(K) S K^T on the
 * stored matrix S, which is the convention the reference's gate path uses for S
 * (src/dm_simulator.jl:130-140).  Matrix index bit j <-> targets[j].  Written as the
 * superoperator M[(r,c),(a,b)] = sum_q conj(K_q[r,a]) K_q[c,b] applied to every dk x dk
 * block of S whose row and column share their non-target bits (blocks are disjoint, so the
 * update is in place and parallel over blocks). */
static inline int64_t dep_bits(int64_t x, const int* e, int k) {
    int64_t g = 0;
    for (int i = 0; i < k; i++) g |= ((x >> i) & 1) << e[i];
    return g;
}
void orc_dm_kraus_full(cplx* rho, int64_t dim, const cplx* K, int nk, int k, const int* targets) {
    int nq = log2i(dim);
    int64_t dk = (int64_t)1 << k, dk2 = dk * dk;
    int e[32];
    int sorted[32];
    for (int i = 0; i < k; i++) { e[i] = nq - 1 - targets[i]; sorted[i] = e[i]; }
    sort_ints(sorted, k);
    cplx* M = (cplx*)malloc(sizeof(cplx) * (size_t)(dk2 * dk2));
    for (int64_t r = 0; r < dk; r++) for (int64_t c = 0; c < dk; c++)
        for (int64_t a = 0; a < dk; a++) for (int64_t b = 0; b < dk; b++) {
            cplx w = 0;
            for (int q = 0; q < nk; q++) {
                const cplx* Kq = K + (int64_t)q * dk2;
                w += conj(Kq[r * dk + a]) * Kq[c * dk + b];
            }
            M[(r * dk + c) * dk2 + a * dk + b] = w;
        }
    const int64_t nb = dim >> k;   /* row (and column) bases */
#pragma omp parallel for schedule(static) if (nb * nb >= 64)
    for (int64_t ib = 0; ib < nb * nb; ib++) {
        int64_t rb = pad_bits(ib % nb, sorted, k), cb = pad_bits(ib / nb, sorted, k);
        cplx v[1024], o[1024];   /* dk <= 32 */
        for (int64_t a = 0; a < dk; a++)
            for (int64_t b = 0; b < dk; b++) v[a * dk + b] = rho[(rb | dep_bits(a, e, k)) + (cb | dep_bits(b, e, k)) * dim];
        for (int64_t x = 0; x < dk2; x++) {
            const cplx* Mx = M + x * dk2;
            cplx s = 0;
            for (int64_t y = 0; y < dk2; y++) s += Mx[y] * v[y];
            o[x] = s;
        }
        for (int64_t r = 0; r < dk; r++)
            for (int64_t c = 0; c < dk; c++) rho[(rb | dep_bits(r, e, k)) + (cb | dep_bits(c, e, k)) * dim] = o[r * dk + c];
    }
    free(M);
}

/* ---------------- sampling ---------------- */

/* Julia Base.sum on a Float64 vector is pairwise above 1024 elements; below that
 * the leaf is an @simd loop whose association LLVM chooses.  The leaf here is a
 * plain left fold, so wsum matches the reference to within rounding; tests pass
 * the same wsum to both sides when they compare bit-for-bit. */
static double pairwise(const double* x, int64_t n) {
    if (n <= 1024) { double s = 0; for (int64_t i = 0; i < n; i++) s += x[i]; return s; }
    int64_t h = n >> 1;
    return pairwise(x, h) + pairwise(x + h, n - h);
}
double orc_pairwise_sum(const double* x, int64_t n) { return pairwise(x, n); }

/* Alias table, src/result_types.jl:8-54 (same LIFO push/pop order, same
 * acceptance update).  alias[] holds 0-based indices; entries never assigned stay -1. */
void orc_make_alias_table(const double* w, int64_t n, double wsum, double* ap, int64_t* alias, int64_t* larges, int64_t* smalls) {
    double ac = (double)n / wsum;
    for (int64_t i = 0; i < n; i++) { ap[i] = w[i] * ac; alias[i] = -1; }
    int64_t kl = 0, ks = 0;
    for (int64_t i = 0; i < n; i++) {
        double ai = ap[i];
        if (ai > 1.0) larges[kl++] = i;
        else if (ai < 1.0) smalls[ks++] = i;
    }
    while (kl > 0 && ks > 0) {
        int64_t s = smalls[--ks];
        int64_t l = larges[--kl];
        alias[s] = l;
        volatile double t = ap[l] - 1.0;   /* keep the reference's two roundings */
        double al = ap[l] = t + ap[s];
        if (al > 1.0) larges[kl++] = l;
        else smalls[ks++] = l;
    }
    for (int64_t i = 0; i < ks; i++) ap[smalls[i]] = 1.0;
}

/* Alias draw, src/result_types.jl:68-72, on a supplied stream:
 * j[s] in 0..n-1 plays rand(rng, sampler) - 1 and u[s] in [0,1) plays rand(rng). */
void orc_sample_alias(const double* ap, const int64_t* alias, const int64_t* j, const double* u, int64_t shots, int64_t* out) {
    for (int64_t s = 0; s < shots; s++) out[s] = (u[s] < ap[j[s]]) ? j[s] : alias[j[s]];
}

/* Direct sampling for >= 30 qubits, src/result_types.jl:73-77, via StatsBase 0.34
 * sample(rng, wv::AbstractWeights): t = rand()*sum(wv); linear scan of the running
 * sum until cw >= t.  Returns 0-based indices. */
void orc_sample_direct(const double* w, int64_t n, double wsum, const double* u, int64_t shots, int64_t* out) {
    for (int64_t s = 0; s < shots; s++) {
        double t = u[s] * wsum;
        int64_t i = 0;
        double cw = w[0];
        while (cw < t && i < n - 1) { i++; cw += w[i]; }
        out[s] = i;
    }
}

/* ---------------- Pauli expectations in one pass ---------------- */

/* <psi|P|psi> for a Pauli string P, evaluated in one read of psi.  The reference
 * computes the same number by applying the observable's gates to a copy of psi and
 * taking real(dot(psi, copy)) (src/sv_simulator.jl:240-248, src/result_types.jl:196-221);
 * a Pauli string acts on basis state i as
 *   (P psi)_i = (-i)^{#Y} (-1)^{popcount(i & zidx)} psi_{i ^ xidx},
 * with xidx / zidx the index bits of the X-or-Y / Z-or-Y factors (qubit q <-> bit n-1-q).
 * Used for the oracle's parameter-shift gradients, where the apply-then-dot form would
 * cost one sweep per factor per term. */
double orc_expect_pauli(const cplx* psi, int64_t n_amps, uint64_t xidx, uint64_t zidx, int n_y) {
    double re = 0.0, im = 0.0;
#pragma omp parallel for reduction(+:re, im) schedule(static) if (n_amps >= ORC_PAR_MIN)
    for (int64_t i = 0; i < n_amps; i++) {
        cplx v = conj(psi[i]) * psi[i ^ (int64_t)xidx];
        if (__builtin_popcountll((uint64_t)i & zidx) & 1) v = -v;
        re += creal(v);
        im += cimag(v);
    }
    /* multiply by (-i)^{n_y} and keep the real part */
    switch (n_y & 3) {
        case 0: return re;
        case 1: return im;      /* (-i)(re + i im) = im - i re */
        case 2: return -re;
        default: return -im;    /* (i)(re + i im) = -im + i re */
    }
}
