// Host side of gate application: lowering of a reference-convention gate or
// channel into canonical gates on endian bits, and the fusion planner that packs
// consecutive gates into tile sweeps.
//
// Reference conventions mapped here (src/gate_kernels.jl):
//   1- and 2-target kernels: matrix bit j <-> targets[j]            (:489-576)
//   >= 3 targets: matrix bit j <-> j-th smallest endian bit         (:753-775)
//   density-matrix gate: U on the column bits of vec(S), conj(U) on the row bits
//   (src/dm_simulator.jl:130-140).
#include <algorithm>
#include <cmath>
#include <complex>
#include "bs_internal.h"

namespace {

using cd = std::complex<double>;

bool valid_qubits(int n, int k, const int* t, int nc, const int* c, const int* cv, std::string& why) {
    uint64_t seen = 0;
    for (int i = 0; i < k; i++) {
        if (t[i] < 0 || t[i] >= n) { why = "target qubit out of range"; return false; }
        if ((seen >> t[i]) & 1ULL) { why = "repeated qubit"; return false; }
        seen |= 1ULL << t[i];
    }
    for (int i = 0; i < nc; i++) {
        if (c[i] < 0 || c[i] >= n) { why = "control qubit out of range"; return false; }
        if ((seen >> c[i]) & 1ULL) { why = "repeated qubit"; return false; }
        seen |= 1ULL << c[i];
        if (cv && cv[i] != 0 && cv[i] != 1) { why = "control value must be 0 or 1"; return false; }
    }
    return true;
}

// canonical target order: bit j <-> ct[j]
void canonical_targets(int k, const int* targets, unsigned flags, int* ct) {
    for (int j = 0; j < k; j++) ct[j] = targets[j];
    if (flags & BS_GATE_SORTED_TARGETS) {
        std::sort(ct, ct + k, [](int a, int b) { return a > b; });   // largest qubit = smallest endian bit
    } else if (flags & BS_GATE_MSB_FIRST) {
        for (int j = 0; j < k; j++) ct[j] = targets[k - 1 - j];
    }
}

void classify(HostGate& g) {
    const int D = 1 << g.k;
    if (g.kind == 1) return;
    bool diag = true;
    for (int r = 0; r < D && diag; r++)
        for (int c = 0; c < D; c++)
            if (r != c && (g.mat[2 * (r * D + c)] != 0.0 || g.mat[2 * (r * D + c) + 1] != 0.0)) { diag = false; break; }
    if (diag) {
        std::vector<double> d(2 * D);
        for (int i = 0; i < D; i++) { d[2 * i] = g.mat[2 * (i * D + i)]; d[2 * i + 1] = g.mat[2 * (i * D + i) + 1]; }
        g.mat.swap(d);
        g.kind = 1;
        return;
    }
    // monomial with unit phases (X, Y, CNOT, SWAP, ISWAP, CCNOT, ...)
    std::vector<int> perm(2 * D, -1);
    std::vector<int> rows_used(D, 0);
    for (int c = 0; c < D; c++) {
        int nz = 0, row = -1, ph = -1;
        for (int r = 0; r < D; r++) {
            double re = g.mat[2 * (r * D + c)], im = g.mat[2 * (r * D + c) + 1];
            if (re == 0.0 && im == 0.0) continue;
            nz++;
            row = r;
            if (im == 0.0 && re == 1.0) ph = 0;
            else if (re == 0.0 && im == 1.0) ph = 1;
            else if (im == 0.0 && re == -1.0) ph = 2;
            else if (re == 0.0 && im == -1.0) ph = 3;
        }
        if (nz != 1 || ph < 0 || rows_used[row]) return;
        rows_used[row] = 1;
        perm[2 * c] = row;
        perm[2 * c + 1] = ph;
    }
    g.perm = perm;
    g.kind = 2;
}

}  // namespace

int bs_lower_gate(bs_sim* s, const double* matrix, int k, const int* targets, int nc, const int* controls,
                  const int* cvals, unsigned flags, bool dm_superop, std::vector<HostGate>& out) {
    const int nvec = bs_vec_bits(s);
    const int nq = dm_superop ? s->n : nvec;   // qubit range of the arguments
    if (k < 1 || k > BS_MAX_TARGETS) return bs_fail(s, BS_ERR_INVALID_ARG, "gate needs 1..10 targets");
    if (nc < 0 || nc > BS_MAX_CONTROLS) return bs_fail(s, BS_ERR_INVALID_ARG, "too many controls");
    if (!matrix) return bs_fail(s, BS_ERR_INVALID_ARG, "null matrix");
    std::string why;
    if (!valid_qubits(nq, k, targets, nc, controls, cvals, why)) return bs_fail(s, BS_ERR_INVALID_ARG, why);
    const int D = 1 << k;
    int ct[BS_MAX_TARGETS];
    canonical_targets(k, targets, flags, ct);
    HostGate g;
    g.k = k;
    const bool diag = (flags & BS_GATE_DIAGONAL) != 0;
    g.kind = diag ? 1 : 0;
    const int ne = diag ? D : D * D;
    g.mat.assign(matrix, matrix + 2 * ne);
    if (flags & BS_GATE_CONJ)
        for (int i = 0; i < ne; i++) g.mat[2 * i + 1] = -g.mat[2 * i + 1];
    for (double v : g.mat)
        if (!std::isfinite(v)) return bs_fail(s, BS_ERR_INVALID_ARG, "matrix has non-finite entries");
    classify(g);
    auto put = [&](int offset, bool conj, bool last) {
        HostGate h = last ? std::move(g) : g;
        for (int j = 0; j < k; j++) h.ebit[j] = offset + (nq - 1 - ct[j]);
        h.cmask = 0;
        h.cval = 0;
        for (int i = 0; i < nc; i++) {
            int e = offset + (nq - 1 - controls[i]);
            h.cmask |= 1ULL << e;
            if (!cvals || cvals[i]) h.cval |= 1ULL << e;
        }
        if (conj) {
            if (h.kind == 2) {
                for (int c = 0; c < D; c++) h.perm[2 * c + 1] = (4 - h.perm[2 * c + 1]) & 3;
            } else {
                for (size_t i = 1; i < h.mat.size(); i += 2) h.mat[i] = -h.mat[i];
            }
        }
        out.push_back(std::move(h));
    };
    if (dm_superop) {
        put(s->n, false, false);   // column bits: U
        put(0, true, true);        // row bits: conj(U)
    } else {
        put(0, false, true);
    }
    return BS_OK;
}

// Full channel on the stored matrix: S <- sum_q conj(K_q) S K_q^T, as one dense
// gate on (row bits, column bits) of vec(S).
int bs_lower_kraus_physical(bs_sim* s, const double* kraus, int nk, int k, const int* targets, unsigned flags,
                            std::vector<HostGate>& out) {
    if (s->kind != BS_KIND_DM) return bs_fail(s, BS_ERR_STATE, "noise needs a density-matrix simulator");
    if (k < 1 || 2 * k > BS_MAX_TARGETS) return bs_fail(s, BS_ERR_UNSUPPORTED, "physical channel supports 1..5 targets");
    if (nk < 1) return bs_fail(s, BS_ERR_INVALID_ARG, "no Kraus matrices");
    std::string why;
    if (!valid_qubits(s->n, k, targets, 0, nullptr, nullptr, why)) return bs_fail(s, BS_ERR_INVALID_ARG, why);
    const int D = 1 << k, D2 = D * D;
    int ct[BS_MAX_TARGETS];
    canonical_targets(k, targets, flags, ct);
    HostGate g;
    g.kind = 0;
    g.k = 2 * k;
    for (int j = 0; j < k; j++) {
        g.ebit[j] = s->n - 1 - ct[j];           // row bits
        g.ebit[k + j] = 2 * s->n - 1 - ct[j];   // column bits
    }
    g.mat.assign((size_t)2 * D2 * D2, 0.0);
    for (int q = 0; q < nk; q++) {
        const double* K = kraus + (size_t)q * 2 * D2;
        for (double* p = (double*)K; p < K + 2 * D2; p++)
            if (!std::isfinite(*p)) return bs_fail(s, BS_ERR_INVALID_ARG, "Kraus matrix has non-finite entries");
        for (int br = 0; br < D; br++)
            for (int bc = 0; bc < D; bc++)
                for (int ar = 0; ar < D; ar++)
                    for (int ac = 0; ac < D; ac++) {
                        cd kr(K[2 * (br * D + ar)], -K[2 * (br * D + ar) + 1]);   // conj(K)[br, ar]
                        cd kc(K[2 * (bc * D + ac)], K[2 * (bc * D + ac) + 1]);    // K[bc, ac]
                        cd v = kr * kc;
                        size_t row = (size_t)(br | (bc << k)), col = (size_t)(ar | (ac << k));
                        g.mat[2 * (row * D2 + col)] += v.real();
                        g.mat[2 * (row * D2 + col) + 1] += v.imag();
                    }
    }
    classify(g);
    out.push_back(std::move(g));
    return BS_OK;
}

int bs_tile_bits(const bs_sim* s) {
    int b = s ? s->tune.tile_bits : -1;
    if (b < 0) {
        const char* e = getenv("BS_TILE_BITS");
        b = e ? atoi(e) : BS_TILE_MAX_BITS;
    }
    return (b >= 10 && b <= BS_TILE_MAX_BITS) ? b : BS_TILE_MAX_BITS;
}

int bs_tile_threads(const bs_sim* s) {
    int t = s ? s->tune.tile_threads : -1;
    if (t < 0) {
        const char* e = getenv("BS_TILE_THREADS");
        t = e ? atoi(e) : 256;
    }
    return (t == 512) ? 512 : 256;
}

bool bs_tc_enabled(const bs_sim* s) {
    if (s && s->tune.tc >= 0) return s->tune.tc != 0;
    const char* v = getenv("BS_TC");   // read on every call, so a process can compare both paths
    return !(v && v[0] == '0');
}

int bs_tc_min_bits(const bs_sim* s) {
    if (s && s->tune.tc_min_bits >= 0) return s->tune.tc_min_bits;
    const char* v = getenv("BS_TC_MIN_BITS");
    return v ? atoi(v) : 22;   // measured wins from 24 bits up; small states are bound by host planning
}

double bs_tc_cost(const bs_sim* s) {
    if (s && s->tune.tc_cost >= 0) return s->tune.tc_cost;
    const char* v = getenv("BS_TC_COST");
    return v ? atof(v) : 2.0;
}

// Greedy sweep planner.  A gate may move ahead of gates it does not share a bit
// with; a dense or monomial gate needs its target bits inside the tile, a
// diagonal gate or a control never does (their bits are read from the index).
void bs_plan_sweeps(std::vector<HostGate>& gates, int n_bits, int tile_bits, std::vector<Sweep>& out) {
    const int T = std::min(tile_bits, n_bits);
    const int L = std::min(BS_TILE_LOW_BITS, T);
    const int cap = T - L;
    const size_t G = gates.size();
    std::vector<char> done(G, 0);
    size_t remaining = G, first = 0;
    // kind 5 (reference-rule channel) acts on the elements whose row and column agree on every other
    // bit: it commutes with nothing, so it touches every bit, and it needs its row and column bits
    auto touch = [&](const HostGate& g) {
        if (g.kind == 5) return ~(uint64_t)0;
        uint64_t m = g.cmask;
        for (int q = 0; q < g.k; q++) m |= 1ULL << g.ebit[q];
        return m;
    };
    auto need = [&](const HostGate& g) {
        uint64_t m = 0;
        if (g.kind == 1) return m;
        const int nb = g.kind == 5 ? 2 * g.k : g.k;
        for (int q = 0; q < nb; q++) if (g.ebit[q] >= L) m |= 1ULL << g.ebit[q];
        return m;
    };
    while (remaining) {
        Sweep sw;
        uint64_t chosen = 0, blocked = 0;
        int nchosen = 0;
        bool big_alone = false;
        for (size_t i = first; i < G; i++) {
            if (done[i]) continue;
            const HostGate& g = gates[i];
            uint64_t t = touch(g);
            if (t & blocked) { blocked |= t; continue; }
            uint64_t nb = need(g) & ~chosen;
            int add = __builtin_popcountll(nb);
            bool too_big = (g.kind != 1) && (g.k > BS_TILE_MAXK || __builtin_popcountll(need(g)) > cap);
            if (too_big) {
                // a gate no tile can hold runs in a sweep of its own
                if (sw.gates.empty()) { sw.gates.push_back(std::move(gates[i])); done[i] = 1; remaining--; big_alone = true; }
                blocked |= t;
                break;
            }
            if (nchosen + add <= cap) {
                chosen |= nb;
                nchosen += add;
                sw.gates.push_back(std::move(gates[i]));
                done[i] = 1;
                remaining--;
            } else {
                blocked |= t;
            }
        }
        while (first < G && done[first]) first++;
        if (!big_alone) {
            for (int b = L; b < n_bits; b++) if ((chosen >> b) & 1ULL) sw.hi_bits.push_back(b);
            for (int b = L; b < n_bits && (int)sw.hi_bits.size() < cap; b++)
                if (!((chosen >> b) & 1ULL)) sw.hi_bits.push_back(b);
            std::sort(sw.hi_bits.begin(), sw.hi_bits.end());
        }
        out.push_back(std::move(sw));
    }
}
