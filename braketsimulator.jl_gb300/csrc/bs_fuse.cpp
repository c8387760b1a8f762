// Gate fusion for the tensor-core tile path.
//
// Inside one tile sweep, runs of gates are folded into dense unitaries on 5
// tile bits.  A gate can join a block when its dense targets lie in the tile and
// its tile bits fit the block; bits outside the tile (controls, and target bits
// of diagonal gates) are constant within a CTA, so the block is built once per
// assignment of those "uniform" bits (at most 3 of them) and each CTA picks its
// variant.  The products are formed here in FP64; the device applies them to the
// tile as real 64x64 GEMMs on tcgen05 tensor cores, with both operands split
// into exact 8-bit bf16 digits (an Ozaki-style split) so that the result keeps
// float-float accuracy.  This replaces, for those gates, the per-gate amplitude
// loops of the reference (src/gate_kernels.jl:489-775, src/custom_gates.jl:364-416);
// the fused product itself has no counterpart there.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include "bs_internal.h"

namespace {

using cd = std::complex<double>;
constexpr int kMaxUniform = 3;

// cost of a gate on the float-float path, in units of one dense 1-qubit gate
double ff_cost(const HostGate& g) {
    if (g.kind == 0) return (double)(1 << g.k) / 2.0;
    if (g.kind == 2) return 0.25;
    return 0.3;
}

bool is_plain_cz(const HostGate& g) {
    return g.kind == 1 && g.k == 1 && g.mat.size() == 4 && g.mat[0] == 1.0 && g.mat[1] == 0.0 && g.mat[2] == -1.0 &&
           g.mat[3] == 0.0 && __builtin_popcountll(g.cmask) == 1 && g.cval == g.cmask;
}

// Left-multiply the 32x32 block matrix U (row r, column c at U[r * 32 + c]) by a canonical gate.
// pos[e]: block bit of endian bit e, or -1 for a uniform bit whose value is (uval >> e) & 1.
void apply_block(const HostGate& g, const int* pos, uint64_t uval, cd* U) {
    // controls: in-block ones become a row-index condition, uniform ones decide whether the gate acts
    uint32_t cm = 0, cv = 0;
    uint64_t rest = g.cmask;
    while (rest) {
        const int e = __builtin_ctzll(rest);
        rest &= rest - 1;
        const uint64_t want = (g.cval >> e) & 1ULL;
        if (pos[e] < 0) {
            if (((uval >> e) & 1ULL) != want) return;
        } else {
            cm |= 1u << pos[e];
            cv |= (uint32_t)want << pos[e];
        }
    }
    const int D = 1 << g.k;
    if (g.kind == 1) {
        // diagonal: target bits may be uniform (constant over the block); row r scales by d[index(r)]
        for (uint32_t r = 0; r < 32; r++) {
            if ((r & cm) != cv) continue;
            int di = 0;
            for (int q = 0; q < g.k; q++) {
                const int e = g.ebit[q];
                const int bit = pos[e] >= 0 ? (int)((r >> pos[e]) & 1u) : (int)((uval >> e) & 1ULL);
                di |= bit << q;
            }
            const double dr = g.mat[2 * di], dim = g.mat[2 * di + 1];
            for (int c = 0; c < 32; c++) {
                const double ur = U[r * 32 + c].real(), ui = U[r * 32 + c].imag();
                U[r * 32 + c] = cd(dr * ur - dim * ui, dr * ui + dim * ur);
            }
        }
        return;
    }
    uint32_t off[32];
    uint32_t tmask = 0;
    for (int q = 0; q < g.k; q++) tmask |= 1u << pos[g.ebit[q]];
    for (int c = 0; c < D; c++) {
        uint32_t j = 0;
        for (int q = 0; q < g.k; q++) if ((c >> q) & 1) j |= 1u << pos[g.ebit[q]];
        off[c] = j;
    }
    static const cd ipow[4] = {cd(1, 0), cd(0, 1), cd(-1, 0), cd(0, -1)};
    cd x[32], y[32];
    for (uint32_t i = 0; i < 32; i++) {
        if (i & tmask) continue;
        if ((i & cm) != cv) continue;
        for (int col = 0; col < 32; col++) {
            for (int c = 0; c < D; c++) x[c] = U[(i | off[c]) * 32 + col];
            if (g.kind == 0) {
                // plain real arithmetic (std::complex products go through a NaN-checking library call)
                for (int r = 0; r < D; r++) {
                    double sr = 0, si = 0;
                    const double* mr = g.mat.data() + 2 * r * D;
                    for (int c = 0; c < D; c++) {
                        const double ar = mr[2 * c], ai = mr[2 * c + 1], xr = x[c].real(), xi = x[c].imag();
                        sr += ar * xr - ai * xi;
                        si += ar * xi + ai * xr;
                    }
                    y[r] = cd(sr, si);
                }
            } else {
                for (int c = 0; c < D; c++) y[g.perm[2 * c]] = ipow[g.perm[2 * c + 1] & 3] * x[c];
            }
            for (int r = 0; r < D; r++) U[(i | off[r]) * 32 + col] = y[r];
        }
    }
}

struct Block {
    uint64_t bits = 0;               // tile bits touched
    uint64_t ubits = 0;              // uniform (out-of-tile) bits the gates depend on
    std::vector<int> idx;            // gate indices, in order
    double cost = 0;
};

}  // namespace

void bs_fuse_tc(const std::vector<HostGate>& in, const int* local, int T, double threshold, std::vector<HostGate>& out) {
    out.clear();
    std::vector<Block> open;
    auto emit = [&](Block& b) {
        int ndense = 0;
        bool wide = false;   // 3- and 4-target gates always fuse: the tensor-core sweep has no float-float path for them
        for (int i : b.idx) {
            ndense += in[(size_t)i].kind == 0;
            wide = wide || (in[(size_t)i].kind != 1 && in[(size_t)i].k >= 3);
        }
        if (!wide && (b.cost <= threshold || ndense == 0)) {
            for (int i : b.idx) out.push_back(in[(size_t)i]);
            return;
        }
        // block bits ascending by tile position, padded to 5 with other tile bits (high ones first, so that
        // the low contiguous bits stay column bits of the GEMM where possible)
        std::vector<int> eb;
        for (int e = 0; e < 64; e++) if ((b.bits >> e) & 1ULL) eb.push_back(e);
        std::vector<int> tile_e(T, -1);
        for (int e = 0; e < 64; e++) if (local[e] >= 0 && local[e] < T) tile_e[local[e]] = e;
        for (int p = T - 1; p >= 0 && (int)eb.size() < 5; p--) {
            int e = tile_e[p];
            if (e >= 0 && !((b.bits >> e) & 1ULL)) eb.push_back(e);
        }
        std::sort(eb.begin(), eb.end(), [&](int a, int c) { return local[a] < local[c]; });
        int pos[64];
        for (int e = 0; e < 64; e++) pos[e] = -1;
        for (int q = 0; q < 5; q++) pos[eb[(size_t)q]] = q;
        HostGate f;
        f.kind = 4;
        f.k = 5;
        for (int q = 0; q < 5; q++) f.ebit[q] = eb[(size_t)q];
        for (int e = 0; e < 64; e++) if ((b.ubits >> e) & 1ULL) f.ubits.push_back(e);
        const int nvar = 1 << f.ubits.size();
        f.mat.assign((size_t)nvar * 2 * 32 * 32, 0.0);
        for (int var = 0; var < nvar; var++) {
            uint64_t uval = 0;
            for (size_t i = 0; i < f.ubits.size(); i++) if ((var >> i) & 1) uval |= 1ULL << f.ubits[i];
            double* m = f.mat.data() + (size_t)var * 2048;
            std::vector<cd> U(32 * 32, cd(0, 0));
            for (int r = 0; r < 32; r++) U[(size_t)r * 33] = 1;
            for (int i : b.idx) apply_block(in[(size_t)i], pos, uval, U.data());
            for (int r = 0; r < 32 * 32; r++) {
                m[2 * r] = U[(size_t)r].real();
                m[2 * r + 1] = U[(size_t)r].imag();
            }
        }
        out.push_back(std::move(f));
    };
    auto flush_if = [&](uint64_t bits) {
        for (size_t j = 0; j < open.size();) {
            if (open[j].bits & bits) {
                emit(open[j]);
                open.erase(open.begin() + (long)j);
            } else {
                j++;
            }
        }
    };
    for (size_t i = 0; i < in.size(); i++) {
        const HostGate& g = in[i];
        if (g.kind == 5) {
            // a reference-rule channel commutes with nothing: every open block closes before it
            for (Block& b : open) emit(b);
            open.clear();
            out.push_back(g);
            continue;
        }
        // tile bits and uniform bits of the gate; dense and monomial targets must be in the tile
        uint64_t bits = 0, ub = 0;
        bool fusable = g.kind <= 2 && g.k <= 5;
        for (int q = 0; q < g.k; q++) {
            const int e = g.ebit[q];
            if (local[e] >= 0) bits |= 1ULL << e;
            else if (g.kind == 1) ub |= 1ULL << e;
            else fusable = false;
        }
        for (int e = 0; e < 64; e++)
            if ((g.cmask >> e) & 1ULL) {
                if (local[e] >= 0) bits |= 1ULL << e;
                else ub |= 1ULL << e;
            }
        if (__builtin_popcountll(bits) > 5 || __builtin_popcountll(ub) > kMaxUniform || bits == 0) fusable = false;
        if (!fusable) {
            // close every block sharing a bit with the gate, uniform bits included (the gate may act on them)
            const uint64_t all = bits | ub | g.cmask;
            uint64_t tgt = 0;
            for (int q = 0; q < g.k; q++) tgt |= 1ULL << g.ebit[q];
            for (size_t j = 0; j < open.size();) {
                if ((open[j].bits | open[j].ubits) & (all | tgt)) {
                    emit(open[j]);
                    open.erase(open.begin() + (long)j);
                } else {
                    j++;
                }
            }
            out.push_back(g);
            continue;
        }
        const double gc = is_plain_cz(g) ? 0.1 : ff_cost(g);
        uint64_t uni = bits, uu = ub;
        for (const Block& b : open) if (b.bits & bits) { uni |= b.bits; uu |= b.ubits; }
        if (__builtin_popcountll(uni) > 5 || __builtin_popcountll(uu) > kMaxUniform) {
            // the gate links blocks that cannot all merge: keep the costliest block it fits into and close
            // the others (their gates precede it and touch none of the kept block's tile bits)
            int keep = -1;
            for (size_t j = 0; j < open.size(); j++)
                if ((open[j].bits & bits) && __builtin_popcountll(open[j].bits | bits) <= 5 &&
                    __builtin_popcountll(open[j].ubits | ub) <= kMaxUniform &&
                    (keep < 0 || open[j].cost > open[(size_t)keep].cost))
                    keep = (int)j;
            if (keep >= 0) {
                const uint64_t kb = open[(size_t)keep].bits;
                for (size_t j = 0; j < open.size();) {
                    if ((open[j].bits & bits) && open[j].bits != kb) {
                        emit(open[j]);
                        open.erase(open.begin() + (long)j);
                    } else {
                        j++;
                    }
                }
                for (const Block& b : open) if (b.bits == kb) { uni = kb | bits; uu = b.ubits | ub; }
            }
        }
        if (__builtin_popcountll(uni) <= 5 && __builtin_popcountll(uu) <= kMaxUniform) {
            Block nb;
            nb.bits = uni;
            nb.ubits = uu;
            // merge the intersecting blocks (pairwise disjoint in tile bits, so their gates commute)
            for (size_t j = 0; j < open.size();) {
                if (open[j].bits & bits) {
                    nb.idx.insert(nb.idx.end(), open[j].idx.begin(), open[j].idx.end());
                    nb.cost += open[j].cost;
                    open.erase(open.begin() + (long)j);
                } else {
                    j++;
                }
            }
            std::sort(nb.idx.begin(), nb.idx.end());
            nb.idx.push_back((int)i);
            nb.cost += gc;
            open.push_back(std::move(nb));
        } else {
            flush_if(bits);
            Block nb;
            nb.bits = bits;
            nb.ubits = ub;
            nb.idx.push_back((int)i);
            nb.cost = gc;
            open.push_back(std::move(nb));
        }
    }
    for (Block& b : open) emit(b);
}

// Fusion for the sweeps that run on the CUDA cores (float-float and complex64 tile kernels): runs of
// gates whose tile bits (targets and controls) fit in maxk bits become one dense maxk-bit gate when
// that is cheaper, counting one shared-memory pass of the tile (pass, in units of a dense 1-qubit
// gate's arithmetic) per gate applied.  The kernels apply every gate as one pass, so fusing two
// 1-qubit gates on different bits into a 4x4 keeps the arithmetic and halves the passes.  Gates with
// bits outside the tile, 3+-bit gates and channels stay as they are and close the blocks they touch.
void bs_fuse_small(const std::vector<HostGate>& in, const int* local, double pass, int maxk, std::vector<HostGate>& out) {
    out.clear();
    struct SBlock {
        uint64_t bits = 0;
        std::vector<int> idx;
        double cost = 0;
    };
    std::vector<SBlock> open;
    auto gate_bits = [&](const HostGate& g, bool& in_tile) {
        uint64_t b = g.cmask;
        for (int q = 0; q < g.k; q++) b |= 1ULL << g.ebit[q];
        in_tile = true;
        for (uint64_t r = b; r; r &= r - 1)
            if (local[__builtin_ctzll(r)] < 0) in_tile = false;
        return b;
    };
    auto emit = [&](SBlock& b) {
        const int k = __builtin_popcountll(b.bits);
        if (b.idx.size() < 2 || pass + (double)(1 << k) / 2.0 >= b.cost) {
            for (int i : b.idx) out.push_back(in[(size_t)i]);
            return;
        }
        // the block's bits take block positions 0..k-1; the 32x32 product then holds U (x) I
        int pos[64];
        for (int e = 0; e < 64; e++) pos[e] = -1;
        HostGate f;
        f.kind = 0;
        f.k = k;
        int q = 0;
        for (int e = 0; e < 64; e++)
            if ((b.bits >> e) & 1ULL) { pos[e] = q; f.ebit[q] = e; q++; }
        std::vector<cd> U(32 * 32, cd(0, 0));
        for (int r = 0; r < 32; r++) U[(size_t)r * 33] = 1;
        for (int i : b.idx) apply_block(in[(size_t)i], pos, 0, U.data());
        const int D = 1 << k;
        f.mat.assign((size_t)2 * D * D, 0.0);
        for (int r = 0; r < D; r++)
            for (int c = 0; c < D; c++) {
                f.mat[(size_t)2 * (r * D + c)] = U[(size_t)r * 32 + c].real();
                f.mat[(size_t)2 * (r * D + c) + 1] = U[(size_t)r * 32 + c].imag();
            }
        out.push_back(std::move(f));
    };
    auto close_touching = [&](uint64_t bits) {
        for (size_t j = 0; j < open.size();) {
            if (open[j].bits & bits) {
                emit(open[j]);
                open.erase(open.begin() + (long)j);
            } else {
                j++;
            }
        }
    };
    for (size_t i = 0; i < in.size(); i++) {
        const HostGate& g = in[i];
        if (g.kind == 5) {   // a reference-rule channel commutes with nothing
            for (SBlock& b : open) emit(b);
            open.clear();
            out.push_back(g);
            continue;
        }
        bool in_tile = false;
        const uint64_t bits = gate_bits(g, in_tile);
        const bool fusable = g.kind <= 2 && in_tile && bits && __builtin_popcountll(bits) <= maxk;
        if (!fusable) {
            close_touching(bits);
            out.push_back(g);
            continue;
        }
        uint64_t uni = bits;
        for (const SBlock& b : open) if (b.bits & bits) uni |= b.bits;
        if (__builtin_popcountll(uni) > maxk) {
            close_touching(bits);
            uni = bits;
        }
        SBlock nb;
        nb.bits = uni;
        // merge the intersecting blocks (pairwise disjoint, so their gates commute), then the gate
        for (size_t j = 0; j < open.size();) {
            if (open[j].bits & bits) {
                nb.idx.insert(nb.idx.end(), open[j].idx.begin(), open[j].idx.end());
                nb.cost += open[j].cost;
                open.erase(open.begin() + (long)j);
            } else {
                j++;
            }
        }
        std::sort(nb.idx.begin(), nb.idx.end());
        nb.idx.push_back((int)i);
        nb.cost += is_plain_cz(g) ? 0.1 : pass + ff_cost(g);   // CZs share one parity pass anyway
        open.push_back(std::move(nb));
    }
    for (SBlock& b : open) emit(b);
}

bool bs_tc_exponent(const double* mat, int n_mat, int& eu) {
    double mx = 0;
    for (size_t i = 0; i < (size_t)n_mat * 2048; i++) {
        if (!std::isfinite(mat[i])) return false;
        mx = std::max(mx, std::fabs(mat[i]));
    }
    int e = 0;
    if (mx > 0) std::frexp(mx, &e);          // mx < 2^e
    if (e > 12) return false;
    eu = std::max(e, -60);
    return true;
}
