// Tensor-core application of a fused 5-bit unitary to a 2^12-amplitude tile.
//
// The tile (float-float complex values in shared memory) is viewed as 128
// columns of 32 amplitudes: the 5 target bits index a column's amplitudes, the
// other 7 tile bits index the column.  With the real embedding
//     out[2t'+c'] = sum_k U_real[2t'+c'][k] x[k],  x[2t+0] = Re a_t, x[2t+1] = Im a_t
// the gate is D[128 x 64] = A[128 x 64] * U_real^T, one tcgen05 GEMM per tile.
//
// Exactness (Ozaki-style split): the tile is scaled by a power of two (from the
// largest exponent over the tile) so that |x| < 2^8, and both x and U_real (on
// the device, from the FP64 matrix) are split into six balanced 8-bit digits, digit j carried as bf16 d_j * 2^(-8j) with
// |d_j| <= 128 (256 for the one digit that absorbs the float-float low word).
// The 26 digit pairs with i + j <= 6 are accumulated in five rounds by digit
// weight: i+j = 0, 1, 2, 3 each alone (every product a multiple of the same
// power of two and every partial sum below 2^24 of it, so these FP32 sums are
// exact) and i+j = 4, 5, 6 together (rounding at 2^-56 of the result).  After
// each round the CUDA cores fold the FP32 accumulator into a running
// float-float sum, while the tensor cores run other rounds in the other of two
// accumulators; two threads issue, one per accumulator, so that neither chain
// of issue, fold and re-issue waits for the other.  What remains is the 48-bit
// truncation of both operands, ~2^-46 of the tile's largest value per fused gate.
//
// TMEM (256 columns per CTA, so that two CTAs share an SM and one's MMAs
// overlap the other's CUDA-core work):
//   D0, D1 (FP32 accumulators, lane m): columns 0..63, and columns 192..255 once
//     the MMAs of round 4 that read A digit slices 4 and 5 (the only readers of
//     those slices, issued first) have completed.
//   A (state digits): lanes 0..127 = columns m, TMEM columns kA0 + 32 j + t hold
//     (Re, Im) of digit j of amplitude t as a bf16 pair (low half = Re).
// B (matrix digits): shared memory, K-major, no swizzle: 8x8 core matrices of
//   128 B; per (digit i, k-step s) a 2 KiB block, row groups 256 B apart (SBO),
//   the two K halves 128 B apart (LBO).  Made on the device by k_tc_digits.
#pragma once
#include <cstdint>

namespace tc {

constexpr int kA0 = 64;         // first TMEM column of the six A digit slices
constexpr uint32_t kCols = 256; // TMEM columns held by one CTA
// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, N = 64, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);
constexpr long long kSpin = 1LL << 31;   // cycles before a wait gives up (~1 s)
constexpr int kPoolBlock = 24576;        // bf16 values per fused matrix (6 digits x 64 x 64)

// Bank swizzle of the 2^12 tile: bits 3..11 folded into bits 0..2, so that strided columns of
// 16-byte values (any 5 target bits) spread over all bank groups.  A bijection on [0, 4096).
__device__ __forceinline__ int sw(int j) { return j ^ (((j >> 3) ^ (j >> 6) ^ (j >> 9)) & 7); }

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, LBO 128 B, SBO 256 B, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t bdesc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           (1ULL << 46);
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait for the phase with the given parity; false if it did not complete in kSpin cycles.
// Each try_wait suspends the thread until the phase completes or ~20 us pass, so waiting warps do not
// take issue slots from the working ones.
__device__ __forceinline__ bool mbar_wait_for(uint32_t bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity), "r"(20000u)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > limit) return false;
    }
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) { return mbar_wait_for(bar, parity, kSpin); }

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init_n(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// generic-proxy shared-memory writes become visible to the async proxy (bulk copies, MMA operands)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t slot) {   // whole warp
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {   // whole warp
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kCols));
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void st8(uint32_t taddr, const uint32_t (&w)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(w[0]),
                 "r"(w[1]), "r"(w[2]), "r"(w[3]), "r"(w[4]), "r"(w[5]), "r"(w[6]), "r"(w[7])
                 : "memory");
}
__device__ __forceinline__ void st4(uint32_t taddr, const uint32_t (&w)[4]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(w[0]), "r"(w[1]),
                 "r"(w[2]), "r"(w[3])
                 : "memory");
}
// no memory clobber: TMEM stores stay ordered against the other tcgen05 asm (all volatile), and
// shared-memory loads of the slicing may be scheduled across them
__device__ __forceinline__ void st2(uint32_t taddr, uint32_t w0, uint32_t w1) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1,%2};" ::"r"(taddr), "r"(w0), "r"(w1));
}
// wait for this thread's TMEM loads; the registers they fill are tied to the wait so that no use of
// them is scheduled before it
__device__ __forceinline__ void wait_ld16(uint32_t (&r)[8], uint32_t (&q)[8]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(q[0]), "+r"(q[1]), "+r"(q[2]), "+r"(q[3]), "+r"(q[4]), "+r"(q[5]), "+r"(q[6]), "+r"(q[7])
                 :
                 : "memory");
}
__device__ __forceinline__ void ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
}

__device__ __forceinline__ void mma(uint32_t d, uint32_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
        "r"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Six digits of y = yh + yl (|y| < 2^7 after scaling): q[j] = d_j 2^(-8j), y ~ sum_j q[j].
// Rounding to the digit grid uses the 1.5 * 2^(23-8j) shift, exact while |R| < 2^(22-8j).
__device__ __forceinline__ void digits(float yh, float yl, float (&q)[6]) {
    float R = yh;
    q[0] = __fsub_rn(__fadd_rn(R, 12582912.0f), 12582912.0f);            // grid 1
    R = __fsub_rn(R, q[0]);
    q[1] = __fsub_rn(__fadd_rn(R, 49152.0f), 49152.0f);                  // grid 2^-8
    R = __fsub_rn(R, q[1]);
    q[2] = __fsub_rn(__fadd_rn(R, 192.0f), 192.0f);                      // grid 2^-16
    R = __fadd_rn(__fsub_rn(R, q[2]), yl);                               // low word joins here
    q[3] = __fsub_rn(__fadd_rn(R, 0.75f), 0.75f);                        // grid 2^-24
    R = __fsub_rn(R, q[3]);
    q[4] = __fsub_rn(__fadd_rn(R, 0.0029296875f), 0.0029296875f);        // grid 2^-32
    R = __fsub_rn(R, q[4]);
    q[5] = __fsub_rn(__fadd_rn(R, 1.1444091796875e-05f), 1.1444091796875e-05f);   // grid 2^-40
}

// error-free s + g (Knuth TwoSum): s <- rounded sum, returns the rounding error
__device__ __forceinline__ float two_sum(float& s, float g) {
    const float t = __fadd_rn(s, g);
    const float bb = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(g, bb));
    s = t;
    return e;
}

// digits() on both halves
__device__ __forceinline__ void digits2(f2 yh, f2 yl, f2 (&q)[6]) {
    const f2 c0 = pk(12582912.0f, 12582912.0f), c1 = pk(49152.0f, 49152.0f), c2 = pk(192.0f, 192.0f),
             c3 = pk(0.75f, 0.75f), c4 = pk(0.0029296875f, 0.0029296875f),
             c5 = pk(1.1444091796875e-05f, 1.1444091796875e-05f);
    f2 R = yh;
    q[0] = sub2(add2(R, c0), c0);
    R = sub2(R, q[0]);
    q[1] = sub2(add2(R, c1), c1);
    R = sub2(R, q[1]);
    q[2] = sub2(add2(R, c2), c2);
    R = add2(sub2(R, q[2]), yl);
    q[3] = sub2(add2(R, c3), c3);
    R = sub2(R, q[3]);
    q[4] = sub2(add2(R, c4), c4);
    R = sub2(R, q[4]);
    q[5] = sub2(add2(R, c5), c5);
}
// two_sum() on both halves
__device__ __forceinline__ f2 two_sum2(f2& s, f2 g) {
    const f2 t = add2(s, g);
    const f2 bb = sub2(t, s);
    const f2 e = add2(sub2(s, sub2(t, bb)), sub2(g, bb));
    s = t;
    return e;
}

struct State {
    uint32_t tmem;   // TMEM base address
    uint32_t bar;    // seven mbarriers 8 bytes apart: digit-slice copy (1 arrival + bytes), MMAs done into
                     // D0, into D1 (commits), D0 read, D1 read (one arrival per warp), round 4's
                     // state-digit-4/5 MMAs done, round 0 done into D2 (commits)
    uint32_t ph;     // expected phase parity of barrier k in bit k
    bool pref;       // the digit slices of the gate about to run were copied ahead (uniform)
};

constexpr uint32_t kD1 = kA0 + 128;   // second accumulator: the columns of A digit slices 4 and 5
constexpr uint32_t kD2 = kA0 + 64;    // third accumulator (round 0 only): the columns of A digit slices 2 and 3

// Source of a fused gate's digit slices for the CTA: the matrix variant selected by the base bits.
__device__ __forceinline__ const uint16_t* slice_src(const TileGate& g, const uint16_t* pool, int64_t base) {
    const int nu = g.tc_nu;
    int var = 0;
#pragma unroll
    for (int i = 0; i < 3; i++)
        if (i < nu) var |= (int)((base >> g.tc_ub[i]) & 1) << i;
    return pool + (size_t)(g.tc_off + var) * kPoolBlock;
}
// One thread: the 48 KiB of digit slices into sB, completing on barrier bar.
__device__ __forceinline__ void copy_slices(uint32_t sB, const uint16_t* src, uint32_t bar) {
    mbar_expect_tx(bar, (uint32_t)kPoolBlock * 2);
    bulk_g2s(sB, src, (uint32_t)kPoolBlock * 2, bar);
}

// One thread issues the MMAs of the digit pairs (i, j) with G0 <= i + j <= G1 and JLO <= j <= JHI
// (j: state digit, i: matrix digit) into the accumulator at TMEM column dcol; the first one
// overwrites when OVERWRITE.  The pair set is a compile-time constant so that the loops unroll and
// every operand address is the base plus a constant: a single thread issues back to back (a
// run-time loop here doubled the time per MMA).  b0 = descriptor of the first digit slice; slice
// (i, s) starts (i*4+s)*2048 bytes later, which adds (i*4+s)*128 to the 14-bit start-address field
// without carry (the slices span 48 KiB).
template <int G0, int G1, int JLO, int JHI, bool OVERWRITE>
__device__ __forceinline__ void issue_pairs(uint32_t tmem, uint32_t dcol, uint64_t b0_) {
    // an opaque copy, so that the descriptors are formed here and not hoisted into registers
    // held across the caller's code
    uint64_t b0;
    asm volatile("mov.b64 %0, %1;" : "=l"(b0) : "l"(b0_));
    int n = 0;
#pragma unroll
    for (int gs = G0; gs <= G1; gs++)
#pragma unroll
        for (int j = 0; j <= gs; j++)
#pragma unroll
            for (int s = 0; s < 4; s++) {
                const int i = gs - j;
                if (i > 5 || j > 5 || j < JLO || j > JHI) continue;
                mma(tmem + dcol, tmem + (uint32_t)(kA0 + 32 * j + 8 * s), b0 + (uint64_t)((i * 4 + s) * 128),
                    (OVERWRITE && n == 0) ? 0u : 1u);
                n++;
            }
}
// Round r < 4: the pairs of weight r, overwriting the accumulator, then a commit to bar.
template <int ROUND>
__device__ __forceinline__ void issue_round(uint32_t tmem, uint32_t dcol, uint64_t b0, uint32_t bar) {
    issue_pairs<ROUND, ROUND, 0, 5, true>(tmem, dcol, b0);
    commit(bar);
}

// Fold of one round's accumulator columns (this thread's NA amplitudes, re and im packed) into the
// float-float sums: MODE 0: E = D, 1: E += D, 2: S = D, 3: E += TwoSum(S, D) error with S updated.
template <int MODE, int NA>
__device__ __forceinline__ void fold(uint32_t taddr, f2 (&S)[NA], f2 (&E)[NA]) {
#pragma unroll
    for (int c2 = 0; c2 < NA / 4; c2 += 2) {   // two 8-column loads in flight, one wait
        uint32_t r[2][8];
        ld8(taddr + (uint32_t)(8 * c2), r[0]);
        ld8(taddr + (uint32_t)(8 * c2 + 8), r[1]);
        wait_ld16(r[0], r[1]);
#pragma unroll
        for (int u = 0; u < 2; u++)
#pragma unroll
            for (int p = 0; p < 4; p++) {
                const int o = 4 * (c2 + u) + p;
                const f2 gv = pk(__uint_as_float(r[u][2 * p]), __uint_as_float(r[u][2 * p + 1]));
                if (MODE == 0) E[o] = gv;
                else if (MODE == 1) E[o] = add2(E[o], gv);
                else if (MODE == 2) S[o] = gv;
                else E[o] = add2(E[o], two_sum2(S[o], gv));
            }
    }
}

// Warp-uniform bounded wait on barrier k of the state for its expected parity, then the parity flips.
__device__ __forceinline__ bool wait_bar(State& st, int k, int lane_id) {
    uint32_t done = 1;
    if (lane_id == 0) done = mbar_wait(st.bar + 8u * (uint32_t)k, (st.ph >> k) & 1u) ? 1u : 0u;
    done = __shfl_sync(0xffffffffu, done, 0);
    st.ph ^= 1u << k;
    fence_after();
    return done != 0;
}
// One thread's bounded wait (the parity flip is left to the caller, which flips it on every thread).
__device__ __forceinline__ bool wait_bar1(const State& st, int k) {
    const bool ok = mbar_wait(st.bar + 8u * (uint32_t)k, (st.ph >> k) & 1u);
    fence_after();
    return ok;
}

// Applies fused gate g to the (swizzled) 2^12 tile sm of float4 (re hi, im hi, re lo, im lo).
// Called by all NT threads of the CTA (NT/128 threads per tile column, 32*128/NT amplitudes each),
// which then synchronise.  base: the CTA's global base index (selects the matrix variant).  s_tsw:
// 32 ints of shared scratch; s_wmax: NT/32 per-warp maxima of the high words' exponent fields.
// gnext: the tile's next fused gate, whose digit slices are copied ahead as soon as this gate's
// MMAs have completed (null: none, or it copies its own); s_nsrc: shared scratch for their source.
// The swizzle is linear over XOR, so the position of column m's amplitude t is
// sw(column bits) ^ sw(target bits of t); both come from the gate's host-made table (tab: 56
// uint16, sw of the column bits of m & 15 and of m >> 4, then sw of the target bits of t).
// On a wait that gives up, sets *fail and *err and leaves the tile partly updated.
template <int NT>
__device__ __forceinline__ void apply(float4* sm, const TileGate& g, const TileGate* gnext,
                                      const uint16_t* __restrict__ pool, const uint16_t* __restrict__ tab,
                                      uint16_t* sB, State& st, int64_t base,
                                      uint32_t* s_wmax, bool emax_ok, int* s_tsw, const uint16_t** s_nsrc, int* s_fail,
                                      int* err) {
    constexpr int HP = NT / 128;   // threads per column
    constexpr int NA = 32 / HP;    // amplitudes per thread
    const int tid = threadIdx.x, warp = tid >> 5, lane_id = tid & 31, m = tid & 127, h = tid >> 7;
    // the previous readers of sB (the MMAs of the previous fused gate) have completed
    if (!st.pref && tid == 0) copy_slices(su32(sB), slice_src(g, pool, base), st.bar);
    if (tid < 32) s_tsw[tid] = tab[24 + tid];
    const int spm = tab[m & 15] ^ tab[16 + (m >> 4)];
    const int* tsw = s_tsw + NA * h;
    // Tile scale: the largest exponent of the high words over the tile, per warp in s_wmax.  It was
    // left there by the previous fused gate's write-back or the tile load unless a gate that may
    // change magnitudes ran since (emax_ok false); then it is taken here in one pass.
    if (!emax_ok) {
        const float2* hi = reinterpret_cast<const float2*>(sm);
        uint32_t eb = 0;
#pragma unroll 4
        for (int a = 0; a < 4096 / NT; a++) {
            const float2 va = hi[2 * (a * NT + tid)];
            eb = max(eb, max(__float_as_uint(va.x) & 0x7F800000u, __float_as_uint(va.y) & 0x7F800000u));
        }
        eb = __reduce_max_sync(0xffffffffu, eb);
        if (lane_id == 0) s_wmax[warp] = eb;
    }
    __syncthreads();
    uint32_t eall = s_wmax[0];
#pragma unroll
    for (int w = 1; w < NT / 32; w++) eall = max(eall, s_wmax[w]);
    const int ebc = max((int)(eall >> 23), max(6, 14 - g.tc_eu));
    const float sc = __uint_as_float((uint32_t)(260 - ebc) << 23);                 // 2^(7 - E)
    const float osc = __uint_as_float((uint32_t)(ebc - 13 + g.tc_eu) << 23);       // 2^(E + eu - 14)
    const uint32_t lane = (uint32_t)((warp & 3) * 32) << 16;
    const f2 sc2 = pk(sc, sc);
    // all of the thread's amplitudes loaded first (the loads overlap), then split and stored
    float4 vv[NA];
#pragma unroll
    for (int a = 0; a < NA; a++) vv[a] = sm[spm ^ tsw[a]];
#pragma unroll
    for (int c = 0; c < NA / 4; c++) {   // four amplitudes, then one 4-column TMEM store per digit slice
        uint32_t w[6][4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const float4 v = vv[4 * c + a];
            f2 q[6];
            digits2(mul2(pk(v.x, v.y), sc2), mul2(pk(v.z, v.w), sc2), q);
#pragma unroll
            for (int j = 0; j < 6; j++) {
                const float2 d = up(q[j]);
                w[j][a] = __byte_perm(__float_as_uint(d.x), __float_as_uint(d.y), 0x7632);
            }
        }
#pragma unroll
        for (int j = 0; j < 6; j++) st4(st.tmem + lane + (uint32_t)(kA0 + 32 * j + NA * h + 4 * c), w[j]);
    }
    wait_st();
    fence_before();
    __syncthreads();
    fence_after();
    const uint64_t b0 = bdesc(su32(sB));
    // Round 4 (weights 4..6, 64 MMAs) into D0 by thread 0: first the 20 MMAs that read state digits 4
    // and 5, committed to barrier 5, so that D1, which takes their columns, is free once they have
    // completed; thread 128 then issues round 3 into D1 while thread 0 still issues round 4.  Two
    // issuers, each waiting only for the reads of its own accumulator: thread 0 runs D0 (rounds 4,
    // 1), thread 128 runs D1 (rounds 3, 2) and round 0 into D2, the columns of state digits 2 and 3,
    // which are free once rounds 4, 3 and 2 have completed.  Every warp folds the rounds in the order
    // 4, 3, 2, 1, 0 (smallest digit weights first), E collecting rounds 4 and 3 in FP32 and S rounds
    // 2, 1, 0 with their TwoSum errors into E.
    bool ok = true;
    if (tid == 0) {
        if (mbar_wait(st.bar, st.ph & 1u)) {
            fence_after();
            issue_pairs<4, 6, 4, 5, true>(st.tmem, 0u, b0);
            commit(st.bar + 40u);
            issue_pairs<4, 6, 0, 3, false>(st.tmem, 0u, b0);
            commit(st.bar + 8u);
        } else {
            ok = false;
        }
    } else if (tid == 128) {
        if (wait_bar1(st, 5)) issue_round<3>(st.tmem, kD1, b0, st.bar + 16u);
        else ok = false;
        if (gnext) *s_nsrc = slice_src(*gnext, pool, base);   // read back by this thread only
    }
    st.ph ^= 1u | (1u << 5);
    if (!ok) { *s_fail = 1; atomicExch(err, 1); }
    f2 S[NA], E[NA];
    const uint32_t tl = st.tmem + lane + (uint32_t)(2 * NA * h);
    // round 4 (D0)
    ok = wait_bar(st, 1, lane_id);
    if (ok) {
        fold<0>(tl, S, E);
        fence_before();
        __syncwarp();
        if (lane_id == 0) mbar_arrive(st.bar + 24u);
    }
    // round 3 (D1)
    if (ok) ok = wait_bar(st, 2, lane_id);
    if (ok) {
        fold<1>(tl + kD1, S, E);
        fence_before();
        __syncwarp();
        if (lane_id == 0) mbar_arrive(st.bar + 32u);
        // each issuer has already arrived for its own warp
        if (tid == 0) {
            if (wait_bar1(st, 3)) issue_round<1>(st.tmem, 0u, b0, st.bar + 8u);
            else ok = false;
        } else if (tid == 128) {
            if (wait_bar1(st, 4)) issue_round<2>(st.tmem, kD1, b0, st.bar + 16u);
            else ok = false;
        }
    }
    st.ph ^= (1u << 3) | (1u << 4);
    // round 2 (D1); once it has completed, round 0 goes into D2
    if (ok) ok = wait_bar(st, 2, lane_id);
    if (ok) {
        if (tid == 128) issue_round<0>(st.tmem, kD2, b0, st.bar + 48u);
        fold<2>(tl + kD1, S, E);
    }
    // round 1 (D0), round 0 (D2)
    if (ok) ok = wait_bar(st, 1, lane_id);
    if (ok) fold<3>(tl, S, E);
    if (ok) ok = wait_bar(st, 6, lane_id);
    if (ok) {
        // every MMA of this gate has completed: sB takes the next gate's digit slices
        if (tid == 128 && gnext) copy_slices(su32(sB), *s_nsrc, st.bar);
        fold<3>(tl + kD2, S, E);
    }
    st.pref = ok && gnext != nullptr;
    if (!ok) {
        *s_fail = 1;
        atomicExch(err, 1);
        return;
    }
    const f2 osc2 = pk(osc, osc);
    float mx = 0.f;   // largest |high word|: its exponent field is the largest exponent field
#pragma unroll
    for (int a = 0; a < NA; a++) {
        const f2 hs = add2(S[a], E[a]);
        const f2 ls = sub2(E[a], sub2(hs, S[a]));
        const float2 hh = up(mul2(hs, osc2)), ll = up(mul2(ls, osc2));
        sm[spm ^ tsw[a]] = make_float4(hh.x, hh.y, ll.x, ll.y);
        mx = fmaxf(mx, fmaxf(fabsf(hh.x), fabsf(hh.y)));
    }
    // the next fused gate's tile scale (read after the caller's barrier)
    const uint32_t eb = __reduce_max_sync(0xffffffffu, __float_as_uint(mx) & 0x7F800000u);
    if (lane_id == 0) s_wmax[warp] = eb;
}

}  // namespace tc
