// Float-float ("double-single") arithmetic for complex128 states on GB300.
//
// GB300 issues FP64 FMA at ~2/clk/SM (~1.2 TFLOP/s), and FP64<->FP32 conversions
// at the same rate, while FP32 and INT32 issue at 128/clk/SM.  A complex128 gate
// applied with FP64 arithmetic is FP64-bound at ~2 TB/s.  The kernels here keep
// the state in HBM as complex128 and compute on the FP32 pipes with a float-float
// value x = h + l (|l| <= ulp(h)), which carries ~48 significant bits:
//   - double -> (h, l): integer bit extraction plus one int->float conversion,
//   - products: TwoProd via FMA (exact), sums: TwoSum (exact), small terms in FP32,
//   - (h, l) -> double: integer mantissa assembly (no FP64 instruction).
// Every intrinsic is an explicitly rounded __f*_rn form, so the compiler cannot
// contract or reassociate the error-free transforms.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

struct ff { float h, l; };
struct cff { float rh, rl, ih, il; };   // complex float-float

// ---------------------------------------------------------------- conversions

// double -> float-float.  h holds the top 24 mantissa bits (truncated), l the
// remaining 29 bits rounded to 24 (relative error <= 2^-48).  |x| < 2^-126 maps to 0.
__device__ __forceinline__ ff d2ff(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
    unsigned sign = hi32 & 0x80000000u;
    int e = (int)((hi32 >> 20) & 0x7ffu);
    int fe = e - 896;                                    // float biased exponent of h
    unsigned m23 = __funnelshift_l(lo32, hi32, 3) & 0x7fffffu;
    float h = __uint_as_float(sign | ((unsigned)fe << 23) | m23);
    float rf = __uint2float_rn(lo32 & 0x1fffffffu);     // remainder, 2^(e-1075) units
    int p = e - 948;                                     // biased exponent of 2^(e-1075)
    float sc = __uint_as_float(sign | ((unsigned)p << 23));
    float l = __fmul_rn(rf, sc);
    if (p < 1) l = 0.0f;
    if (fe < 1) { h = 0.0f; l = 0.0f; }
    return {h, l};
}

// float-float -> double (round-to-nearest of h + l, integer assembly).
__device__ __forceinline__ double ff2d(float h, float l) {
    // normalise so |l| <= ulp(h)/2
    float s = __fadd_rn(h, l);
    float t = __fsub_rn(l, __fsub_rn(s, h));
    h = s; l = t;
    unsigned hb = __float_as_uint(h);
    int eh = (int)((hb >> 23) & 0xffu);
    if (eh == 0) return 0.0;                             // zero (or float denormal: negligible)
    unsigned sign = hb & 0x80000000u;
    unsigned m24 = (hb & 0x7fffffu) | 0x800000u;
    // l in units of 2^(E_h - 52):  k = l * 2^(52 - E_h) = l * 2^(179 - eh)
    int ps = 306 - eh;                                   // biased exponent of 2^(179-eh)
    long long k = 0;
    if (ps <= 254) {
        float kl = __fmul_rn(l, __uint_as_float((unsigned)ps << 23));
        k = (long long)__float2int_rn(kl);
    }
    if (sign) k = -k;                                    // magnitude arithmetic
    long long mant = ((long long)m24 << 29) + k;         // in [2^52 - 2^28, 2^53)
    int ed = eh + 896;                                   // double biased exponent
    if (mant < (1LL << 52)) { mant <<= 1; ed -= 1; }
    unsigned long long bits = ((unsigned long long)sign << 32) | ((unsigned long long)ed << 52) |
                              ((unsigned long long)mant & 0xfffffffffffffULL);
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ cff load_c128(const double2& v) {
    ff r = d2ff(v.x), i = d2ff(v.y);
    return {r.h, r.l, i.h, i.l};
}
__device__ __forceinline__ double2 store_c128(const cff& v) {
    return make_double2(ff2d(v.rh, v.rl), ff2d(v.ih, v.il));
}

// Storage policy: complex128 (double2) or complex64 (float2) amplitudes, read into the
// float-float form used by reductions.  A float is exactly h with l = 0, so products
// and sums of complex64 inputs are carried at FP64-level accuracy.
template <bool C64> struct Elem;
template <> struct Elem<false> {
    using T = double2;
    static __device__ __forceinline__ cff load(const T& v) { return load_c128(v); }
    static __device__ __forceinline__ T store(const cff& c) { return store_c128(c); }
};
template <> struct Elem<true> {
    using T = float2;
    static __device__ __forceinline__ cff load(const T& v) { return {v.x, 0.f, v.y, 0.f}; }
    static __device__ __forceinline__ T store(const cff& c) {
        return make_float2(__fadd_rn(c.rh, c.rl), __fadd_rn(c.ih, c.il));
    }
};

// ---------------------------------------------------------------- accumulation
// Sum of exact products: s carries the running sum of the leading products with
// every rounding error recovered by TwoSum; c collects the error terms and the
// cross products (each already ~2^-24 of the leading term).
struct ffacc { float s, c; };

__device__ __forceinline__ void acc_first(ffacc& a, float ch, float cl, float xh, float xl) {
    a.s = __fmul_rn(ch, xh);
    float e = __fmaf_rn(ch, xh, -a.s);
    e = __fmaf_rn(ch, xl, e);
    a.c = __fmaf_rn(cl, xh, e);
}
__device__ __forceinline__ void acc_add(ffacc& a, float ch, float cl, float xh, float xl) {
    float p = __fmul_rn(ch, xh);
    float e = __fmaf_rn(ch, xh, -p);
    e = __fmaf_rn(ch, xl, e);
    e = __fmaf_rn(cl, xh, e);
    float t = __fadd_rn(a.s, p);
    float bb = __fsub_rn(t, a.s);
    float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    a.s = t;
    a.c = __fadd_rn(a.c, __fadd_rn(e, err));
}
// add a float-float value (no product)
__device__ __forceinline__ void acc_add_ff(ffacc& a, float xh, float xl) {
    float t = __fadd_rn(a.s, xh);
    float bb = __fsub_rn(t, a.s);
    float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bb)), __fsub_rn(xh, bb));
    a.s = t;
    a.c = __fadd_rn(a.c, __fadd_rn(xl, err));
}
__device__ __forceinline__ ff acc_done(const ffacc& a) {
    float s = __fadd_rn(a.s, a.c);
    return {s, __fsub_rn(a.c, __fsub_rn(s, a.s))};
}

// Two FP32 values in one aligned register pair (low half first), for the packed f32x2 instructions:
// one issue slot per pair instead of two, the same rounding (round to nearest even) per half.
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 up(f2 v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// complex MAC into two accumulators: (ar, ai) += m * x, m = (mrh+mrl) + i(mih+mil)
__device__ __forceinline__ void cmac_first(ffacc& ar, ffacc& ai, const cff& m, const cff& x) {
    acc_first(ar, m.rh, m.rl, x.rh, x.rl);
    acc_add(ar, -m.ih, -m.il, x.ih, x.il);
    acc_first(ai, m.rh, m.rl, x.ih, x.il);
    acc_add(ai, m.ih, m.il, x.rh, x.rl);
}
__device__ __forceinline__ void cmac(ffacc& ar, ffacc& ai, const cff& m, const cff& x) {
    acc_add(ar, m.rh, m.rl, x.rh, x.rl);
    acc_add(ar, -m.ih, -m.il, x.ih, x.il);
    acc_add(ai, m.rh, m.rl, x.ih, x.il);
    acc_add(ai, m.ih, m.il, x.rh, x.rl);
}
__device__ __forceinline__ cff cdone(const ffacc& ar, const ffacc& ai) {
    ff r = acc_done(ar), i = acc_done(ai);
    return {r.h, r.l, i.h, i.l};
}
// complex product m * x
__device__ __forceinline__ cff cmul(const cff& m, const cff& x) {
    ffacc ar, ai;
    cmac_first(ar, ai, m, x);
    return cdone(ar, ai);
}
__device__ __forceinline__ cff cneg(const cff& x) { return {-x.rh, -x.rl, -x.ih, -x.il}; }
// multiply by i^p (p = 0..3): exact component permutation
__device__ __forceinline__ cff cmul_ipow(const cff& x, int p) {
    switch (p & 3) {
        case 0: return x;
        case 1: return {-x.ih, -x.il, x.rh, x.rl};
        case 2: return {-x.rh, -x.rl, -x.ih, -x.il};
        default: return {x.ih, x.il, -x.rh, -x.rl};
    }
}

// ---------------------------------------------------------------- FP64-exact sums
// Running float-float sum for reductions (probabilities, expectations).
struct ffsum { float h, l; };
__device__ __forceinline__ void fsum_add(ffsum& a, float xh, float xl) {
    float t = __fadd_rn(a.h, xh);
    float bb = __fsub_rn(t, a.h);
    float err = __fadd_rn(__fsub_rn(a.h, __fsub_rn(t, bb)), __fsub_rn(xh, bb));
    float lo = __fadd_rn(a.l, __fadd_rn(xl, err));
    a.h = __fadd_rn(t, lo);
    a.l = __fsub_rn(lo, __fsub_rn(a.h, t));
}
