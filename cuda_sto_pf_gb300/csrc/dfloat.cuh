// dfloat.cuh — double-float arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2
// (about 48 significant bits).  Error-free transforms: Knuth's two-sum,
// Dekker's fast two-sum (|a| >= |b|) and the two-product through the fused
// multiply-add; the sums and products below follow the "sloppy" double-double
// forms of Hida, Li and Bailey (QD library paper, 2001), relative error a few
// units of 2^-48.  GB300 runs FP64 at 1/64 of the FP32 rate, so a per-cell
// evaluation that needs more than float precision is cheaper in this form
// than in double.
#pragma once

#include "dfexp.cuh"

struct dfl { float hi, lo; };

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b) {   // |a| >= |b| or a == 0
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_two_prod(float a, float b) {
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    dfl s = df_two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_add_f(dfl a, float b) {
    dfl s = df_two_sum(a.hi, b);
    s.lo += a.lo;
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    dfl p = df_two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return df_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dfl df_mul_f(dfl a, float b) {
    dfl p = df_two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return df_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
// 1 / d for d >= 1 (one Newton step from the float reciprocal: q0 + q0 (1 - d q0))
__device__ __forceinline__ dfl df_rcp(dfl d) {
    const float q0 = 1.0f / d.hi;
    float e = fmaf(-d.hi, q0, 1.0f);   // exact: q0 is the rounded quotient
    e = fmaf(-d.lo, q0, e);
    return df_fast_two_sum(q0, q0 * e);
}
__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ dfl df_from_double(double v) {
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

// e^w for -40 <= w <= 0 by Tang's table-driven method (ACM TOMS 15, 1989):
// w = N ln2/64 + r (N = 64 k + j, |r| <= ln2/128),
// e^r = 1 + r + r^2/2 + (r^3/6 + r^4/24 + r^5/120) with the bracket in
// float (below 2.7e-8, so its rounding is under 2^-48 of the result), times
// 2^(j/64) from the double-float table, times 2^k (exact).
// tab: dfexp::kExp2Tab staged in shared memory
__device__ __forceinline__ dfl df_exp_neg(dfl w, const float2 *tab) {
    // N = nearest integer to w.hi * 64/ln2 (-3694 .. 0) by the 1.5 * 2^23
    // shift: its float bits hold N, so no float <-> int conversion is issued
    const float tN = fmaf(w.hi, dfexp::kInvL64, 12582912.0f);
    const float fN = tN - 12582912.0f;
    const int N = __float_as_int(tN) - 0x4B400000;
    // w.hi - N C1 is exact (N C1 has 24 bits and is within a factor 2 of w.hi)
    dfl r = df_two_sum(fmaf(-fN, dfexp::kC1, w.hi), w.lo);
    r = df_add(r, df_neg(df_two_prod(fN, dfexp::kC2)));
    r = df_add_f(r, -fN * dfexp::kC3);
    const float rh = r.hi;
    const float tail = rh * rh * rh * (1.0f / 6.0f + rh * (1.0f / 24.0f + rh * (1.0f / 120.0f)));
    dfl q = df_two_prod(rh, rh);   // r^2 / 2 with the lo part of r
    q.lo = fmaf(2.0f * rh, r.lo, q.lo);
    q.hi *= 0.5f;
    q.lo *= 0.5f;
    dfl e = df_add_f(q, tail);
    e = df_add(e, r);
    e = df_add_f(e, 1.0f);
    const int j = N & 63, k = (N - j) / 64;   // N = 64 k + j, 0 <= j < 64, -58 <= k <= 0
    const float2 t = tab[j];
    e = df_mul(e, dfl{t.x, t.y});
    const float s = __int_as_float((127 + k) << 23);   // 2^k, a normal float
    return {e.hi * s, e.lo * s};
}

// sigmoid(z) = 1 / (1 + e^-z) of a double-float z; beyond |z| = 40 the
// float sigmoid (the double-float correction is below 4e-18 there)
__device__ __forceinline__ dfl df_sigmoid(dfl z, const float2 *tab) {
    if (!(fabsf(z.hi) <= 40.0f)) {
        const float zf = z.hi;
        const float s = zf >= 0.0f ? 1.0f / (1.0f + __expf(-zf)) : __expf(zf) / (1.0f + __expf(zf));
        return {s, 0.0f};
    }
    const bool pos = z.hi >= 0.0f;
    const dfl E = df_exp_neg(pos ? df_neg(z) : z, tab);   // e^-|z| <= 1
    const dfl r = df_rcp(df_add_f(E, 1.0f));
    return pos ? r : df_mul(E, r);
}
