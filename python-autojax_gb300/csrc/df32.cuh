// Double-float arithmetic: a value is hi + lo with two float32 words
// (about 48 significant bits, unit roundoff ~2^-47), evaluated on the float32
// pipe, which on GB300 issues ~62x more operations per clock than the float64
// pipe.  Products use the exact error term fma(a, b, -a*b); sums use the
// error-free TwoSum of Knuth; the lo*lo product (~2^-48 relative) is dropped.
// Compiled without fast-math, so nvcc keeps every rounding step (it only ever
// contracts a*b+c, which these formulas already write as fma).
#pragma once

#include <cuda_runtime.h>

namespace aj {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_from(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

// error-free sum: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// acc += a * b in 15 float32 operations: exact product error, TwoSum with the
// running hi, then renormalisation so the error stays ~2^-47 of the running sum
// over arbitrarily long reductions
__device__ __forceinline__ void df_fma_acc(df& acc, df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s, t;
    two_sum(acc.hi, p, s, t);
    t += acc.lo + e;
    acc.hi = s + t;
    acc.lo = t - (acc.hi - s);
}

// acc += a * b without renormalising (11 float32 operations): lo collects the
// TwoSum error and the product error; call df_renorm at least every 8 steps,
// after which the error is the same ~2^-46 of the running sum
__device__ __forceinline__ void df_fma_lazy(df& acc, df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    float s, t;
    two_sum(acc.hi, p, s, t);
    acc.hi = s;
    acc.lo += t + e;
}

__device__ __forceinline__ void df_renorm(df& a) {
    const float s = a.hi + a.lo;
    a.lo = a.lo - (s - a.hi);
    a.hi = s;
}

// acc -= a * b
__device__ __forceinline__ void df_fms_acc(df& acc, df a, df b) { df_fma_acc(acc, {-a.hi, -a.lo}, b); }

__device__ __forceinline__ df df_norm(df a) {
    const float s = a.hi + a.lo;
    return {s, a.lo - (s - a.hi)};
}

__device__ __forceinline__ df df_add(df a, df b) {
    float s, t;
    two_sum(a.hi, b.hi, s, t);
    t += a.lo + b.lo;
    return df_norm({s, t});
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

// a * b, renormalised
__device__ __forceinline__ df dfmul(df a, df b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return df_norm({p, e});
}

__device__ __forceinline__ df dfsqrt(df d) {
    const float y = sqrtf(d.hi);
    if (!(y > 0.f)) return {y, 0.f};
    const float p = y * y;
    const float e = fmaf(y, y, -p);
    const float diff = ((d.hi - p) - e) + d.lo;
    return df_norm({y, diff * (0.5f / y)});
}

__device__ __forceinline__ df dfrcp(df l) {
    const float r0 = 1.0f / l.hi;
    const float q = l.hi * r0;
    const float qe = fmaf(l.hi, r0, -q) + l.lo * r0;
    const float one_minus = (1.0f - q) - qe;
    return df_norm({r0, r0 * one_minus});
}

// 1/sqrt(d) to double-float accuracy: hardware rsqrt, one float Newton step,
// one double-float Newton step (no divisions on the critical path)
__device__ __forceinline__ df dfrsqrt(df d) {
    float r = rsqrtf(d.hi);
    r = r * fmaf(-0.5f * d.hi * r, r, 1.5f);
    const float q = r * r;
    const float qe = fmaf(r, r, -q);
    const df t = dfmul(d, {q, qe});
    const float h = (1.0f - t.hi) - t.lo;
    return df_norm({r, 0.5f * r * h});
}

}  // namespace aj
