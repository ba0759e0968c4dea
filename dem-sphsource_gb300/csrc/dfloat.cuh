// Double-float ("float-float") arithmetic and compensated sums in FP32.
//
// Why: GB300's FP64 rate is a small fraction of its FP32 rate, but three
// places of the step cancel catastrophically in plain FP32:
//   * integrated state - x += v dt and v += a dt add increments 1e-4..1e-6 of
//     the value, so FP32 rounding biases the trajectory;
//   * the DEM overlap delta = r_i + r_j - |x_i - x_j| (1e-7..1e-6 m out of
//     ~1e-3 m): FP32 positions resolve it to ~1e-4 relative;
//   * list cutoffs, which must decide like the FP64 reference.
// A value is carried as an unevaluated sum hi + lo of two floats (~48-bit
// significand).  The error-free transforms are Knuth's TwoSum, Dekker's
// FastTwoSum and the FMA product error (fmaf); the compound operations follow
// the standard double-double algorithms (Hida, Li & Bailey) at float width.
// Everything here is plain IEEE float arithmetic; the build never uses
// --use_fast_math, so the compiler keeps every rounding step.
#pragma once
#include <cuda_runtime.h>

struct dfl {
    float hi, lo;
};

__host__ __device__ __forceinline__ dfl df_make(float hi, float lo = 0.f)
{
    dfl r;
    r.hi = hi;
    r.lo = lo;
    return r;
}

// Splits a double into hi + lo floats (host and device).
__host__ __device__ __forceinline__ dfl df_from_double(double x)
{
    const float hi = (float)x;
    return df_make(hi, (float)(x - (double)hi));
}
__host__ __device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dfl df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return df_make(s, e);
}
__device__ __forceinline__ dfl df_fast_two_sum(float a, float b)  // |a| >= |b|
{
    const float s = __fadd_rn(a, b);
    return df_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dfl df_two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return df_make(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b)
{
    dfl s = df_two_sum(a.hi, b.hi);
    const dfl t = df_two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = df_fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return df_make(-a.hi, -a.lo); }
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ dfl df_add_f(dfl a, float b)
{
    dfl s = df_two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    dfl p = df_two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
    p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
    return df_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dfl df_mul_f(dfl a, float b)
{
    dfl p = df_two_prod(a.hi, b);
    p.lo = __fmaf_rn(a.lo, b, p.lo);
    return df_fast_two_sum(p.hi, p.lo);
}
// a / b: float quotient plus one correction from the double-float remainder.
__device__ __forceinline__ dfl df_div(dfl a, dfl b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const dfl r = df_sub(a, df_mul_f(b, q1));
    return df_fast_two_sum(q1, __fdiv_rn(r.hi, b.hi));
}
// sqrt by one Newton correction of the float root: x + (a - x^2) / (2x).
__device__ __forceinline__ dfl df_sqrt(dfl a)
{
    if (!(a.hi > 0.f)) return df_make(0.f, 0.f);
    const float x = __fsqrt_rn(a.hi);
    const dfl r = df_sub(a, df_two_prod(x, x));
    return df_fast_two_sum(x, __fdiv_rn(r.hi, __fmul_rn(2.f, x)));
}
// Sign test of a normalised double-float.
__device__ __forceinline__ bool df_ge0(dfl a) { return a.hi > 0.f || (a.hi == 0.f && a.lo >= 0.f); }
__device__ __forceinline__ bool df_lt0(dfl a) { return !df_ge0(a); }

// Kahan-compensated FP32 accumulators.
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    // s carries the rounding error c in excess: the compensated total is s - c
    __device__ __forceinline__ float value() const { return __fsub_rn(s, c); }
};
struct KahanF3 {
    KahanF x, y, z;
    __device__ __forceinline__ void add(float3 v)
    {
        x.add(v.x);
        y.add(v.y);
        z.add(v.z);
    }
    __device__ __forceinline__ float3 sum() const { return make_float3(x.value(), y.value(), z.value()); }
};
