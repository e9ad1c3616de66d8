// gb_df32.cuh -- double-float ("two-fp32") arithmetic for the true residual on GB300.
//
// GB300's FP64 pipe runs at a small fraction of its FP32 rate, so the FP64-accurate residual
// r = b - A x of the refinement loop is evaluated as unevaluated sums hi + lo of two fp32 numbers:
// products with the exact error of an FMA (Dekker/Kahan two-product) and sums with Knuth's
// two-sum.  Relative accuracy ~2^-44 per row (24+24 significand bits minus the few lost in the
// renormalisations), far below the 1e-8 residual target; verified against the FP64 oracle.
#pragma once
#include "gb_common.cuh"

namespace gb {

struct df32 {
    float hi, lo;
    __host__ __device__ df32() : hi(0.f), lo(0.f) {}
    __host__ __device__ df32(int v) : hi((float)v), lo(0.f) {}
    __host__ __device__ df32(float h, float l) : hi(h), lo(l) {}
};

__device__ __forceinline__ df32 two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return df32(s, e);
}

__device__ __forceinline__ df32 quick_two_sum(float a, float b)
{
    const float s = a + b;
    return df32(s, b - (s - a));
}

__device__ __forceinline__ df32 operator+(const df32& a, const df32& b)
{
    df32 s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return quick_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df32& operator+=(df32& a, const df32& b)
{
    a = a + b;
    return a;
}

__device__ __forceinline__ df32 operator*(const df32& a, const df32& b)
{
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}

__device__ __forceinline__ df32 operator-(const df32& a) { return df32(-a.hi, -a.lo); }

__device__ __forceinline__ bool operator!=(const df32& a, const df32& b) { return a.hi != b.hi || a.lo != b.lo; }

}  // namespace gb
