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

// A butterfly of df32 adds leaves every lane with the same value (two_sum is exact, so a + b and b + a
// agree bit for bit).
__device__ __forceinline__ df32 warp_sum_df(df32 d)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const df32 other(__shfl_xor_sync(0xffffffffu, d.hi, o), __shfl_xor_sync(0xffffffffu, d.lo, o));
        d = d + other;
    }
    return d;
}

__device__ __forceinline__ bool df_gt(const df32& a, const df32& b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

__device__ __forceinline__ df32 df_from_double(double v)
{
    const float h = (float)v;
    return df32(h, (float)(v - (double)h));
}

__device__ __forceinline__ double df_to_double(const df32& d) { return (double)d.hi + (double)d.lo; }

// Block-wide double-float sum of NV df32 values per thread; result valid in thread 0.  `scratch`
// holds >= 32 * NV float2.
template <int NV> __device__ __forceinline__ void block_sum_df(const df32 (&vin)[NV], float2* scratch, df32 (&v)[NV])
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum_df(vin[k]);
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) scratch[wid * NV + k] = make_float2(v[k].hi, v[k].lo);
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const float2 s = lane < nw ? scratch[lane * NV + k] : make_float2(0.f, 0.f);
            v[k] = warp_sum_df(df32(s.x, s.y));
        }
    }
}

// grid_reduce (gb_common.cuh) for fp32 per-thread partials with double-float sums: per warp in fp32
// (as grid_reduce), across warps and CTAs in double-float (~44 significant bits), in CTA order (so
// deterministic); `finish` receives the totals as doubles.  partials: [NV][gridDim.x] 8-byte slots;
// scratch: >= 32 * NV doubles.  The last CTA's chain is all fp32 operations, where grid_reduce's
// fp64 chain waited on GB300's FP64 latency.
template <int NV, typename Finish>
__device__ __forceinline__ void grid_reduce_df(const float (&vin)[NV], double* partials, unsigned int* counter,
                                               double* scratch, Finish finish)
{
    __shared__ bool s_last;
    float2* part = reinterpret_cast<float2*>(partials);
    float2* sc = reinterpret_cast<float2*>(scratch);
    df32 w[NV], v[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) w[k] = df32(warp_sum(vin[k]), 0.f);
    // warp sums are exact fp32 butterflies, identical in every lane: only lane sums across warps remain
    {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
        __syncthreads();
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) sc[wid * NV + k] = make_float2(w[k].hi, 0.f);
        }
        __syncthreads();
        if (wid == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const float2 s = lane < nw ? sc[lane * NV + k] : make_float2(0.f, 0.f);
                v[k] = warp_sum_df(df32(s.x, s.y));
            }
        }
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) part[(size_t)k * gridDim.x + blockIdx.x] = make_float2(v[k].hi, v[k].lo);
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    df32 acc[NV];
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const float2 p = __ldcg(part + (size_t)k * gridDim.x + i);
            acc[k] += df32(p.x, p.y);
        }
    }
    df32 tot[NV];
    block_sum_df<NV>(acc, sc, tot);
    if (threadIdx.x == 0) {
        *counter = 0u;
        double t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] = df_to_double(tot[k]);
        finish(t);
    }
}

}  // namespace gb
