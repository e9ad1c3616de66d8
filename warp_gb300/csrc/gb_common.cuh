// gb_common.cuh -- shared helpers for the warp_gb300 CUDA library (sm_103a only).
//
// Error convention of the C ABI: every entry point returns 0 on success and a negative code on
// failure; the message is kept per host thread and returned by gb_last_error().  No C++
// exception crosses the ABI.  Device-side problems (a bounded wait that ran out, a capacity
// overflow) are reported through a device status word that the caller reads.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stdio.h>
#include <algorithm>
#include <utility>

#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ < 1000)
#error "warp_gb300 kernels are written for sm_103a (Blackwell) only"
#endif

#define GB_API extern "C" __attribute__((visibility("default")))

enum GbStatus : int {
    GB_OK = 0,
    GB_ERR_INVALID = -1,     // bad argument
    GB_ERR_CUDA = -2,        // a CUDA runtime call failed
    GB_ERR_UNSUPPORTED = -3, // valid but not implemented combination
    GB_ERR_CAPACITY = -4,    // a caller-provided buffer is too small
};

// Device status bits (gb_* kernels OR them into a caller-provided int32 word).
enum GbDeviceStatus : int {
    GB_DEV_WAIT_TIMEOUT = 1,  // a bounded mbarrier / flag wait gave up
    GB_DEV_BREAKDOWN = 2,     // Krylov breakdown (zero or non-finite denominator)
    GB_DEV_NONFINITE = 4,     // non-finite residual detected
    GB_DEV_STAGNATION = 8,    // flexible solver stagnated (fallback requested)
};

// Scalar type codes shared with the Python host side.
enum GbDtype : int {
    GB_F32 = 0,
    GB_F64 = 1,
    GB_BF16 = 2,
    GB_F16 = 3,
};

namespace gb {

void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t err, const char* what);

constexpr int kSmCount = 152;  // GB300: 2 dies x 76 SMs

// Programmatic dependent launch.  A kernel launched with launch_pdl() may be scheduled while the
// previous kernel of the stream drains; every such kernel calls pdl_enter() before its first global
// memory access: it lets its own successor be scheduled (launch_dependents) and then waits until its
// predecessor grid has completed and its writes are visible (wait).  Without the launch attribute both
// instructions are no-ops, so the same kernels may also be launched normally.  Launches into a
// capturing stream stay plain: inside a CUDA graph the early scheduling measured slower (1-2% on the
// graph-captured solves), while eager launch sequences gain (multigrid V-cycle 241 -> 203 us at 97^3).
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Process-wide switch (gb_set_pdl): whether a launch into a capturing / non-capturing stream gets
// the programmatic-serialization attribute.
bool pdl_enabled(bool capturing);

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                              Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t qerr = cudaStreamIsCapturing(stream, &cap);
    if (qerr != cudaSuccess) (void)cudaGetLastError();  // the query's own error; the launch reports its own
    const bool capturing = qerr != cudaSuccess || cap != cudaStreamCaptureStatusNone;
    cfg.numAttrs = pdl_enabled(capturing) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

template <typename T> __host__ __device__ inline T ceil_div(T a, T b) { return (a + b - 1) / b; }

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return (double)v; }
__device__ __forceinline__ double to_f64(__nv_bfloat16 v) { return (double)__bfloat162float(v); }

template <typename T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over groups of G consecutive lanes (G a power of two <= 32); every lane gets its group's sum.
template <int G, typename T> __device__ __forceinline__ T group_sum(T v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NV values; result valid in thread 0.  `scratch` holds >= 32*NV doubles.
// Per-warp sums run in the input type (fp32 per-thread partials keep the FP64 pipe, a small
// fraction of the FP32 rate on GB300, out of the element loops); cross-warp sums in fp64.
template <int NV, typename T> __device__ __forceinline__ void block_sum(T (&vin)[NV], double* scratch, double (&v)[NV])
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = (double)warp_sum(vin[k]);
    __syncthreads();
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) scratch[wid * NV + k] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = (lane < nw) ? scratch[lane * NV + k] : 0.0;
            v[k] = warp_sum(s);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Single-pass grid reduction ("last block done"): every CTA publishes NV partial sums, the last
// CTA to arrive sums all partials in CTA-index order (deterministic regardless of arrival order)
// and runs `finish(total)` on thread 0.  The arrival counter is reset by the last CTA so the
// same buffers serve every launch of a captured graph.  No CTA ever waits on another.
// partials: [NV][gridDim.x] doubles; counter: one unsigned int, zero before the first launch.
// ---------------------------------------------------------------------------------------------
template <int NV, typename T, typename Finish>
__device__ __forceinline__ void grid_reduce(T (&vin)[NV], double* partials, unsigned int* counter,
                                            double* scratch, Finish finish)
{
    __shared__ bool s_last;
    double v[NV];
    block_sum<NV>(vin, scratch, v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partials[(size_t)k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&partials[(size_t)k * gridDim.x + i]);
    }
    double tot[NV];
    block_sum<NV>(acc, scratch, tot);
    if (threadIdx.x == 0) {
        *counter = 0u;
        finish(tot);
    }
}

}  // namespace gb

#define GB_CHECK_CUDA(expr)                                                                                   \
    do {                                                                                                      \
        cudaError_t _e = (expr);                                                                              \
        if (_e != cudaSuccess) return gb::cuda_fail(_e, #expr);                                               \
    } while (0)

#define GB_REQUIRE(cond, ...)                                                                                 \
    do {                                                                                                      \
        if (!(cond)) {                                                                                        \
            gb::set_error(__VA_ARGS__);                                                                       \
            return GB_ERR_INVALID;                                                                            \
        }                                                                                                     \
    } while (0)
