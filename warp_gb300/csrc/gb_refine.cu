// gb_refine.cu -- the high-precision pieces of the mixed-precision solve: the true residual
// r = b - A x with fp32 (or bf16) matrix values and a high-precision solution, its norm, and the
// solution update.
//
// The reference solves in the matrix scalar type only (warp/_src/optim/linear.py:934-1032, fp32
// here).  The mixed-precision drop-in keeps the fp32 Krylov loop of gb_krylov.cu as the inner
// solver and wraps it in iterative refinement: r = b - A x (this file), inner fp32 solve A d = r,
// x += d, until ||b - A x|| / ||b|| meets the tolerance.  The solution is stored in FP64 plus an
// interleaved (hi, lo) fp32 split; the residual product runs in double-float arithmetic
// (gb_df32.cuh) because GB300's FP64 rate is a small fraction of FP32.  An FP64-arithmetic
// variant of the same kernel is kept for verification (mode 1).
#include "gb_common.cuh"
#include "gb_df32.cuh"
#include "gb_spmv.cuh"

namespace gb {

// double-float glue for the SpMV core
template <> __device__ __forceinline__ df32 ldx<df32, float2>(const float2* p)
{
    const float2 v = __ldg(p);
    return df32(v.x, v.y);
}
template <> __device__ __forceinline__ df32 cvt<df32, float>(float v) { return df32(v, 0.f); }
template <> __device__ __forceinline__ df32 cvt<df32, __nv_bfloat16>(__nv_bfloat16 v)
{
    return df32(__bfloat162float(v), 0.f);
}
__device__ __forceinline__ df32 group_reduce(df32 v, int G)
{
    for (int o = G >> 1; o > 0; o >>= 1) {
        df32 w(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
        v = v + w;
    }
    return v;
}

template <int BR, typename AT> struct EpiResid {
    const float* b;
    double* r64;
    float* r32;
    float rr = 0.f, bb = 0.f;
    __device__ __forceinline__ static float hi_of(const df32& v) { return v.hi + v.lo; }
    __device__ __forceinline__ static float hi_of(double v) { return (float)v; }
    __device__ __forceinline__ static double to_d(const df32& v) { return (double)v.hi + (double)v.lo; }
    __device__ __forceinline__ static double to_d(double v) { return v; }
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float bi = b[i];
            const AT ri = AT(bi, 0.f) + (-pick<BR>(acc, lane_g));
            const float r = hi_of(ri);
            if (r64) r64[i] = to_d(ri);
            if (r32) r32[i] = r;
            rr += r * r;
            bb += bi * bi;
        }
    }
};

// FP64 arithmetic variant of the epilogue
template <int BR> struct EpiResid64 {
    const float* b;
    double* r64;
    float* r32;
    float rr = 0.f, bb = 0.f;
    __device__ __forceinline__ void operator()(int row, const double (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float bi = b[i];
            const double ri = (double)bi - pick<BR>(acc, lane_g);
            if (r64) r64[i] = ri;
            const float r = (float)ri;
            if (r32) r32[i] = r;
            rr += r * r;
            bb += bi * bi;
        }
    }
};

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_resid_df(int nrow, SpmvShape sh, const int* __restrict__ offsets,
                                                           const int* __restrict__ row_counts,
                                                           const int* __restrict__ columns,
                                                           const VT* __restrict__ values, const float2* __restrict__ x2,
                                                           const float* __restrict__ b, double* r64, float* r32,
                                                           double* norms, double* partials, unsigned int* counter,
                                                           int* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[64];
    EpiResid<BR, df32> epi{b, r64, r32};
    spmv_run<BR, BR, VT, float2, df32>(nrow, sh, offsets, row_counts, columns, values, x2, smem, status, epi);
    float v[2] = {epi.rr, epi.bb};
    grid_reduce_df<2>(v, partials, counter, s_red, [&](const double (&t)[2]) {
        norms[0] = t[0];
        norms[1] = t[1];
    });
}

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_resid64(int nrow, SpmvShape sh, const int* __restrict__ offsets,
                                                          const int* __restrict__ row_counts,
                                                          const int* __restrict__ columns,
                                                          const VT* __restrict__ values, const double* __restrict__ x,
                                                          const float* __restrict__ b, double* r64, float* r32,
                                                          double* norms, double* partials, unsigned int* counter,
                                                          int* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[64];
    EpiResid64<BR> epi{b, r64, r32};
    spmv_run<BR, BR, VT, double, double>(nrow, sh, offsets, row_counts, columns, values, x, smem, status, epi);
    float v[2] = {epi.rr, epi.bb};
    grid_reduce_df<2>(v, partials, counter, s_red, [&](const double (&t)[2]) {
        norms[0] = t[0];
        norms[1] = t[1];
    });
}

// x64 += alpha * d ; x2 = (hi, lo) split of x64
__global__ void k_update_x(int64_t n, double* __restrict__ x, float2* __restrict__ x2, const float* __restrict__ d,
                           double alpha)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = x[i];
        if (d) v += alpha * (double)d[i];
        x[i] = v;
        if (x2) {
            const float hi = (float)v;
            x2[i] = make_float2(hi, (float)(v - (double)hi));
        }
    }
}

template <int BR, typename VT>
static int launch_resid(int mode, int nrow, SpmvShape sh, const int* offsets, const int* row_counts,
                        const int* columns, const void* values, const double* x, const float2* x2, const float* b,
                        double* r64, float* r32, double* norms, double* partials, unsigned int* counter, int* status,
                        cudaStream_t stream)
{
    const size_t smem = spmv_smem_bytes<BR, BR, VT>(sh.rows, sh.cap, sh.stages);
    finalize_shape(sh, nrow, smem, offsets);
    if (mode == 0) {
        auto kern = k_resid_df<BR, VT>;
        if (smem > 48 * 1024) GB_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<sh.grid, SPMV_THREADS, smem, stream>>>(nrow, sh, offsets, row_counts, columns, (const VT*)values, x2, b,
                                                      r64, r32, norms, partials, counter, status);
    } else {
        auto kern = k_resid64<BR, VT>;
        if (smem > 48 * 1024) GB_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<sh.grid, SPMV_THREADS, smem, stream>>>(nrow, sh, offsets, row_counts, columns, (const VT*)values, x, b,
                                                      r64, r32, norms, partials, counter, status);
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb

using namespace gb;

// Scratch needed by gb_residual_f64: an arrival counter + per-CTA partials.
GB_API size_t gb_residual_f64_workspace_bytes(int block_dim, int nrow, int64_t nnz, int val_dtype)
{
    (void)block_dim;
    (void)nrow;
    (void)nnz;
    (void)val_dtype;
    return 256 + sizeof(double) * 2 * (size_t)(std::max(sm_count(), kSmCount) * 4) + 256;
}

// r = b - A x with A values fp32/bf16, b fp32 and a high-precision x.
//   mode 0: x2 = interleaved (hi, lo) fp32 split of x, double-float arithmetic (fast path);
//   mode 1: x = fp64 array, FP64 arithmetic (verification path).
// Writes r64 and/or r32 (either may be null) and norms[0] = ||r||^2, norms[1] = ||b||^2 (device
// doubles; accumulated per thread in fp32 and across threads in double-float).  The workspace's first 256
// bytes hold the arrival counter: zero before the first call, left zero by the kernel.
GB_API int gb_residual_f64(int block_dim, int nrow, int64_t nnz, int64_t ncap, const int* offsets,
                           const int* row_counts, const int* columns, const void* values, int val_dtype,
                           const double* x, const float* b, double* r64, float* r32, double* norms, void* workspace,
                           size_t workspace_bytes, int* status, cudaStream_t stream)
{
    GB_REQUIRE(block_dim == 1 || block_dim == 3, "residual_f64: block_dim must be 1 or 3");
    GB_REQUIRE(val_dtype == GB_F32 || val_dtype == GB_BF16, "residual_f64: values must be f32 or bf16");
    GB_REQUIRE(nrow > 0 && offsets && columns && values && x && b && norms && workspace && status,
               "residual_f64: null argument");
    GB_REQUIRE(workspace_bytes >= gb_residual_f64_workspace_bytes(block_dim, nrow, nnz, val_dtype),
               "residual_f64: workspace too small");
    const bool aligned = ((uintptr_t)columns % 16 == 0) && ((uintptr_t)values % 16 == 0);
    SpmvShape sh = default_shape(block_dim, block_dim, val_dtype, nrow, nnz, ncap, aligned);
    unsigned int* counter = static_cast<unsigned int*>(workspace);
    double* partials = reinterpret_cast<double*>(static_cast<unsigned char*>(workspace) + 256);
    if (block_dim == 1)
        return val_dtype == GB_BF16
                   ? launch_resid<1, __nv_bfloat16>(1, nrow, sh, offsets, row_counts, columns, values, x, nullptr, b,
                                                    r64, r32, norms, partials, counter, status, stream)
                   : launch_resid<1, float>(1, nrow, sh, offsets, row_counts, columns, values, x, nullptr, b, r64, r32,
                                            norms, partials, counter, status, stream);
    return val_dtype == GB_BF16
               ? launch_resid<3, __nv_bfloat16>(1, nrow, sh, offsets, row_counts, columns, values, x, nullptr, b, r64,
                                                r32, norms, partials, counter, status, stream)
               : launch_resid<3, float>(1, nrow, sh, offsets, row_counts, columns, values, x, nullptr, b, r64, r32,
                                        norms, partials, counter, status, stream);
}

// Same residual in double-float arithmetic from the (hi, lo) split x2 (float2 per dof).
GB_API int gb_residual_df(int block_dim, int nrow, int64_t nnz, int64_t ncap, const int* offsets,
                          const int* row_counts, const int* columns, const void* values, int val_dtype,
                          const void* x2, const float* b, double* r64, float* r32, double* norms, void* workspace,
                          size_t workspace_bytes, int* status, cudaStream_t stream)
{
    GB_REQUIRE(block_dim == 1 || block_dim == 3, "residual_df: block_dim must be 1 or 3");
    GB_REQUIRE(val_dtype == GB_F32 || val_dtype == GB_BF16, "residual_df: values must be f32 or bf16");
    GB_REQUIRE(nrow > 0 && offsets && columns && values && x2 && b && norms && workspace && status,
               "residual_df: null argument");
    GB_REQUIRE(workspace_bytes >= gb_residual_f64_workspace_bytes(block_dim, nrow, nnz, val_dtype),
               "residual_df: workspace too small");
    const bool aligned = ((uintptr_t)columns % 16 == 0) && ((uintptr_t)values % 16 == 0);
    SpmvShape sh = default_shape(block_dim, block_dim, val_dtype, nrow, nnz, ncap, aligned);
    unsigned int* counter = static_cast<unsigned int*>(workspace);
    double* partials = reinterpret_cast<double*>(static_cast<unsigned char*>(workspace) + 256);
    const float2* xs = static_cast<const float2*>(x2);
    if (block_dim == 1)
        return val_dtype == GB_BF16
                   ? launch_resid<1, __nv_bfloat16>(0, nrow, sh, offsets, row_counts, columns, values, nullptr, xs, b,
                                                    r64, r32, norms, partials, counter, status, stream)
                   : launch_resid<1, float>(0, nrow, sh, offsets, row_counts, columns, values, nullptr, xs, b, r64, r32,
                                            norms, partials, counter, status, stream);
    return val_dtype == GB_BF16
               ? launch_resid<3, __nv_bfloat16>(0, nrow, sh, offsets, row_counts, columns, values, nullptr, xs, b, r64,
                                                r32, norms, partials, counter, status, stream)
               : launch_resid<3, float>(0, nrow, sh, offsets, row_counts, columns, values, nullptr, xs, b, r64, r32,
                                        norms, partials, counter, status, stream);
}

// x64 += alpha * d32 (d may be null: only refresh the split); x2 (optional) = (hi, lo) split.
GB_API int gb_update_solution(int64_t n, double* x, void* x2, const float* d, double alpha, cudaStream_t stream)
{
    GB_REQUIRE(n >= 0 && (n == 0 || x), "update_solution: bad argument");
    if (n == 0) return GB_OK;
    const int grid = (int)std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 8);
    k_update_x<<<grid, 256, 0, stream>>>(n, x, static_cast<float2*>(x2), d, alpha);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// x64 += alpha * d32
GB_API int gb_axpy_f64_f32(int64_t n, double* x, const float* d, double alpha, cudaStream_t stream)
{
    return gb_update_solution(n, x, nullptr, d, alpha, stream);
}
