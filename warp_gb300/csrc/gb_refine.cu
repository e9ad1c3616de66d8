// gb_refine.cu -- FP64 pieces of the mixed-precision solve: the true residual r = b - A x with
// fp32 (or bf16) matrix values and an fp64 solution, its norm, and the fp64 solution update.
//
// The reference solves in the matrix scalar type only (warp/_src/optim/linear.py:934-1032, fp32
// here).  The mixed-precision drop-in keeps the fp32 Krylov loop of gb_krylov.cu as the inner
// solver and wraps it in iterative refinement: r64 = b - A x64 (this file), inner fp32 solve
// A d = r64 (cast to fp32), x64 += d, until ||b - A x64|| / ||b|| meets the fp64 tolerance.
#include "gb_common.cuh"
#include "gb_spmv.cuh"

namespace gb {

template <int BR> struct EpiResid64 {
    const float* b;
    double* r64;
    float* r32;
    double rr = 0, bb = 0;
    __device__ __forceinline__ void operator()(int row, const double (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const double bi = (double)b[i];
            const double ri = bi - pick<BR>(acc, lane_g);
            if (r64) r64[i] = ri;
            if (r32) r32[i] = (float)ri;
            rr += ri * ri;
            bb += bi * bi;
        }
    }
};

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
    spmv_tile<BR, BR, VT, double, double>(nrow, sh, offsets, row_counts, columns, values, x, smem, status, epi);
    double v[2] = {epi.rr, epi.bb};
    grid_reduce<2>(v, partials, counter, s_red, [&](const double (&t)[2]) {
        norms[0] = t[0];
        norms[1] = t[1];
    });
}

__global__ void k_axpy_f64_f32(int64_t n, double* __restrict__ x, const float* __restrict__ d, double alpha)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += alpha * (double)d[i];
}

template <int BR, typename VT>
static int launch_resid(int nrow, SpmvShape sh, const int* offsets, const int* row_counts, const int* columns,
                        const void* values, const double* x, const float* b, double* r64, float* r32, double* norms,
                        double* partials, unsigned int* counter, int* status, cudaStream_t stream)
{
    const size_t smem = spmv_smem_bytes<BR, BR, VT>(sh.rows, sh.cap);
    auto kern = k_resid64<BR, VT>;
    if (smem > 48 * 1024) GB_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<ceil_div(nrow, sh.rows), SPMV_THREADS, smem, stream>>>(nrow, sh, offsets, row_counts, columns,
                                                                 (const VT*)values, x, b, r64, r32, norms, partials,
                                                                 counter, status);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb

using namespace gb;

// Scratch needed by gb_residual_f64: partials (doubles) + an arrival counter.
GB_API size_t gb_residual_f64_workspace_bytes(int block_dim, int nrow, int64_t nnz, int val_dtype)
{
    SpmvShape sh = default_shape(block_dim, block_dim, val_dtype, nrow, nnz, nnz, true);
    return 256 + sizeof(double) * 2 * (size_t)ceil_div(std::max(nrow, 1), sh.rows) + 256;
}

// r = b - A x in fp64 (x fp64, b fp32, A values fp32 or bf16).  Writes r64 and/or r32 (either
// may be null) and norms[0] = ||r||^2, norms[1] = ||b||^2 (device doubles).  The workspace's
// first 256 bytes hold the arrival counter and must be zero before the first call (the kernel
// leaves it zero).
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
                   ? launch_resid<1, __nv_bfloat16>(nrow, sh, offsets, row_counts, columns, values, x, b, r64, r32,
                                                    norms, partials, counter, status, stream)
                   : launch_resid<1, float>(nrow, sh, offsets, row_counts, columns, values, x, b, r64, r32, norms,
                                            partials, counter, status, stream);
    return val_dtype == GB_BF16
               ? launch_resid<3, __nv_bfloat16>(nrow, sh, offsets, row_counts, columns, values, x, b, r64, r32, norms,
                                                partials, counter, status, stream)
               : launch_resid<3, float>(nrow, sh, offsets, row_counts, columns, values, x, b, r64, r32, norms,
                                        partials, counter, status, stream);
}

// x64 += alpha * d32
GB_API int gb_axpy_f64_f32(int64_t n, double* x, const float* d, double alpha, cudaStream_t stream)
{
    GB_REQUIRE(n >= 0 && (n == 0 || (x && d)), "axpy_f64_f32: bad argument");
    if (n == 0) return GB_OK;
    const int grid = (int)std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 8);
    k_axpy_f64_f32<<<grid, 256, 0, stream>>>(n, x, d, alpha);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
