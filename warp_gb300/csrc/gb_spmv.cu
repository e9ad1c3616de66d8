// gb_spmv.cu -- y = alpha * A x + beta * y for BSR matrices (bsr_mv).
//
// Replaces the JIT kernels bsr_mv_kernel / bsr_mv_tiled_kernel / bsr_mv_transpose_kernel
// launched by warp/_src/sparse.py:4792-4913 (kernels :4627-4747).  1x1 and 3x3 blocks (the
// shapes of the Q1 scalar and vector spaces) use the staged row-tile kernel of gb_spmv.cuh;
// other block shapes use a one-thread-per-scalar-row kernel like the reference's.
#include "gb_common.cuh"
#include "gb_spmv.cuh"

namespace gb {

template <int BR, typename XT, typename AT> struct EpiAxpby {
    XT* y_out;
    const XT* y_in;
    AT alpha, beta;
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            AT v = alpha * pick<BR>(acc, lane_g);
            if (beta != AT(0)) v += beta * (AT)y_in[i];
            y_out[i] = (XT)v;
        }
    }
};

template <int BR, int BC, typename VT, typename XT, typename AT>
__global__ __launch_bounds__(SPMV_THREADS) void k_bsr_mv(int nrow, SpmvShape sh, const int* __restrict__ offsets,
                                                         const int* __restrict__ row_counts,
                                                         const int* __restrict__ columns,
                                                         const VT* __restrict__ values, const XT* __restrict__ x,
                                                         const XT* y_in, XT* y_out, AT alpha, AT beta, int* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_enter();
    EpiAxpby<BR, XT, AT> epi{y_out, y_in, alpha, beta};
    spmv_run<BR, BC, VT, XT, AT>(nrow, sh, offsets, row_counts, columns, values, x, smem, status, epi);
}

// z_out = z + omega * dinv * (r - A z): one damped Jacobi step fused with its residual product
template <int BR> struct EpiSmooth {
    const float *z, *r, *dinv;
    float omega;
    float* z_out;
    __device__ __forceinline__ void operator()(int row, const float (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            z_out[i] = z[i] + omega * dinv[i] * (r[i] - pick<BR>(acc, lane_g));
        }
    }
};

// Block-Jacobi step on 3x3 block rows: z_out_i = z_i + omega Dinv_i (r - A z)_i, Dinv_i the inverse of the
// row's diagonal block (9 floats, row-major); every lane of the row's group holds all 3 sums.
struct EpiSmoothBlock3 {
    const float *z, *r, *dinv;
    float omega;
    float* z_out;
    __device__ __forceinline__ void operator()(int row, const float (&acc)[3], int lane_g)
    {
        if (lane_g < 3) {
            const size_t b = (size_t)row * 3;
            const float* d = dinv + (size_t)row * 9 + 3 * lane_g;
            const float t0 = r[b] - acc[0], t1 = r[b + 1] - acc[1], t2 = r[b + 2] - acc[2];
            z_out[b + lane_g] = z[b + lane_g] + omega * (d[0] * t0 + d[1] * t1 + d[2] * t2);
        }
    }
};

template <typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_bsr_block_smooth3(int nrow, SpmvShape sh,
                                                                    const int* __restrict__ offsets,
                                                                    const int* __restrict__ columns,
                                                                    const VT* __restrict__ values, const float* z,
                                                                    const float* r, const float* dinv, float omega,
                                                                    float* z_out, int* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_enter();
    EpiSmoothBlock3 epi{z, r, dinv, omega, z_out};
    spmv_run<3, 3, VT, float, float>(nrow, sh, offsets, nullptr, columns, values, z, smem, status, epi);
}

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_bsr_smooth(int nrow, SpmvShape sh, const int* __restrict__ offsets,
                                                             const int* __restrict__ columns,
                                                             const VT* __restrict__ values, const float* z,
                                                             const float* r, const float* dinv, float omega,
                                                             float* z_out, int* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_enter();
    EpiSmooth<BR> epi{z, r, dinv, omega, z_out};
    spmv_run<BR, BR, VT, float, float>(nrow, sh, offsets, nullptr, columns, values, z, smem, status, epi);
}

// alpha == 0: y_out = beta * y_in without reading A or x (reference semantics, sparse.py:4649).
template <typename XT, typename AT>
__global__ void k_scale(int64_t n, const XT* y_in, XT* y_out, AT beta)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y_out[i] = (beta != AT(0)) ? (XT)(beta * (AT)y_in[i]) : XT(0);
}

// Generic block shapes: one thread per scalar row, as bsr_mv_kernel (sparse.py:4627-4665).
template <typename VT, typename XT, typename AT>
__global__ void k_bsr_mv_generic(int nrow, int br, int bc, const int* __restrict__ offsets,
                                 const int* __restrict__ row_counts, const int* __restrict__ columns,
                                 const VT* __restrict__ values, const XT* __restrict__ x, const XT* y_in, XT* y_out,
                                 AT alpha, AT beta)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nrow * br) return;
    const int row = (int)(t / br), sub = (int)(t - (int64_t)row * br);
    const int beg = offsets[row];
    const int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
    AT v = AT(0);
    for (int b = beg; b < end; ++b) {
        const int xs = columns[b] * bc;
        for (int c = 0; c < bc; ++c) v += cvt<AT>(values[((size_t)b * br + sub) * bc + c]) * (AT)x[xs + c];
    }
    v *= alpha;
    if (beta != AT(0)) v += beta * (AT)y_in[t];
    y_out[t] = (XT)v;
}

// Transposed product y += alpha * A^T x with atomics (non-deterministic, as the reference's
// bsr_mv_transpose_kernel, sparse.py:4718-4747).  y must already hold beta * y.
template <typename VT, typename XT, typename AT>
__global__ void k_bsr_mv_transpose(int nrow, int br, int bc, const int* __restrict__ offsets,
                                   const int* __restrict__ row_counts, const int* __restrict__ columns,
                                   const VT* __restrict__ values, const XT* __restrict__ x, XT* y, AT alpha)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nrow * bc) return;
    const int row = (int)(t / bc), j = (int)(t - (int64_t)row * bc);
    const int beg = offsets[row];
    const int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
    for (int b = beg; b < end; ++b) {
        AT s = AT(0);
        for (int i = 0; i < br; ++i) s += cvt<AT>(values[((size_t)b * br + i) * bc + j]) * (AT)x[(size_t)row * br + i];
        atomicAdd(&y[(size_t)columns[b] * bc + j], (XT)(alpha * s));
    }
}

template <int BR, int BC, typename VT, typename XT, typename AT>
static int launch_mv(int nrow, SpmvShape sh, const int* offsets, const int* row_counts, const int* columns,
                     const void* values, const void* x, const void* y_in, void* y_out, double alpha, double beta,
                     int* status, cudaStream_t stream)
{
    const size_t smem = spmv_smem_bytes<BR, BC, VT>(sh.rows, sh.cap, sh.stages);
    finalize_shape(sh, nrow, smem, offsets);
    auto kern = k_bsr_mv<BR, BC, VT, XT, AT>;
    static size_t attr_bytes = 48 * 1024;  // per instantiation: raise the limit only when a launch needs more
    if (smem > attr_bytes) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_bytes = smem;
    }
    GB_CHECK_CUDA(launch_pdl(kern, sh.grid, SPMV_THREADS, smem, stream, nrow, sh, offsets, row_counts, columns,
                             (const VT*)values, (const XT*)x, (const XT*)y_in, (XT*)y_out, (AT)alpha, (AT)beta, status));
    return GB_OK;
}

int sm_count()
{
    static int count = 0;
    if (count == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || count <= 0)
            count = kSmCount;
    }
    return count;
}

// Default tile shape (the autotuner in warp_gb300.tuning may override it per matrix): G lanes per
// block row so that each lane handles ~3-4 blocks; tiles of ~24-32 KB of staged data; 3 stages.
SpmvShape default_shape(int br, int bc, int val_dtype, int nrow, int64_t nnzb, int64_t ncap, bool aligned)
{
    SpmvShape sh;
    const double avg = nrow > 0 ? (double)nnzb / (double)nrow : 0.0;
    const int bb = br * bc;
    const int vbytes = (val_dtype == GB_F64) ? 8 : (val_dtype == GB_BF16 ? 2 : 4);
    // Tile shapes measured on GB300 (sweep over lanes per row x rows per tile on the 96^3 Q1
    // scalar and 64^3 / 128^3 Q1 vector matrices): scalar blocks run best with ~28 KB tiles (two CTAs
    // of 17 warps per SM, 3-deep rings) and 4 lanes per row; 3x3 blocks with ~70-80 KB tiles (one CTA
    // per SM): 8 lanes per block row at 64 rows (fp32), 4 at 128 rows (bf16).  Long rows get more lanes
    // (<= 8 blocks per lane).
    int G, rows;
    const double bytes_per_row = std::max(avg, 1.0) * (4.0 + bb * vbytes);
    if (bb == 1) {
        rows = 128;
        while (rows > 4 && rows * bytes_per_row * 1.05 > 36 * 1024) rows >>= 1;
        G = std::max(1, SPMV_CONSUMERS / rows);
    } else {
        rows = 64;
        while (rows > 4 && rows * bytes_per_row * 1.05 > 104 * 1024) rows >>= 1;
        // smaller value types (bf16): grow the tile while it stays under ~80 KB; measured on the 128^3
        // elasticity matrix: bf16 values 128 rows x 4 lanes 294 us against 360 us at 64 x 8
        // (fp32 values stay at 64 rows x 8 lanes, the best of the same sweep)
        while (rows < 128 && 2.0 * rows * bytes_per_row * 1.05 <= 80 * 1024) rows <<= 1;
        G = rows >= 128 ? 4 : std::max(8, SPMV_CONSUMERS / (rows * 2));
    }
    while (G < 32 && avg > 8.0 * G) G <<= 1;
    G = std::min(G, 32);
    sh.G = G;
    sh.rows = rows;
    int cap = (int)(avg * rows * 1.05) + 2 * SPMV_ALIGN + 16;
    cap = (cap + SPMV_ALIGN - 1) & ~(SPMV_ALIGN - 1);
    sh.cap = aligned ? cap : 0;
    const size_t stage = align16((size_t)(rows + 8) * 4) + align16((size_t)cap * 4) + align16((size_t)cap * bb * vbytes);
    sh.stages = (3 * stage <= 220 * 1024) ? 3 : 2;
    sh.grid = 0;
    sh.off_bulk = 0;
    sh.ncap = ncap;
    return sh;
}

void finalize_shape(SpmvShape& sh, int nrow, size_t smem_bytes, const int* offsets)
{
    sh.rows = std::max(4, (sh.rows + 3) & ~3);
    sh.cap = std::max(0, sh.cap & ~(SPMV_ALIGN - 1));
    sh.stages = std::min(std::max(sh.stages, 1), SPMV_MAX_STAGES);
    sh.off_bulk = ((uintptr_t)offsets % 16 == 0) ? 1 : 0;
    const int ntiles = std::max(1, ceil_div(nrow, sh.rows));
    int per_sm = (int)std::max<size_t>(1, (size_t)(227 * 1024) / std::max<size_t>(smem_bytes + 1024, 1));
    per_sm = std::min(per_sm, 2048 / SPMV_THREADS);
    per_sm = std::min(per_sm, 4);
    sh.grid = std::min(ntiles, sm_count() * per_sm);
}

}  // namespace gb

using namespace gb;

// y_out = alpha * A x + beta * y_in (y_in may equal y_out; x must not alias y_out).
// Replaces bsr_mv (warp/_src/sparse.py:4792-4913).  val_dtype: GB_F32 / GB_F64 / GB_BF16;
// vec_dtype: GB_F32 / GB_F64 (x and y).  ncap: entries available in columns/values.
// rows_per_cta / lanes_per_row / cap_blocks <= 0 select the built-in heuristic.
GB_API int gb_bsr_mv(int block_rows, int block_cols, int nrow, int ncol, int64_t nnz_upper, int64_t ncap,
                     const int* offsets, const int* row_counts, const int* columns, const void* values,
                     int val_dtype, const void* x, const void* y_in, void* y_out, int vec_dtype, double alpha,
                     double beta, int transpose, int rows_per_cta, int lanes_per_row, int cap_blocks, int* status,
                     cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0 && ncol >= 0, "bsr_mv: negative size");
    GB_REQUIRE(block_rows >= 1 && block_cols >= 1, "bsr_mv: bad block shape");
    GB_REQUIRE(status != nullptr, "bsr_mv: status word required");
    const int br = block_rows, bc = block_cols;
    const int64_t ny = (int64_t)(transpose ? ncol * bc : nrow * br);
    if (ny == 0) return GB_OK;
    if (alpha == 0.0 || nrow == 0) {
        const int grid = (int)std::min<int64_t>(ceil_div<int64_t>(ny, 256), kSmCount * 8);
        if (vec_dtype == GB_F32) k_scale<float, float><<<grid, 256, 0, stream>>>(ny, (const float*)y_in, (float*)y_out, (float)beta);
        else k_scale<double, double><<<grid, 256, 0, stream>>>(ny, (const double*)y_in, (double*)y_out, beta);
        GB_CHECK_CUDA(cudaGetLastError());
        return GB_OK;
    }
    GB_REQUIRE(offsets && columns && values && x && y_out, "bsr_mv: null pointer");

    if (transpose) {
        const int grid_s = (int)std::min<int64_t>(ceil_div<int64_t>(ny, 256), kSmCount * 8);
        if (vec_dtype == GB_F32) k_scale<float, float><<<grid_s, 256, 0, stream>>>(ny, (const float*)y_in, (float*)y_out, (float)beta);
        else k_scale<double, double><<<grid_s, 256, 0, stream>>>(ny, (const double*)y_in, (double*)y_out, beta);
        const int grid = (int)ceil_div<int64_t>((int64_t)nrow * bc, 256);
        if (val_dtype == GB_F32 && vec_dtype == GB_F32)
            k_bsr_mv_transpose<float, float, float><<<grid, 256, 0, stream>>>(nrow, br, bc, offsets, row_counts, columns,
                                                                             (const float*)values, (const float*)x,
                                                                             (float*)y_out, (float)alpha);
        else if (val_dtype == GB_F64 && vec_dtype == GB_F64)
            k_bsr_mv_transpose<double, double, double><<<grid, 256, 0, stream>>>(
                nrow, br, bc, offsets, row_counts, columns, (const double*)values, (const double*)x, (double*)y_out,
                alpha);
        else {
            gb::set_error("bsr_mv transpose: unsupported dtype combination");
            return GB_ERR_UNSUPPORTED;
        }
        GB_CHECK_CUDA(cudaGetLastError());
        return GB_OK;
    }

    const bool aligned = ((uintptr_t)columns % 16 == 0) && ((uintptr_t)values % 16 == 0);
    SpmvShape sh = default_shape(br, bc, val_dtype, nrow, nnz_upper, ncap, aligned);
    if (rows_per_cta > 0) sh.rows = rows_per_cta;
    if (lanes_per_row > 0) sh.G = lanes_per_row;
    if (cap_blocks >= 0 && (rows_per_cta > 0 || cap_blocks > 0)) sh.cap = aligned ? (cap_blocks & ~(SPMV_ALIGN - 1)) : 0;
    GB_REQUIRE(sh.G >= 1 && sh.G <= 32 && (sh.G & (sh.G - 1)) == 0, "bsr_mv: lanes_per_row must be a power of two <= 32");
    GB_REQUIRE(sh.rows >= 1 && sh.rows <= 4096, "bsr_mv: rows_per_cta out of range");
    {
        const int vb = (val_dtype == GB_F64) ? 8 : (val_dtype == GB_BF16 ? 2 : 4);
        const size_t stage = align16((size_t)(sh.rows + 8) * 4) + align16((size_t)sh.cap * 4) +
                             align16((size_t)sh.cap * br * bc * vb);
        // ring of up to 3 stages within the 227 KB per-CTA limit
        sh.stages = (int)std::min<size_t>((size_t)sh.stages, (227 * 1024 - 256) / std::max<size_t>(stage, 1));
        GB_REQUIRE(sh.stages >= 1, "bsr_mv: tile does not fit shared memory (rows %d, cap %d)", sh.rows, sh.cap);
    }

    if (br == 1 && bc == 1) {
        if (val_dtype == GB_F32 && vec_dtype == GB_F32)
            return launch_mv<1, 1, float, float, float>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
        if (val_dtype == GB_BF16 && vec_dtype == GB_F32)
            return launch_mv<1, 1, __nv_bfloat16, float, float>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
        if (val_dtype == GB_F32 && vec_dtype == GB_F64)
            return launch_mv<1, 1, float, double, double>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
        if (val_dtype == GB_F64 && vec_dtype == GB_F64)
            return launch_mv<1, 1, double, double, double>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
    } else if (br == 3 && bc == 3) {
        if (val_dtype == GB_F32 && vec_dtype == GB_F32)
            return launch_mv<3, 3, float, float, float>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
        if (val_dtype == GB_BF16 && vec_dtype == GB_F32)
            return launch_mv<3, 3, __nv_bfloat16, float, float>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
        if (val_dtype == GB_F32 && vec_dtype == GB_F64)
            return launch_mv<3, 3, float, double, double>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
        if (val_dtype == GB_F64 && vec_dtype == GB_F64)
            return launch_mv<3, 3, double, double, double>(nrow, sh, offsets, row_counts, columns, values, x, y_in, y_out, alpha, beta, status, stream);
    }
    // generic shapes
    const int grid = (int)ceil_div<int64_t>((int64_t)nrow * br, 256);
    if (val_dtype == GB_F32 && vec_dtype == GB_F32)
        k_bsr_mv_generic<float, float, float><<<grid, 256, 0, stream>>>(nrow, br, bc, offsets, row_counts, columns,
                                                                       (const float*)values, (const float*)x,
                                                                       (const float*)y_in, (float*)y_out, (float)alpha,
                                                                       (float)beta);
    else if (val_dtype == GB_F64 && vec_dtype == GB_F64)
        k_bsr_mv_generic<double, double, double><<<grid, 256, 0, stream>>>(nrow, br, bc, offsets, row_counts,
                                                                          columns, (const double*)values,
                                                                          (const double*)x, (const double*)y_in,
                                                                          (double*)y_out, alpha, beta);
    else if (val_dtype == GB_F32 && vec_dtype == GB_F64)
        k_bsr_mv_generic<float, double, double><<<grid, 256, 0, stream>>>(nrow, br, bc, offsets, row_counts, columns,
                                                                         (const float*)values, (const double*)x,
                                                                         (const double*)y_in, (double*)y_out, alpha,
                                                                         beta);
    else {
        gb::set_error("bsr_mv: unsupported dtype combination (values %d, vectors %d)", val_dtype, vec_dtype);
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// y -= A x for fp32 1x1 / 3x3 matrices without staging (used by the Dirichlet projection).
int gb_bsr_mv_internal(int bdim, int nrow, const int* offsets, const int* columns, const float* values,
                       const float* x, float* y, cudaStream_t stream)
{
    SpmvShape sh = default_shape(bdim, bdim, GB_F32, nrow, 0, 0, false);
    sh.rows = 64;
    sh.G = 8;
    sh.cap = 0;
    sh.stages = 1;
    if (bdim == 1)
        return launch_mv<1, 1, float, float, float>(nrow, sh, offsets, nullptr, columns, values, x, y, y, -1.0, 1.0,
                                                   nullptr, stream);
    return launch_mv<3, 3, float, float, float>(nrow, sh, offsets, nullptr, columns, values, x, y, y, -1.0, 1.0,
                                               nullptr, stream);
}

// One damped Jacobi step fused with its residual product: z_out = z + omega * D^-1 (r - A z)
// (no reference counterpart; the multigrid smoother of the flexible-CG preconditioner).
// z_out must not alias z.  fp32 vectors; fp32 or bf16 values (val_dtype); 1x1 or 3x3 blocks.
template <int BR, typename VT>
static int launch_smooth(int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* columns, const VT* values,
                         const float* r, const float* z, const float* dinv, float omega, float* z_out, int* status,
                         int val_dtype, cudaStream_t stream)
{
    const bool aligned = ((uintptr_t)columns % 16 == 0) && ((uintptr_t)values % 16 == 0);
    SpmvShape sh = default_shape(BR, BR, val_dtype, nrow, nnz, ncap, aligned);
    const size_t smem = spmv_smem_bytes<BR, BR, VT>(sh.rows, sh.cap, sh.stages);
    finalize_shape(sh, nrow, smem, offsets);
    static size_t attr_bytes = 48 * 1024;  // raised only when a launch needs more
    if (smem > attr_bytes) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_bsr_smooth<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_bytes = smem;
    }
    GB_CHECK_CUDA(launch_pdl(k_bsr_smooth<BR, VT>, sh.grid, SPMV_THREADS, smem, stream, nrow, sh, offsets, columns,
                             values, z, r, dinv, omega, z_out, status));
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

template <typename VT>
static int launch_block_smooth3(int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* columns,
                                const VT* values, const float* r, const float* z, const float* dinv, float omega,
                                float* z_out, int* status, int val_dtype, cudaStream_t stream)
{
    const bool aligned = ((uintptr_t)columns % 16 == 0) && ((uintptr_t)values % 16 == 0);
    SpmvShape sh = default_shape(3, 3, val_dtype, nrow, nnz, ncap, aligned);
    const size_t smem = spmv_smem_bytes<3, 3, VT>(sh.rows, sh.cap, sh.stages);
    finalize_shape(sh, nrow, smem, offsets);
    static size_t attr_bytes = 48 * 1024;  // raised only when a launch needs more
    if (smem > attr_bytes) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_bsr_block_smooth3<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_bytes = smem;
    }
    GB_CHECK_CUDA(launch_pdl(k_bsr_block_smooth3<VT>, sh.grid, SPMV_THREADS, smem, stream, nrow, sh, offsets, columns,
                             values, z, r, dinv, omega, z_out, status));
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// z_out = z + omega Dinv (r - A z) with Dinv the inverses of A's 3x3 diagonal blocks (gb_bsr_block_inverse_diagonal3).
GB_API int gb_bsr_block_jacobi_smooth3(int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* columns,
                                       const void* values, int val_dtype, const float* r, const float* z,
                                       const float* dinv_blocks, float omega, float* z_out, int* status,
                                       cudaStream_t stream)
{
    GB_REQUIRE(val_dtype == GB_F32 || val_dtype == GB_BF16, "block_jacobi_smooth3: fp32 or bf16 values");
    GB_REQUIRE(nrow > 0 && offsets && columns && values && r && z && dinv_blocks && z_out && z_out != z,
               "block_jacobi_smooth3: bad arguments");
    if (val_dtype == GB_F32)
        return launch_block_smooth3<float>(nrow, nnz, ncap, offsets, columns, (const float*)values, r, z, dinv_blocks,
                                           omega, z_out, status, val_dtype, stream);
    return launch_block_smooth3<__nv_bfloat16>(nrow, nnz, ncap, offsets, columns, (const __nv_bfloat16*)values, r, z,
                                               dinv_blocks, omega, z_out, status, val_dtype, stream);
}

GB_API int gb_bsr_jacobi_smooth(int bdim, int nrow, int64_t nnz, int64_t ncap, const int* offsets, const int* columns,
                                const void* values, int val_dtype, const float* r, const float* z, const float* dinv,
                                float omega, float* z_out, int* status, cudaStream_t stream)
{
    GB_REQUIRE(bdim == 1 || bdim == 3, "jacobi_smooth: block dim must be 1 or 3");
    GB_REQUIRE(val_dtype == GB_F32 || val_dtype == GB_BF16, "jacobi_smooth: fp32 or bf16 values");
    GB_REQUIRE(nrow > 0 && offsets && columns && values && r && z && dinv && z_out && z_out != z,
               "jacobi_smooth: bad arguments");
    if (val_dtype == GB_F32)
        return bdim == 1 ? launch_smooth<1, float>(nrow, nnz, ncap, offsets, columns, (const float*)values, r, z, dinv,
                                                   omega, z_out, status, val_dtype, stream)
                         : launch_smooth<3, float>(nrow, nnz, ncap, offsets, columns, (const float*)values, r, z, dinv,
                                                   omega, z_out, status, val_dtype, stream);
    return bdim == 1 ? launch_smooth<1, __nv_bfloat16>(nrow, nnz, ncap, offsets, columns, (const __nv_bfloat16*)values,
                                                       r, z, dinv, omega, z_out, status, val_dtype, stream)
                     : launch_smooth<3, __nv_bfloat16>(nrow, nnz, ncap, offsets, columns, (const __nv_bfloat16*)values,
                                                       r, z, dinv, omega, z_out, status, val_dtype, stream);
}

// Reports the tile shape the heuristic picks (for the autotuner and the roofline accounting).
GB_API int gb_bsr_mv_default_shape(int block_rows, int block_cols, int val_dtype, int nrow, int64_t nnz,
                                   int* rows_per_cta, int* lanes_per_row, int* cap_blocks)
{
    SpmvShape sh = default_shape(block_rows, block_cols, val_dtype, nrow, nnz, nnz, true);
    sh.rows = std::max(4, (sh.rows + 3) & ~3);
    *rows_per_cta = sh.rows;
    *lanes_per_row = sh.G;
    *cap_blocks = sh.cap;
    return GB_OK;
}
