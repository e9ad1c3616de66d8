// gb_misc.cu -- small kernels around the solve path: BSR diagonal extraction and the Jacobi
// inverse diagonal, diagonal / dense operator products, deterministic multi-column dot products
// and axpby for the generic (non-BSR) LinearOperator path.
//
// Replaces: bsr_get_diag (warp/_src/sparse.py:2871-2887), _extract_inverse_diagonal_* and
// _inverse_diag_coefficient (warp/_src/optim/linear.py:2290-2329), _diag_mv_kernel (:2271-2287),
// _dense_mv_kernel (:2250-2268), TiledDot.compute (:506-568) and array_axpy.
#include "gb_common.cuh"

namespace gb {

template <typename T>
__global__ void k_bsr_get_diag(int nrow, int br, int bc, const int* __restrict__ offsets,
                               const int* __restrict__ row_counts, const int* __restrict__ columns,
                               const T* __restrict__ values, T* __restrict__ out)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    const int bs = br * bc;
    int beg = offsets[row];
    const int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
    // columns are sorted within a row: binary search for the diagonal block
    int lo = beg, hi = end - 1, found = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = columns[mid];
        if (c == row) {
            found = mid;
            break;
        }
        if (c < row) lo = mid + 1; else hi = mid - 1;
    }
    for (int q = 0; q < bs; ++q) out[(size_t)row * bs + q] = (found >= 0) ? values[(size_t)found * bs + q] : T(0);
}

// inverse of the diagonal entries of the diagonal blocks: 1/d, 1/|d| (use_abs) or 1 when d == 0.
template <typename T>
__global__ void k_bsr_inverse_diag(int nrow, int bdim, const int* __restrict__ offsets,
                                   const int* __restrict__ row_counts, const int* __restrict__ columns,
                                   const T* __restrict__ values, int use_abs, T* __restrict__ inv)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    const int bs = bdim * bdim;
    const int beg = offsets[row];
    const int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
    int lo = beg, hi = end - 1, found = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = columns[mid];
        if (c == row) {
            found = mid;
            break;
        }
        if (c < row) lo = mid + 1; else hi = mid - 1;
    }
    for (int k = 0; k < bdim; ++k) {
        T d = (found >= 0) ? values[(size_t)found * bs + k * bdim + k] : T(0);
        if (use_abs) d = d < T(0) ? -d : d;
        inv[(size_t)row * bdim + k] = (d == T(0)) ? T(1) : T(1) / d;
    }
}

// Inverse of every 3x3 diagonal block (the block-Jacobi smoother of vec3 multigrid levels), computed
// in double by the adjugate; a missing or singular block gives the identity.  inv: 9 floats per block
// row, row-major.
__global__ void k_bsr_block_inverse_diag3(int nrow, const int* __restrict__ offsets, const int* __restrict__ row_counts,
                                          const int* __restrict__ columns, const float* __restrict__ values,
                                          float* __restrict__ inv)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    const int beg = offsets[row];
    const int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
    int lo = beg, hi = end - 1, found = -1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = columns[mid];
        if (c == row) {
            found = mid;
            break;
        }
        if (c < row) lo = mid + 1; else hi = mid - 1;
    }
    double m[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (found >= 0)
        for (int k = 0; k < 9; ++k) m[k] = (double)values[(size_t)found * 9 + k];
    const double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    float* o = inv + (size_t)row * 9;
    if (!(det != 0.0) || !isfinite(det)) {
        for (int k = 0; k < 9; ++k) o[k] = (k % 4 == 0) ? 1.f : 0.f;
        return;
    }
    const double id = 1.0 / det;
    o[0] = (float)(c00 * id);
    o[1] = (float)((m[2] * m[7] - m[1] * m[8]) * id);
    o[2] = (float)((m[1] * m[5] - m[2] * m[4]) * id);
    o[3] = (float)(c01 * id);
    o[4] = (float)((m[0] * m[8] - m[2] * m[6]) * id);
    o[5] = (float)((m[2] * m[3] - m[0] * m[5]) * id);
    o[6] = (float)(c02 * id);
    o[7] = (float)((m[1] * m[6] - m[0] * m[7]) * id);
    o[8] = (float)((m[0] * m[4] - m[1] * m[3]) * id);
}

template <typename T>
__global__ void k_diag_mv(int64_t n, const T* __restrict__ A, const T* __restrict__ x, const T* y, T* z, T alpha,
                          T beta)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T s = T(0);
        if (alpha != T(0)) s += alpha * (A[i] * x[i]);
        if (beta != T(0)) s += beta * y[i];
        z[i] = s;
    }
}

// z = alpha A x + beta y for a dense row-major m x n matrix; one warp per row.
template <typename T>
__global__ void k_dense_mv(int m, int n, const T* __restrict__ A, const T* __restrict__ x, const T* y, T* z, T alpha,
                           T beta)
{
    pdl_enter();
    const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (row >= m) return;
    T s = T(0);
    if (alpha != T(0))
        for (int c = lane; c < n; c += 32) s += A[(size_t)row * n + c] * x[c];
    s = warp_sum(s);
    if (lane == 0) {
        T v = alpha * s;
        if (beta != T(0)) v += beta * y[row];
        z[row] = v;
    }
}

// The same product for long rows (the multigrid's coarsest inverse, a few thousand columns): one CTA of
// DMV_THREADS per row, so that thousands of rows keep enough loads in flight to stream the matrix;
// per-thread partials in order, then a fixed-order reduction (deterministic).
constexpr int DMV_THREADS = 128;
template <typename T>
__global__ void __launch_bounds__(DMV_THREADS) k_dense_mv_rows(int n, const T* __restrict__ A, const T* __restrict__ x,
                                                              const T* y, T* z, T alpha, T beta)
{
    pdl_enter();
    __shared__ T s_part[DMV_THREADS / 32];
    const int row = blockIdx.x;
    const T* __restrict__ a = A + (size_t)row * n;
    T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
    int c = threadIdx.x;
    if (alpha != T(0)) {
        for (; c + 3 * DMV_THREADS < n; c += 4 * DMV_THREADS) {
            s0 += a[c] * x[c];
            s1 += a[c + DMV_THREADS] * x[c + DMV_THREADS];
            s2 += a[c + 2 * DMV_THREADS] * x[c + 2 * DMV_THREADS];
            s3 += a[c + 3 * DMV_THREADS] * x[c + 3 * DMV_THREADS];
        }
        for (; c < n; c += DMV_THREADS) s0 += a[c] * x[c];
    }
    T s = warp_sum((s0 + s1) + (s2 + s3));
    if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        T t = s_part[0];
#pragma unroll
        for (int w = 1; w < DMV_THREADS / 32; ++w) t += s_part[w];
        T v = alpha * t;
        if (beta != T(0)) v += beta * y[row];
        z[row] = v;
    }
}

// Multi-column dot products out[k] = sum_i x_k[i] y_k[i] (k < ncols <= 4), accumulated in fp64,
// single-pass deterministic grid reduction.
struct DotPtrs {
    const void* x[4];
    const void* y[4];
};

template <typename T>
__global__ void k_dots(int64_t n, int ncols, DotPtrs P, double* partials, unsigned int* counter, double* out)
{
    __shared__ double s_red[32 * 4];
    T acc[4] = {T(0), T(0), T(0), T(0)};  // per-thread partials in T, fp64 across warps
    for (int k = 0; k < ncols; ++k) {
        const T* x = static_cast<const T*>(P.x[k]);
        const T* y = static_cast<const T*>(P.y[k]);
        T a = T(0);
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            a += x[i] * y[i];
        acc[k] = a;
    }
    grid_reduce<4>(acc, partials, counter, s_red, [&](const double (&t)[4]) {
        for (int k = 0; k < ncols; ++k) out[k] = t[k];
    });
}

template <typename T>
__global__ void k_axpby(int64_t n, T alpha, const T* __restrict__ x, T beta, const T* y, T* out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T v = alpha * x[i];
        if (beta != T(0)) v += beta * y[i];
        out[i] = v;
    }
}

static int vgrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 8)); }

}  // namespace gb

using namespace gb;

GB_API int gb_bsr_get_diag(int dtype, int br, int bc, int nrow, const int* offsets, const int* row_counts,
                           const int* columns, const void* values, void* out, cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0 && br >= 1 && bc >= 1, "bsr_get_diag: bad shape");
    if (nrow == 0) return GB_OK;
    const int grid = ceil_div(nrow, 128);
    if (dtype == GB_F32)
        k_bsr_get_diag<float><<<grid, 128, 0, stream>>>(nrow, br, bc, offsets, row_counts, columns,
                                                        (const float*)values, (float*)out);
    else if (dtype == GB_F64)
        k_bsr_get_diag<double><<<grid, 128, 0, stream>>>(nrow, br, bc, offsets, row_counts, columns,
                                                         (const double*)values, (double*)out);
    else {
        gb::set_error("bsr_get_diag: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_bsr_inverse_diagonal(int dtype, int bdim, int nrow, const int* offsets, const int* row_counts,
                                   const int* columns, const void* values, int use_abs, void* inv, cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0 && bdim >= 1, "bsr_inverse_diagonal: bad shape");
    if (nrow == 0) return GB_OK;
    const int grid = ceil_div(nrow, 128);
    if (dtype == GB_F32)
        k_bsr_inverse_diag<float><<<grid, 128, 0, stream>>>(nrow, bdim, offsets, row_counts, columns,
                                                            (const float*)values, use_abs, (float*)inv);
    else if (dtype == GB_F64)
        k_bsr_inverse_diag<double><<<grid, 128, 0, stream>>>(nrow, bdim, offsets, row_counts, columns,
                                                             (const double*)values, use_abs, (double*)inv);
    else {
        gb::set_error("bsr_inverse_diagonal: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_diag_mv(int dtype, int64_t n, const void* A, const void* x, const void* y, void* z, double alpha,
                      double beta, cudaStream_t stream)
{
    if (n <= 0) return GB_OK;
    if (dtype == GB_F32)
        k_diag_mv<float><<<vgrid(n), 256, 0, stream>>>(n, (const float*)A, (const float*)x, (const float*)y,
                                                       (float*)z, (float)alpha, (float)beta);
    else if (dtype == GB_F64)
        k_diag_mv<double><<<vgrid(n), 256, 0, stream>>>(n, (const double*)A, (const double*)x, (const double*)y,
                                                        (double*)z, alpha, beta);
    else {
        gb::set_error("diag_mv: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_bsr_block_inverse_diagonal3(int nrow, const int* offsets, const int* row_counts, const int* columns,
                                          const float* values, float* inv, cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0, "bsr_block_inverse_diagonal3: bad shape");
    if (nrow == 0) return GB_OK;
    GB_REQUIRE(offsets && columns && values && inv, "bsr_block_inverse_diagonal3: missing argument");
    k_bsr_block_inverse_diag3<<<ceil_div(nrow, 128), 128, 0, stream>>>(nrow, offsets, row_counts, columns, values, inv);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_dense_mv(int dtype, int m, int n, const void* A, const void* x, const void* y, void* z, double alpha,
                       double beta, cudaStream_t stream)
{
    if (m <= 0) return GB_OK;
    if (n >= 4 * DMV_THREADS) {  // long rows: one CTA per row
        if (dtype == GB_F32)
            GB_CHECK_CUDA(launch_pdl(k_dense_mv_rows<float>, m, DMV_THREADS, 0, stream, n, (const float*)A,
                                     (const float*)x, (const float*)y, (float*)z, (float)alpha, (float)beta));
        else if (dtype == GB_F64)
            GB_CHECK_CUDA(launch_pdl(k_dense_mv_rows<double>, m, DMV_THREADS, 0, stream, n, (const double*)A,
                                     (const double*)x, (const double*)y, (double*)z, alpha, beta));
        else {
            gb::set_error("dense_mv: unsupported dtype");
            return GB_ERR_UNSUPPORTED;
        }
        GB_CHECK_CUDA(cudaGetLastError());
        return GB_OK;
    }
    const int grid = ceil_div(m, 8);
    if (dtype == GB_F32)
        GB_CHECK_CUDA(launch_pdl(k_dense_mv<float>, grid, 256, 0, stream, m, n, (const float*)A, (const float*)x,
                                 (const float*)y, (float*)z, (float)alpha, (float)beta));
    else if (dtype == GB_F64)
        GB_CHECK_CUDA(launch_pdl(k_dense_mv<double>, grid, 256, 0, stream, m, n, (const double*)A, (const double*)x,
                                 (const double*)y, (double*)z, alpha, beta));
    else {
        gb::set_error("dense_mv: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API size_t gb_dots_workspace_bytes(void) { return 256 + sizeof(double) * 4 * (size_t)(kSmCount * 2); }

// out[k] = x_k . y_k for k < ncols (<= 4), fp64 accumulation, deterministic.  xs/ys are host
// arrays of device pointers (passed by value to the kernel, so the call is capturable).  The
// workspace's first bytes hold the arrival counter (zero before first use; the kernel leaves it 0).
GB_API int gb_dots(int dtype, int64_t n, int ncols, const void* const* xs, const void* const* ys, double* out,
                   void* workspace, cudaStream_t stream)
{
    GB_REQUIRE(ncols >= 1 && ncols <= 4, "dots: 1 to 4 columns");
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    unsigned int* counter = reinterpret_cast<unsigned int*>(ws);
    double* partials = reinterpret_cast<double*>(ws + 256);
    DotPtrs P = {};
    for (int k = 0; k < ncols; ++k) {
        P.x[k] = xs[k];
        P.y[k] = ys[k];
    }
    const int grid = kSmCount * 2;
    if (dtype == GB_F32)
        k_dots<float><<<grid, 256, 0, stream>>>(n, ncols, P, partials, counter, out);
    else if (dtype == GB_F64)
        k_dots<double><<<grid, 256, 0, stream>>>(n, ncols, P, partials, counter, out);
    else {
        gb::set_error("dots: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_axpby(int dtype, int64_t n, double alpha, const void* x, double beta, const void* y, void* out,
                    cudaStream_t stream)
{
    if (n <= 0) return GB_OK;
    if (dtype == GB_F32)
        k_axpby<float><<<vgrid(n), 256, 0, stream>>>(n, (float)alpha, (const float*)x, (float)beta, (const float*)y,
                                                     (float*)out);
    else if (dtype == GB_F64)
        k_axpby<double><<<vgrid(n), 256, 0, stream>>>(n, alpha, (const double*)x, beta, (const double*)y,
                                                      (double*)out);
    else {
        gb::set_error("axpby: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// ---- multi-column dot / axpy (Gram-Schmidt steps of GMRES) -------------------------------------
namespace gb {
constexpr int MD_PARTS = 152;

template <typename T>
__global__ void k_multi_dot_part(int64_t n, const T* __restrict__ V, int64_t ldv, const T* __restrict__ w,
                                 double* __restrict__ partials)
{
    __shared__ double scratch[32];
    const int c = blockIdx.y;
    const T* v = V + (int64_t)c * ldv;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * chunk, i1 = min(n, i0 + chunk);
    double s = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) s += (double)v[i] * (double)w[i];
    double in[1] = {s}, out[1];
    block_sum<1, double>(in, scratch, out);
    if (threadIdx.x == 0) partials[(int64_t)c * gridDim.x + blockIdx.x] = out[0];
}

__global__ void k_multi_dot_finish(int parts, const double* __restrict__ partials, double* __restrict__ out)
{
    const int c = blockIdx.x;
    double s = 0.0;
    for (int p = threadIdx.x; p < parts; p += 32) s += partials[(int64_t)c * parts + p];
    s = warp_sum(s);
    if (threadIdx.x == 0) out[c] = s;
}

// w = beta * w + alpha * sum_c coef[c] * V[c]
template <typename T>
__global__ void k_multi_axpy(int64_t n, int ncols, const T* __restrict__ V, int64_t ldv, const double* __restrict__ coef,
                             double alpha, double beta, T* __restrict__ w)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < ncols; ++c) s += coef[c] * (double)V[(int64_t)c * ldv + i];
        w[i] = (T)(beta * (double)w[i] + alpha * s);
    }
}
}  // namespace gb

GB_API size_t gb_multi_dot_workspace_bytes(int ncols) { return sizeof(double) * (size_t)std::max(ncols, 1) * gb::MD_PARTS; }

// out[c] = V[c] . w for c < ncols (rows of V are ldv apart), fp64 accumulation, deterministic.
GB_API int gb_multi_dot(int dtype, int64_t n, int ncols, const void* V, int64_t ldv, const void* w, double* out,
                        void* workspace, size_t workspace_bytes, cudaStream_t stream)
{
    GB_REQUIRE(ncols >= 1 && ncols <= 65535 && n >= 0, "multi_dot: bad sizes");
    GB_REQUIRE(workspace_bytes >= gb_multi_dot_workspace_bytes(ncols), "multi_dot: workspace too small");
    double* partials = static_cast<double*>(workspace);
    dim3 grid(gb::MD_PARTS, ncols);
    if (dtype == GB_F32)
        gb::k_multi_dot_part<float><<<grid, 256, 0, stream>>>(n, (const float*)V, ldv, (const float*)w, partials);
    else if (dtype == GB_F64)
        gb::k_multi_dot_part<double><<<grid, 256, 0, stream>>>(n, (const double*)V, ldv, (const double*)w, partials);
    else {
        gb::set_error("multi_dot: dtype must be f32 or f64");
        return GB_ERR_UNSUPPORTED;
    }
    gb::k_multi_dot_finish<<<ncols, 32, 0, stream>>>(gb::MD_PARTS, partials, out);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// w = beta * w + alpha * sum_c coef[c] * V[c]  (coef: device doubles)
GB_API int gb_multi_axpy(int dtype, int64_t n, int ncols, const void* V, int64_t ldv, const double* coef, double alpha,
                         double beta, void* w, cudaStream_t stream)
{
    GB_REQUIRE(ncols >= 0 && n >= 0, "multi_axpy: bad sizes");
    if (n == 0) return GB_OK;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 8));
    if (dtype == GB_F32)
        gb::k_multi_axpy<float><<<grid, 256, 0, stream>>>(n, ncols, (const float*)V, ldv, coef, alpha, beta, (float*)w);
    else if (dtype == GB_F64)
        gb::k_multi_axpy<double><<<grid, 256, 0, stream>>>(n, ncols, (const double*)V, ldv, coef, alpha, beta,
                                                           (double*)w);
    else {
        gb::set_error("multi_axpy: dtype must be f32 or f64");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
