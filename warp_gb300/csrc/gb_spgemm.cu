// gb_spgemm.cu -- BSR x BSR products (bsr_mm) expressed through the triplet assembly.
//
// Replaces the bsr_mm pipeline of warp/_src/sparse.py:4200-4624 (kernels :3620-3917: count ->
// scan -> list coefficients -> _bsr_set_from_triplets_native -> compute values).  Every product
// term x[r,k] * y[k,c] becomes a triplet (r, c) whose payload is the pair of factor blocks; the
// radix-sort assembly (gb_triplets.cu) yields the product topology and, per output block, the
// run of terms in a stable order, which k_spgemm_values sums (plus beta * z for the existing
// blocks of z, also entered as triplets).
#include "gb_common.cuh"

namespace gb {

// count[i] = number of blocks in row columns[i] of y, for every block i of x (0 past x's nnz)
__global__ void k_spgemm_count(int x_nrow, const int* __restrict__ x_offsets, const int* __restrict__ x_columns,
                               const int* __restrict__ y_offsets, int x_nnz_cap, int* __restrict__ count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= x_nnz_cap) return;
    const int nnz = x_offsets[x_nrow];
    if (i >= nnz) {
        count[i] = 0;
        return;
    }
    const int k = x_columns[i];
    count[i] = y_offsets[k + 1] - y_offsets[k];
}

// row of block i by binary search in offsets (offsets non-decreasing)
__device__ __forceinline__ int block_row(const int* offsets, int nrow, int i)
{
    int lo = 0, hi = nrow - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// emit triplets: for block i = (r, k) of x and each block j of y row k: (r, col_j) with payload
// (i, j).  start = exclusive scan of count.  z's blocks follow at [z_base, z_base + z_nnz) with
// payload (-1, zb).
__global__ void k_spgemm_emit(int x_nrow, const int* __restrict__ x_offsets, const int* __restrict__ x_columns,
                              const int* __restrict__ y_offsets, const int* __restrict__ y_columns, int x_nnz_cap,
                              const int* __restrict__ start, int* __restrict__ rows, int* __restrict__ cols,
                              int2* __restrict__ pairs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= x_nnz_cap) return;
    if (i >= x_offsets[x_nrow]) return;
    const int r = block_row(x_offsets, x_nrow, i);
    const int k = x_columns[i];
    int o = start[i];
    for (int j = y_offsets[k]; j < y_offsets[k + 1]; ++j, ++o) {
        rows[o] = r;
        cols[o] = y_columns[j];
        pairs[o] = make_int2(i, j);
    }
}

__global__ void k_spgemm_emit_z(int z_nrow, const int* __restrict__ z_offsets, const int* __restrict__ z_columns,
                                int z_nnz_cap, int base, int* __restrict__ rows, int* __restrict__ cols,
                                int2* __restrict__ pairs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= z_nnz_cap) return;
    const int o = base + i;
    if (i >= z_offsets[z_nrow]) {
        rows[o] = -1;  // pruned by the assembly
        cols[o] = -1;
        pairs[o] = make_int2(-1, -1);
        return;
    }
    rows[o] = block_row(z_offsets, z_nrow, i);
    cols[o] = z_columns[i];
    pairs[o] = make_int2(-1, i);
}

// value of output block b, scalar (p, q): sum over its run of alpha * (X[i] Y[j])_(p,q) or
// beta * Z[zb]_(p,q), in run order.  X blocks br x bk, Y bk x bc, Z br x bc, fp32 or fp64.
template <typename T>
__global__ void k_spgemm_values(int nrow, const int* __restrict__ out_offsets, const int* __restrict__ run_ends,
                                const int* __restrict__ run_ids, const int2* __restrict__ pairs, int br, int bk,
                                int bc, const T* __restrict__ X, const T* __restrict__ Y, const T* __restrict__ Z,
                                T alpha, T beta, T* __restrict__ out)
{
    const int64_t nnzb = out_offsets[nrow];
    const int bs = br * bc;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnzb * bs;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = t / bs;
        const int s = (int)(t - b * bs);
        const int p = s / bc, q = s - (s / bc) * bc;
        const int beg = b == 0 ? 0 : run_ends[b - 1];
        const int end = run_ends[b];
        T acc = T(0);
        for (int k = beg; k < end; ++k) {
            const int2 pr = pairs[run_ids[k]];
            if (pr.x < 0) {
                acc += beta * Z[(size_t)pr.y * bs + s];
            } else {
                T d = T(0);
                for (int m = 0; m < bk; ++m)
                    d += X[((size_t)pr.x * br + p) * bk + m] * Y[((size_t)pr.y * bk + m) * bc + q];
                acc += alpha * d;
            }
        }
        out[t] = acc;
    }
}

}  // namespace gb

using namespace gb;

GB_API int gb_spgemm_count(int x_nrow, const int* x_offsets, const int* x_columns, const int* y_offsets, int x_nnz_cap,
                           int* count, cudaStream_t stream)
{
    if (x_nnz_cap <= 0) return GB_OK;
    k_spgemm_count<<<ceil_div(x_nnz_cap, 256), 256, 0, stream>>>(x_nrow, x_offsets, x_columns, y_offsets, x_nnz_cap,
                                                                 count);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_spgemm_emit(int x_nrow, const int* x_offsets, const int* x_columns, const int* y_offsets,
                          const int* y_columns, int x_nnz_cap, const int* start, int z_nrow, const int* z_offsets,
                          const int* z_columns, int z_nnz_cap, int z_base, int* rows, int* cols, void* pairs,
                          cudaStream_t stream)
{
    if (x_nnz_cap > 0)
        k_spgemm_emit<<<ceil_div(x_nnz_cap, 256), 256, 0, stream>>>(x_nrow, x_offsets, x_columns, y_offsets,
                                                                     y_columns, x_nnz_cap, start, rows, cols,
                                                                     (int2*)pairs);
    if (z_offsets && z_nnz_cap > 0)
        k_spgemm_emit_z<<<ceil_div(z_nnz_cap, 256), 256, 0, stream>>>(z_nrow, z_offsets, z_columns, z_nnz_cap, z_base,
                                                                       rows, cols, (int2*)pairs);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_spgemm_values(int dtype, int nrow, const int* out_offsets, const int* run_ends, const int* run_ids,
                            const void* pairs, int br, int bk, int bc, const void* X, const void* Y, const void* Z,
                            double alpha, double beta, void* out, int nnz_upper, cudaStream_t stream)
{
    if (nnz_upper <= 0) return GB_OK;
    const int grid = (int)std::min<int64_t>(ceil_div<int64_t>((int64_t)nnz_upper * br * bc, 256), kSmCount * 32);
    if (dtype == GB_F32)
        k_spgemm_values<float><<<grid, 256, 0, stream>>>(nrow, out_offsets, run_ends, run_ids, (const int2*)pairs, br,
                                                         bk, bc, (const float*)X, (const float*)Y, (const float*)Z,
                                                         (float)alpha, (float)beta, (float*)out);
    else if (dtype == GB_F64)
        k_spgemm_values<double><<<grid, 256, 0, stream>>>(nrow, out_offsets, run_ends, run_ids, (const int2*)pairs,
                                                          br, bk, bc, (const double*)X, (const double*)Y,
                                                          (const double*)Z, alpha, beta, (double*)out);
    else {
        gb::set_error("spgemm_values: unsupported dtype");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
