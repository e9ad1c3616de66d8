// gb_spmv.cuh -- the BSR row-tile SpMV core shared by bsr_mv and the fused Krylov kernels.
//
// One CTA owns `rows` consecutive block rows.  Their column indices and block values form one
// contiguous range [offsets[r0], offsets[r0+rows]); it is copied global -> shared with two
// cp.async.bulk (TMA) transfers completing on one mbarrier (start rounded down to 8 blocks so
// both copies are 16-byte aligned; the < 8-block tail past the last aligned block is loaded with
// plain loads).  Lane groups of G lanes then walk their rows out of shared memory, gather x
// through the read-only path (x of every config fits the 129 MB L2) and reduce with shuffles.
// A tile whose range does not fit the shared buffer is computed straight from global memory.
#pragma once
#include "gb_bulk.cuh"
#include "gb_common.cuh"

namespace gb {

constexpr int SPMV_THREADS = 256;
constexpr int SPMV_ALIGN = 8;  // blocks; 8 int32 columns = 32 B, 8 blocks of values = multiple of 16 B

struct SpmvShape {
    int rows;   // block rows per CTA
    int G;      // lanes per block row (power of two, 1..32)
    int cap;    // staged blocks per CTA (0 disables staging)
    int64_t ncap;  // number of valid entries in the columns/values arrays
};

template <int BR, int BC, typename VT>
__host__ __device__ inline size_t spmv_smem_bytes(int rows, int cap)
{
    size_t b = 16;                                   // mbarrier + pad
    b += (size_t)(2 * rows + 1) * sizeof(int);       // s_off[rows+1], s_end[rows]
    b = (b + 15) & ~(size_t)15;
    b += (size_t)cap * sizeof(int);                  // staged columns
    b = (b + 15) & ~(size_t)15;
    b += (size_t)cap * BR * BC * sizeof(VT);         // staged values
    return b;
}

template <typename AT, typename XT> __device__ __forceinline__ AT ldx(const XT* p) { return (AT)__ldg(p); }

template <typename AT, typename VT> __device__ __forceinline__ AT cvt(VT v);
template <> __device__ __forceinline__ float cvt<float, float>(float v) { return v; }
template <> __device__ __forceinline__ float cvt<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ double cvt<double, float>(float v) { return (double)v; }
template <> __device__ __forceinline__ double cvt<double, double>(double v) { return v; }
template <> __device__ __forceinline__ double cvt<double, __nv_bfloat16>(__nv_bfloat16 v)
{
    return (double)__bfloat162float(v);
}

// Runtime-G group reduction (all 32 lanes participate).
template <typename T> __device__ __forceinline__ T group_reduce(T v, int G)
{
    for (int o = G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Computes acc[BR] = sum_blocks A[row] x for every block row of this CTA's tile and calls
// epi(row, acc, lane_in_group) with the group-reduced sums (all lanes of the group hold them).
// Returns false (status updated) if the staging wait timed out; the tile is then skipped.
template <int BR, int BC, typename VT, typename XT, typename AT, typename Epi>
__device__ __forceinline__ bool spmv_tile(int nrow, const SpmvShape sh, const int* __restrict__ offsets,
                                          const int* __restrict__ row_counts, const int* __restrict__ columns,
                                          const VT* __restrict__ values, const XT* __restrict__ x,
                                          unsigned char* smem, int* status, Epi& epi)
{
    constexpr int BB = BR * BC;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    int* s_off = reinterpret_cast<int*>(smem + 16);
    int* s_end = s_off + sh.rows + 1;
    size_t o = 16 + (size_t)(2 * sh.rows + 1) * sizeof(int);
    o = (o + 15) & ~(size_t)15;
    int* s_cols = reinterpret_cast<int*>(smem + o);
    o += (size_t)sh.cap * sizeof(int);
    o = (o + 15) & ~(size_t)15;
    VT* s_vals = reinterpret_cast<VT*>(smem + o);

    const int r0 = blockIdx.x * sh.rows;
    const int nr = min(sh.rows, nrow - r0);
    for (int k = threadIdx.x; k <= nr; k += blockDim.x) {
        const int r = r0 + k;
        s_off[k] = offsets[r];
        if (k < nr) s_end[k] = row_counts ? offsets[r] + row_counts[r] : offsets[r + 1];
    }
    __syncthreads();
    const int b0 = s_off[0];
    const int b1 = s_off[nr];
    const int a0 = b0 & ~(SPMV_ALIGN - 1);
    const bool staged = (sh.cap > 0) && (b1 - a0 <= sh.cap);
    if (staged) {
        int a1 = min((b1 + SPMV_ALIGN - 1) & ~(SPMV_ALIGN - 1), (int)(sh.ncap & ~(int64_t)(SPMV_ALIGN - 1)));
        a1 = max(a1, a0);
        const uint32_t nb = (uint32_t)(a1 - a0);
        if (threadIdx.x == 0) {
            mbar_init(bar, 1);
            fence_mbar_init();
            mbar_arrive_expect_tx(bar, nb * (uint32_t)(sizeof(int) + BB * sizeof(VT)));
            if (nb > 0) {
                bulk_g2s(s_cols, columns + a0, nb * (uint32_t)sizeof(int), bar);
                bulk_g2s(s_vals, values + (size_t)a0 * BB, nb * (uint32_t)(BB * sizeof(VT)), bar);
            }
        }
        // ragged tail (< 8 blocks) past the last aligned block of the arrays
        for (int b = max(a1, a0) + (int)threadIdx.x; b < b1; b += blockDim.x) {
            s_cols[b - a0] = columns[b];
#pragma unroll
            for (int q = 0; q < BB; ++q) s_vals[(size_t)(b - a0) * BB + q] = values[(size_t)b * BB + q];
        }
        __syncthreads();
        if (!mbar_wait_bounded(bar, 0)) {
            if (threadIdx.x == 0 && status) atomicOr(status, GB_DEV_WAIT_TIMEOUT);
            mbar_wait_bounded(bar, 0);  // drain (bounded) before the CTA exits
            return false;
        }
    }

    const int G = sh.G;
    const int lane_g = threadIdx.x & (G - 1);
    const int ngroups = blockDim.x / G;
    const int* cbase = staged ? s_cols - a0 : columns;
    const VT* vbase = staged ? s_vals - (size_t)a0 * BB : values;
    for (int k = threadIdx.x / G; k < nr; k += ngroups) {
        const int beg = s_off[k], end = s_end[k];
        AT acc[BR];
#pragma unroll
        for (int i = 0; i < BR; ++i) acc[i] = AT(0);
        for (int b = beg + lane_g; b < end; b += G) {
            const int c = cbase[b];
            const VT* v = vbase + (size_t)b * BB;
            AT xv[BC];
#pragma unroll
            for (int j = 0; j < BC; ++j) xv[j] = ldx<AT>(x + (size_t)c * BC + j);
#pragma unroll
            for (int i = 0; i < BR; ++i) {
#pragma unroll
                for (int j = 0; j < BC; ++j) acc[i] += cvt<AT>(v[i * BC + j]) * xv[j];
            }
        }
#pragma unroll
        for (int i = 0; i < BR; ++i) acc[i] = group_reduce(acc[i], G);
        epi(r0 + k, acc, lane_g);
    }
    return true;
}

// Default tile shape for a matrix (defined in gb_spmv.cu).
SpmvShape default_shape(int br, int bc, int val_dtype, int nrow, int64_t nnzb, int64_t ncap, bool aligned);

// Select acc[i] for a runtime i without dynamic register indexing.
template <int BR, typename AT> __device__ __forceinline__ AT pick(const AT (&acc)[BR], int i)
{
    AT v = acc[0];
#pragma unroll
    for (int q = 1; q < BR; ++q)
        if (i == q) v = acc[q];
    return v;
}

}  // namespace gb
