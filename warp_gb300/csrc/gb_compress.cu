// gb_compress.cu -- row-local BSR compression: the "row_compress" construction of fem.integrate.
//
// Reference: bsr_compress (warp/_src/sparse.py:1571-1640) with inplace=True ->
// wp_bsr_compress_inplace_device (warp/native/sparse.cu:1494-1656) -> bsr_compress_inplace_row
// (warp/native/sparse_util.h:82-139): inside each active row range [offsets[r], offsets[r] +
// row_counts[r]) blocks whose scalars are all zero (under the zero mask) are dropped when pruning,
// the remaining blocks are stably sorted by column, and runs of equal columns are summed in their
// original order; row_counts become the coalesced counts.  fem.integrate(bsr_options={"construction":
// "row_compress"}) (warp/_src/fem/integrate.py:1650-1730, :1850) assembles candidate blocks row by
// row (test node, element, trial node) straight into that padded layout, so no global sort is needed.
//
// Here: one warp per row.  Candidates (<= 128 per row; longer rows take the reference's serial
// insertion sort) are keyed (column, slot) -- unique keys, so ranking them is a stable sort -- and
// ranked in shared memory; each run head sums its run in slot order (the order the triplet path
// accumulates in, so values are bit-identical to bsr_set_from_triplets on the same candidates), and
// the row is rewritten in place after every read of it has finished.  A compaction pass (scan of the
// counts + one warp per row gather) produces the compact CSR.
#include "gb_common.cuh"
#include "gb_scan.cuh"

namespace gb {

constexpr int CMP_WARPS = 8;
constexpr int CMP_CAP = 128;  // candidates per row handled by the warp path

// offsets of the padded layout from row indices sorted in non-decreasing order (empty rows allowed)
__global__ void k_rows_to_offsets(int64_t T, const int* __restrict__ rows, int nrow, int* __restrict__ offsets,
                                  int* __restrict__ status)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = rows[t];
        const int prev = t > 0 ? rows[t - 1] : -1;
        if (r < 0 || r >= nrow || r < prev) {
            atomicOr(status, GB_DEV_BREAKDOWN);
            continue;
        }
        for (int rr = prev + 1; rr <= r; ++rr) offsets[rr] = (int)t;
        if (t == T - 1)
            for (int rr = r + 1; rr <= nrow; ++rr) offsets[rr] = (int)T;
    }
}

template <typename T>
__device__ __forceinline__ bool block_is_zero(const T* v, int64_t blk, int bb, uint64_t mask)
{
    for (int c = 0; c < bb; ++c) {
        uint64_t bits;
        if constexpr (sizeof(T) == 4) bits = __float_as_uint((float)v[blk * bb + c]);
        else bits = (uint64_t)__double_as_longlong((double)v[blk * bb + c]);
        if (bits & mask) return false;
    }
    return true;
}

// the reference's serial row routine (insertion sort, then coalesce), for rows longer than CMP_CAP
template <typename T, int BB>
__device__ void compress_row_serial(int beg, int end, int* columns, T* values, bool prune, uint64_t mask, int& count)
{
    if (prune)
        for (int b = beg; b < end; ++b)
            if (columns[b] >= 0 && block_is_zero(values, b, BB, mask)) columns[b] = -1;
    for (int b = beg + 1; b < end; ++b) {
        int s = b;
        while (s > beg && columns[s] < columns[s - 1]) {
            const int c = columns[s];
            columns[s] = columns[s - 1];
            columns[s - 1] = c;
            for (int q = 0; q < BB; ++q) {
                const T tmp = values[(int64_t)s * BB + q];
                values[(int64_t)s * BB + q] = values[(int64_t)(s - 1) * BB + q];
                values[(int64_t)(s - 1) * BB + q] = tmp;
            }
            --s;
        }
    }
    int w = beg, r = beg;
    while (r < end) {
        const int c = columns[r];
        if (c < 0) {
            ++r;
            continue;
        }
        if (w != r) {
            columns[w] = c;
            for (int q = 0; q < BB; ++q) values[(int64_t)w * BB + q] = values[(int64_t)r * BB + q];
        }
        ++r;
        while (r < end && columns[r] == c) {
            for (int q = 0; q < BB; ++q) values[(int64_t)w * BB + q] += values[(int64_t)r * BB + q];
            ++r;
        }
        ++w;
    }
    count = w - beg;
}

template <typename T, int BB>
__global__ void __launch_bounds__(CMP_WARPS * 32)
    k_compress_rows(int nrow, const int* __restrict__ offsets, const int* __restrict__ row_counts, int* columns,
                    T* values, int prune, uint64_t mask, int* __restrict__ out_counts)
{
    __shared__ unsigned long long s_key[CMP_WARPS][CMP_CAP];
    __shared__ unsigned long long s_srt[CMP_WARPS][CMP_CAP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long* key = s_key[warp];
    unsigned long long* srt = s_srt[warp];
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int row = blockIdx.x * CMP_WARPS + warp; row < nrow; row += gridDim.x * CMP_WARPS) {
        const int beg = offsets[row];
        const int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
        const int cnt = end - beg;
        if (cnt > CMP_CAP) {
            if (lane == 0) {
                int c = 0;
                compress_row_serial<T, BB>(beg, end, columns, values, prune != 0, mask, c);
                out_counts[row] = c;
            }
            __syncwarp();
            continue;
        }
        // keys (column << 8 | slot): unique, so ranking them sorts stably; dropped candidates -> ~0
        int nv = 0;
        for (int s = lane; s < CMP_CAP; s += 32) {
            unsigned long long k = ~0ull;
            if (s < cnt) {
                const int c = columns[beg + s];
                if (c >= 0 && !(prune && block_is_zero(values, (int64_t)beg + s, BB, mask)))
                    k = ((unsigned long long)(unsigned)c << 8) | (unsigned)s;
            }
            key[s] = k;
            nv += (k != ~0ull);
        }
        const int nvalid = warp_sum(nv);
        __syncwarp();
        for (int s = lane; s < cnt; s += 32) {
            const unsigned long long k = key[s];
            if (k == ~0ull) continue;
            int rank = 0;
            for (int j = 0; j < cnt; ++j) rank += key[j] < k;
            srt[rank] = k;
        }
        __syncwarp();
        // run heads: sum the run in slot order (reads only)
        T acc[CMP_CAP / 32][BB];
        int hcol[CMP_CAP / 32], hrank[CMP_CAP / 32];
        bool head[CMP_CAP / 32];
        int base = 0;
#pragma unroll
        for (int j = 0; j < CMP_CAP / 32; ++j) {
            const int e = j * 32 + lane;
            bool h = false;
            int col = -1;
            if (e < nvalid) {
                col = (int)(srt[e] >> 8);
                h = (e == 0) || ((int)(srt[e - 1] >> 8) != col);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, h);
            head[j] = h;
            hcol[j] = col;
            hrank[j] = base + __popc(bal & lt_mask);
            base += __popc(bal);
            if (h) {
                const int64_t s0 = (int64_t)beg + (int)(srt[e] & 0xFF);
#pragma unroll
                for (int q = 0; q < BB; ++q) acc[j][q] = values[s0 * BB + q];
                for (int k = e + 1; k < nvalid && (int)(srt[k] >> 8) == col; ++k) {
                    const int64_t sk = (int64_t)beg + (int)(srt[k] & 0xFF);
#pragma unroll
                    for (int q = 0; q < BB; ++q) acc[j][q] += values[sk * BB + q];
                }
            }
        }
        __syncwarp();  // every read of this row is done: rewrite it in place
#pragma unroll
        for (int j = 0; j < CMP_CAP / 32; ++j)
            if (head[j]) {
                const int64_t d = (int64_t)beg + hrank[j];
                columns[d] = hcol[j];
#pragma unroll
                for (int q = 0; q < BB; ++q) values[d * BB + q] = acc[j][q];
            }
        if (lane == 0) out_counts[row] = base;
        __syncwarp();
    }
}

template <typename T, int BB>
__global__ void k_compact_rows(int nrow, const int* __restrict__ old_off, const int* __restrict__ counts,
                               const int* __restrict__ new_off, const int* __restrict__ cols_in,
                               const T* __restrict__ vals_in, int* __restrict__ cols_out, T* __restrict__ vals_out)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int row = warp; row < nrow; row += nw) {
        const int n = counts[row];
        const int64_t src = old_off[row], dst = new_off[row];
        for (int i = lane; i < n; i += 32) cols_out[dst + i] = cols_in[src + i];
        for (int i = lane; i < n * BB; i += 32) vals_out[dst * BB + i] = vals_in[src * BB + i];
    }
}

template <typename T>
static int launch_compress(int bb, int nrow, const int* offsets, const int* row_counts, int* columns, void* values,
                           int prune, uint64_t mask, int* out_counts, cudaStream_t stream)
{
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nrow, CMP_WARPS), kSmCount * 16));
    T* v = static_cast<T*>(values);
    switch (bb) {
    case 1: k_compress_rows<T, 1><<<grid, CMP_WARPS * 32, 0, stream>>>(nrow, offsets, row_counts, columns, v, prune, mask, out_counts); break;
    case 4: k_compress_rows<T, 4><<<grid, CMP_WARPS * 32, 0, stream>>>(nrow, offsets, row_counts, columns, v, prune, mask, out_counts); break;
    case 9: k_compress_rows<T, 9><<<grid, CMP_WARPS * 32, 0, stream>>>(nrow, offsets, row_counts, columns, v, prune, mask, out_counts); break;
    default: gb::set_error("bsr_compress: block size must be 1, 4 or 9 scalars"); return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

template <typename T>
static int launch_compact(int bb, int nrow, const int* old_off, const int* counts, const int* new_off,
                          const int* cols_in, const void* vals_in, int* cols_out, void* vals_out, cudaStream_t stream)
{
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nrow, 8), kSmCount * 16));
    const T* vi = static_cast<const T*>(vals_in);
    T* vo = static_cast<T*>(vals_out);
    switch (bb) {
    case 1: k_compact_rows<T, 1><<<grid, 256, 0, stream>>>(nrow, old_off, counts, new_off, cols_in, vi, cols_out, vo); break;
    case 4: k_compact_rows<T, 4><<<grid, 256, 0, stream>>>(nrow, old_off, counts, new_off, cols_in, vi, cols_out, vo); break;
    case 9: k_compact_rows<T, 9><<<grid, 256, 0, stream>>>(nrow, old_off, counts, new_off, cols_in, vi, cols_out, vo); break;
    default: gb::set_error("bsr_compact: block size must be 1, 4 or 9 scalars"); return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb

using namespace gb;

// Row starts of a candidate array whose row indices are non-decreasing (offsets[nrow + 1]; empty
// rows allowed).  Rows out of range or out of order set GB_DEV_BREAKDOWN in *status.
GB_API int gb_bsr_rows_to_offsets(int64_t T, const int* rows, int nrow, int* offsets, int* status, cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0 && T >= 0 && status != nullptr, "bsr_rows_to_offsets: bad arguments");
    if (T == 0) {
        GB_CHECK_CUDA(cudaMemsetAsync(offsets, 0, sizeof(int) * ((size_t)nrow + 1), stream));
        return GB_OK;
    }
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(T, 256), kSmCount * 32));
    k_rows_to_offsets<<<grid, 256, 0, stream>>>(T, rows, nrow, offsets, status);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// In-place row compression (see the file comment).  dtype GB_F32 / GB_F64; block_size = scalars per
// block (1, 4 or 9); row_counts may be null (rows end at offsets[r + 1]); out_counts[nrow].
GB_API int gb_bsr_compress_rows(int block_size, int dtype, int nrow, const int* offsets, const int* row_counts,
                                int* columns, void* values, int prune, uint64_t zero_mask, int* out_counts,
                                cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0, "bsr_compress_rows: negative row count");
    if (nrow == 0) return GB_OK;
    if (dtype == GB_F32)
        return launch_compress<float>(block_size, nrow, offsets, row_counts, columns, values, prune, zero_mask,
                                      out_counts, stream);
    if (dtype == GB_F64)
        return launch_compress<double>(block_size, nrow, offsets, row_counts, columns, values, prune, zero_mask,
                                       out_counts, stream);
    gb::set_error("bsr_compress_rows: dtype must be f32 or f64");
    return GB_ERR_UNSUPPORTED;
}

GB_API size_t gb_bsr_compact_workspace_bytes(int nrow) { return gb::scan_workspace_bytes((int64_t)nrow + 1); }

// Compact CSR from compressed rows: offsets_out = exclusive scan of counts (counts[nrow] must be 0,
// offsets_out[nrow] = total), then each row's first counts[r] blocks are gathered to offsets_out[r].
GB_API int gb_bsr_compact(int block_size, int dtype, int nrow, const int* old_offsets, int* counts,
                          const int* columns_in, const void* values_in, int* offsets_out, int* columns_out,
                          void* values_out, void* workspace, size_t workspace_bytes, cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0, "bsr_compact: negative row count");
    GB_REQUIRE(workspace_bytes >= gb_bsr_compact_workspace_bytes(nrow), "bsr_compact: workspace too small");
    int rc = gb::scan_i32(counts, offsets_out, (int64_t)nrow + 1, false, workspace, stream);
    if (rc != GB_OK) return rc;
    if (nrow == 0) return GB_OK;
    if (dtype == GB_F32)
        return launch_compact<float>(block_size, nrow, old_offsets, counts, offsets_out, columns_in, values_in,
                                     columns_out, values_out, stream);
    if (dtype == GB_F64)
        return launch_compact<double>(block_size, nrow, old_offsets, counts, offsets_out, columns_in, values_in,
                                      columns_out, values_out, stream);
    gb::set_error("bsr_compact: dtype must be f32 or f64");
    return GB_ERR_UNSUPPORTED;
}

// ---------------------------------------------------------------------------------------------
// Padded topology of bsr_set_from_triplets (warp/_src/sparse.py:1173-1230, 1335-1420): a compact
// triplet structure is written into the destination's existing row capacity.
// ---------------------------------------------------------------------------------------------
namespace gb {

// One thread per row: rows whose compact block count exceeds their capacity get row_counts = 0 and
// raise the status word (BSR_STATUS_ROW_CAPACITY_EXCEEDED = 1, atomic max); otherwise the compact
// columns are copied to the front of the padded row.  block_map[b] = compact block of padded slot b,
// or -1 for an unused slot (block_map may be null).
__global__ void k_scatter_padded(int nrow, const int* __restrict__ c_off, const int* __restrict__ c_cols,
                                 const int* __restrict__ d_off, int* __restrict__ d_counts, int* __restrict__ d_cols,
                                 int* __restrict__ block_map, int* __restrict__ status)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    const int cb = c_off[row];
    int cnt = c_off[row + 1] - cb;
    const int beg = d_off[row], cap_end = d_off[row + 1];
    if (beg + cnt > cap_end) {
        cnt = 0;
        atomicMax(status, 1);
    }
    d_counts[row] = cnt;
    for (int k = 0; k < cnt; ++k) {
        d_cols[beg + k] = c_cols[cb + k];
        if (block_map) block_map[beg + k] = cb + k;
    }
    if (block_map)
        for (int b = beg + cnt; b < cap_end; ++b) block_map[b] = -1;
}

// dst[b] = block_map[b] >= 0 ? src[block_map[b]] : 0, block_size scalars per block
template <typename T>
__global__ void k_gather_blocks(int64_t nblocks, int block_size, const int* __restrict__ block_map,
                                const T* __restrict__ src, T* __restrict__ dst)
{
    const int64_t total = nblocks * block_size;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = t / block_size;
        const int s = (int)(t - b * block_size);
        const int m = block_map[b];
        dst[t] = m >= 0 ? src[(size_t)m * block_size + s] : T(0);
    }
}

}  // namespace gb

GB_API int gb_bsr_scatter_padded(int nrow, const int* compact_offsets, const int* compact_columns,
                                 const int* dest_offsets, int* dest_row_counts, int* dest_columns, int* block_map,
                                 int* status, cudaStream_t stream)
{
    GB_REQUIRE(nrow >= 0, "bsr_scatter_padded: negative row count");
    GB_REQUIRE(nrow == 0 || (compact_offsets && compact_columns && dest_offsets && dest_row_counts && dest_columns &&
                             status), "bsr_scatter_padded: null argument");
    if (nrow == 0) return GB_OK;
    gb::k_scatter_padded<<<gb::ceil_div(nrow, 256), 256, 0, stream>>>(nrow, compact_offsets, compact_columns,
                                                                      dest_offsets, dest_row_counts, dest_columns,
                                                                      block_map, status);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_bsr_gather_blocks(int dtype, int block_size, int64_t nblocks, const int* block_map, const void* src,
                                void* dst, cudaStream_t stream)
{
    GB_REQUIRE(block_size >= 1 && nblocks >= 0, "bsr_gather_blocks: bad sizes");
    if (nblocks == 0) return GB_OK;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(gb::ceil_div<int64_t>(nblocks * block_size, 256),
                                                                 gb::kSmCount * 16));
    if (dtype == GB_F32)
        gb::k_gather_blocks<float><<<grid, 256, 0, stream>>>(nblocks, block_size, block_map,
                                                             static_cast<const float*>(src), static_cast<float*>(dst));
    else if (dtype == GB_F64)
        gb::k_gather_blocks<double><<<grid, 256, 0, stream>>>(nblocks, block_size, block_map,
                                                              static_cast<const double*>(src), static_cast<double*>(dst));
    else {
        gb::set_error("bsr_gather_blocks: float32 or float64 values");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
