// gb_triplets.cu -- COO triplets -> BSR topology and values (bsr_set_from_triplets).
//
// Drop-in replacement for wp_bsr_matrix_from_triplets_device (warp/native/sparse.cu:1168-1325)
// and the value pass _bsr_accumulate_triplet_values (warp/_src/sparse.py:1073-1090,1122-1141).
//
// Design (GB300): the reference sorts full 64-bit (row<<32|col) keys with CUB (8 radix passes).
// Here the key is packed into only bitlen(nrow) + bitlen(ncol-1) bits -- 32-bit keys when that
// fits -- and sorted by an LSD radix sort with 8-bit digits, so a 96^3 Q1 problem (40-bit keys)
// takes 5 passes and a 64^2 one (26-bit keys) 4 passes over 4-byte keys.  Each pass is a
// per-tile digit histogram, one device scan of the (digit, tile) table and a stable scatter
// that ranks keys inside a tile with warp match-any and stages the tile in shared memory so
// global writes are runs per digit.  Pruned triplets get the key (nrow << colbits), which sorts
// after every valid key exactly as the reference's ~0 key does, so tpl_block_indices and the
// BSR structure are identical to the reference's stable device path.
#include "gb_common.cuh"
#include "gb_scan.cuh"

namespace gb {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_IPL = 16;                            // items per lane
constexpr int RS_TILE = RS_THREADS * RS_IPL;          // 4096 keys per CTA tile
constexpr int RS_WARP_ITEMS = 32 * RS_IPL;            // 512 consecutive keys per warp
constexpr int RS_RADIX = 256;

static inline int bitlen(uint32_t v)
{
    int b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

// ---------------------------------------------------------------------------------------------
// Key construction (restates bsr_fill_triplet_key_values, sparse.cu:315-336, with the pruning
// predicates BsrBlockInMask and BsrBlockIsNotZero, sparse.cu:245-311).
// ---------------------------------------------------------------------------------------------
template <typename K>
__global__ void k_fill_keys(int nnz, const int* __restrict__ tpl_nnz, const int* __restrict__ rows,
                            const int* __restrict__ cols, const void* __restrict__ values, int scalar_size,
                            int block_size, uint64_t zero_mask, int nrow, int ncol, int colbits,
                            const int* __restrict__ m_offsets, const int* __restrict__ m_row_counts,
                            const int* __restrict__ m_columns, K* __restrict__ keys, int* __restrict__ idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnz) return;
    const K pruned = (K)nrow << colbits;
    const int r = rows[i], c = cols[i];
    bool keep = (r >= 0 && r < nrow && c >= 0 && c < ncol);
    if (keep && tpl_nnz) keep = i < *tpl_nnz;
    if (keep && m_offsets) {
        int lower = m_offsets[r];
        int end = m_row_counts ? lower + m_row_counts[r] : m_offsets[r + 1];
        int upper = end - 1;
        if (upper < lower) {
            keep = false;
        } else {
            while (lower < upper) {
                int mid = lower + (upper - lower) / 2;
                if (m_columns[mid] < c) lower = mid + 1; else upper = mid;
            }
            keep = (m_columns[lower] == c);
        }
    }
    if (keep && values && zero_mask) {
        bool nonzero = false;
        const char* p = static_cast<const char*>(values) + (size_t)i * block_size * scalar_size;
        for (int s = 0; s < block_size && !nonzero; ++s) {
            uint64_t bits;
            switch (scalar_size) {
            case 1: bits = reinterpret_cast<const uint8_t*>(p)[s]; break;
            case 2: bits = reinterpret_cast<const uint16_t*>(p)[s]; break;
            case 4: bits = reinterpret_cast<const uint32_t*>(p)[s]; break;
            default: bits = reinterpret_cast<const uint64_t*>(p)[s]; break;
            }
            nonzero = (bits & zero_mask) != 0;
        }
        keep = nonzero;
    }
    keys[i] = keep ? (((K)r << colbits) | (K)c) : pruned;
    idx[i] = i;
}

// ---------------------------------------------------------------------------------------------
// Radix pass, step 1: per-tile digit histogram, digit-major: hist[d * ntiles + tile].
// ---------------------------------------------------------------------------------------------
template <typename K>
__global__ __launch_bounds__(RS_THREADS) void k_radix_hist(const K* __restrict__ keys, int n, int shift, int ntiles,
                                                           int* __restrict__ hist)
{
    __shared__ int s_hist[RS_RADIX];
    s_hist[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int k = 0; k < RS_IPL; ++k) {
        int64_t i = base + k * RS_THREADS + threadIdx.x;
        int d = (i < n) ? (int)((keys[i] >> shift) & 0xFF) : RS_RADIX;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        if (d < RS_RADIX && lane == __ffs(peers) - 1) atomicAdd(&s_hist[d], __popc(peers));
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = s_hist[threadIdx.x];
}

// ---------------------------------------------------------------------------------------------
// Radix pass, step 3: stable scatter.  Warp w owns keys [w*512, (w+1)*512) of the tile, so the
// tile order is (warp, round, lane) = input order.  Rank of a key inside its digit =
// (same digit in earlier warps) + (same digit in earlier rounds of this warp) + (earlier lanes
// of this round, via match-any).  Keys are placed in shared memory in (digit, rank) order and
// written out as contiguous runs per digit.
// ---------------------------------------------------------------------------------------------
template <typename K>
__global__ __launch_bounds__(RS_THREADS) void k_radix_scatter(const K* __restrict__ kin, const int* __restrict__ vin,
                                                              K* __restrict__ kout, int* __restrict__ vout, int n,
                                                              int shift, int ntiles, const int* __restrict__ hist_scan)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    K* s_k = reinterpret_cast<K*>(smem_raw);
    int* s_v = reinterpret_cast<int*>(s_k + RS_TILE);
    int* s_whist = s_v + RS_TILE;                     // [RS_WARPS][RS_RADIX]
    int* s_dstart = s_whist + RS_WARPS * RS_RADIX;    // [RS_RADIX] tile-local digit start
    int* s_gbase = s_dstart + RS_RADIX;               // [RS_RADIX] global start of (digit, tile)
    int* s_scan = s_gbase + RS_RADIX;                 // [33] block scan scratch

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t tile_base = (int64_t)blockIdx.x * RS_TILE;
    const int64_t wbase = tile_base + w * RS_WARP_ITEMS;
    const unsigned lt_mask = (1u << lane) - 1u;

    for (int t = threadIdx.x; t < RS_WARPS * RS_RADIX; t += RS_THREADS) s_whist[t] = 0;
    __syncthreads();

    K k[RS_IPL];
    int v[RS_IPL];
    int d[RS_IPL];
#pragma unroll
    for (int r = 0; r < RS_IPL; ++r) {
        int64_t i = wbase + r * 32 + lane;
        bool valid = i < n;
        k[r] = valid ? kin[i] : (K)0;
        v[r] = valid ? vin[i] : 0;
        d[r] = valid ? (int)((k[r] >> shift) & 0xFF) : RS_RADIX;
    }
#pragma unroll
    for (int r = 0; r < RS_IPL; ++r) {
        unsigned peers = __match_any_sync(0xffffffffu, d[r]);
        if (d[r] < RS_RADIX && lane == __ffs(peers) - 1) s_whist[w * RS_RADIX + d[r]] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    // Thread t owns digit t: prefix over warps, then exclusive scan of digit totals in the tile.
    {
        const int t = threadIdx.x;
        int tot = 0;
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ++ww) {
            int c = s_whist[ww * RS_RADIX + t];
            s_whist[ww * RS_RADIX + t] = tot;
            tot += c;
        }
        // block exclusive scan of tot over the 256 digits
        int incl = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_scan[w] = incl;
        __syncthreads();
        if (w == 0) {
            int x = (lane < RS_WARPS) ? s_scan[lane] : 0;
            int xi = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, xi, o);
                if (lane >= o) xi += y;
            }
            if (lane < RS_WARPS) s_scan[lane] = xi - x;
        }
        __syncthreads();
        const int dstart = incl - tot + s_scan[w];
        s_dstart[t] = dstart;
        s_gbase[t] = hist_scan[(size_t)t * ntiles + blockIdx.x];
#pragma unroll
        for (int ww = 0; ww < RS_WARPS; ++ww) s_whist[ww * RS_RADIX + t] += dstart;
    }
    __syncthreads();

#pragma unroll
    for (int r = 0; r < RS_IPL; ++r) {
        unsigned peers = __match_any_sync(0xffffffffu, d[r]);
        if (d[r] < RS_RADIX) {
            int pos = s_whist[w * RS_RADIX + d[r]] + __popc(peers & lt_mask);
            s_k[pos] = k[r];
            s_v[pos] = v[r];
        }
        __syncwarp();
        if (d[r] < RS_RADIX && lane == __ffs(peers) - 1) s_whist[w * RS_RADIX + d[r]] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();

    const int count = (int)min((int64_t)RS_TILE, (int64_t)n - tile_base);
    for (int i = threadIdx.x; i < count; i += RS_THREADS) {
        K kk = s_k[i];
        int dd = (int)((kk >> shift) & 0xFF);
        int o = s_gbase[dd] + (i - s_dstart[dd]);
        kout[o] = kk;
        vout[o] = s_v[i];
    }
}

// ---------------------------------------------------------------------------------------------
// Run encoding of the sorted keys (replaces cub::DeviceRunLengthEncode + bsr_find_row_offsets
// + bsr_set_column, sparse.cu:339-381,1267-1300).
// ---------------------------------------------------------------------------------------------
template <typename K>
__global__ void k_run_flags(const K* __restrict__ keys, int n, K pruned, int* __restrict__ flags)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    K k = keys[i];
    flags[i] = (k != pruned && (i == 0 || keys[i - 1] != k)) ? 1 : 0;
}

// blk = inclusive scan of the run-start flags: run index of element i is blk[i]-1.
template <typename K>
__global__ void k_run_emit(const K* __restrict__ keys, const int* __restrict__ blk, int n, K pruned, int colbits,
                           int nrow, int* __restrict__ bsr_offsets, int* __restrict__ bsr_columns,
                           int* __restrict__ tpl_block_offsets)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const K k = keys[i];
    if (k == pruned) return;
    const int b = blk[i] - 1;
    const int row = (int)(k >> colbits);
    const K colmask = ((K)1 << colbits) - 1;
    const bool start = (i == 0) || (keys[i - 1] != k);
    const bool last_valid = (i == n - 1) || (keys[i + 1] == pruned);
    const bool end = last_valid || (keys[i + 1] != k);
    if (start) {
        bsr_columns[b] = (int)(k & colmask);
        const int prev_row = (i == 0) ? -1 : (int)(keys[i - 1] >> colbits);
        for (int r = prev_row + 1; r <= row; ++r) bsr_offsets[r] = b;
    }
    if (end) tpl_block_offsets[b] = i + 1;
    if (last_valid) {
        for (int r = row + 1; r <= nrow; ++r) bsr_offsets[r] = b + 1;
    }
}

// ---------------------------------------------------------------------------------------------
// Values: bsr_values[b, s] = sum over the run of tpl_values[idx[k], s], first term assigned then
// added in sorted order in the matrix scalar type (restates sparse.py:1122-1141).  Grid-stride
// over (block, scalar) with the block count read on the device (no host sync).
// ---------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_accumulate_values(int nrow, const int* __restrict__ bsr_offsets,
                                    const int* __restrict__ tpl_block_offsets,
                                    const int* __restrict__ tpl_block_indices, const T* __restrict__ tpl_values,
                                    int block_size, T* __restrict__ bsr_values)
{
    const int64_t nnzb = bsr_offsets[nrow];
    const int64_t total = nnzb * block_size;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = t / block_size;
        const int s = (int)(t - b * block_size);
        const int beg = (b == 0) ? 0 : tpl_block_offsets[b - 1];
        const int end = tpl_block_offsets[b];
        T v = tpl_values[(size_t)tpl_block_indices[beg] * block_size + s];
        for (int q = beg + 1; q < end; ++q) v += tpl_values[(size_t)tpl_block_indices[q] * block_size + s];
        bsr_values[t] = v;
    }
}

struct TripletPlan {
    int colbits, bits, npasses, key_bytes, ntiles;
    size_t keys_bytes, hist_bytes, scan_bytes, idx_bytes, total;
};

static TripletPlan make_plan(int nnz, int nrow, int ncol)
{
    TripletPlan p;
    p.colbits = bitlen((uint32_t)(ncol > 0 ? ncol - 1 : 0));
    p.bits = p.colbits + bitlen((uint32_t)nrow);
    p.key_bytes = (p.bits <= 32) ? 4 : 8;
    p.npasses = (p.bits + 7) / 8;
    p.ntiles = (int)ceil_div<int64_t>(nnz, RS_TILE);
    auto align = [](size_t b) { return (b + 255) & ~(size_t)255; };
    p.keys_bytes = align((size_t)nnz * p.key_bytes);
    p.hist_bytes = align((size_t)RS_RADIX * p.ntiles * sizeof(int));
    p.idx_bytes = align((size_t)nnz * sizeof(int));
    size_t scan_n = std::max<size_t>((size_t)RS_RADIX * p.ntiles, (size_t)nnz);
    p.scan_bytes = align(scan_workspace_bytes((int64_t)scan_n));
    // keysA, keysB, hist, scan scratch, and two index buffers used when the caller does not
    // return the summed-block arrays.
    p.total = 2 * p.keys_bytes + p.hist_bytes + p.scan_bytes + 2 * p.idx_bytes + 256;
    return p;
}

template <typename K>
static int from_triplets_impl(const TripletPlan& P, int block_size, int scalar_size, int nrow, int ncol, int nnz,
                              const int* tpl_nnz, const int* rows, const int* cols, const void* values,
                              uint64_t zero_mask, bool masked, int* tbo, int* tbi, int* bsr_offsets,
                              const int* bsr_row_counts, int* bsr_columns, int* bsr_nnz_host, cudaEvent_t nnz_event,
                              unsigned char* ws, cudaStream_t stream)
{
    K* keysA = reinterpret_cast<K*>(ws);
    K* keysB = reinterpret_cast<K*>(ws + P.keys_bytes);
    int* hist = reinterpret_cast<int*>(ws + 2 * P.keys_bytes);
    void* scan_ws = ws + 2 * P.keys_bytes + P.hist_bytes;
    unsigned char* idx_area = ws + 2 * P.keys_bytes + P.hist_bytes + P.scan_bytes;
    if (!tbo || !tbi) {
        tbo = reinterpret_cast<int*>(idx_area);
        tbi = reinterpret_cast<int*>(idx_area + P.idx_bytes);
    }
    const K pruned = (K)nrow << P.colbits;

    if (nnz == 0) GB_CHECK_CUDA(cudaMemsetAsync(bsr_offsets, 0, sizeof(int) * (size_t)(nrow + 1), stream));
    if (nnz > 0) {
        const int T = 256;
        // Indices start in tpl_block_indices; tpl_block_offsets is the alternate buffer (as in
        // the reference, sparse.cu:1193).
        k_fill_keys<K><<<ceil_div(nnz, T), T, 0, stream>>>(
            nnz, tpl_nnz, rows, cols, values, scalar_size, block_size, zero_mask, nrow, ncol, P.colbits,
            masked ? bsr_offsets : nullptr, masked ? bsr_row_counts : nullptr, masked ? bsr_columns : nullptr, keysA,
            tbi);
        GB_CHECK_CUDA(cudaGetLastError());

        const size_t smem = (size_t)RS_TILE * (sizeof(K) + sizeof(int)) +
                            (size_t)(RS_WARPS * RS_RADIX + 2 * RS_RADIX + 64) * sizeof(int);
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_radix_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        K* kin = keysA;
        K* kout = keysB;
        int* vin = tbi;
        int* vout = tbo;
        for (int pass = 0; pass < P.npasses; ++pass) {
            const int shift = pass * 8;
            k_radix_hist<K><<<P.ntiles, RS_THREADS, 0, stream>>>(kin, nnz, shift, P.ntiles, hist);
            GB_CHECK_CUDA(cudaGetLastError());
            int rc = scan_i32(hist, hist, (int64_t)RS_RADIX * P.ntiles, false, scan_ws, stream);
            if (rc) return rc;
            k_radix_scatter<K><<<P.ntiles, RS_THREADS, smem, stream>>>(kin, vin, kout, vout, nnz, shift, P.ntiles,
                                                                       hist);
            GB_CHECK_CUDA(cudaGetLastError());
            std::swap(kin, kout);
            std::swap(vin, vout);
        }
        if (vin != tbi) GB_CHECK_CUDA(cudaMemcpyAsync(tbi, vin, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToDevice, stream));
        // Sorted keys are in kin; kout is free and serves as the run-index buffer.
        int* blk = reinterpret_cast<int*>(kout);
        k_run_flags<K><<<ceil_div(nnz, T), T, 0, stream>>>(kin, nnz, pruned, blk);
        GB_CHECK_CUDA(cudaGetLastError());
        int rc = scan_i32(blk, blk, nnz, true, scan_ws, stream);
        if (rc) return rc;
        // Offsets are cleared only now: in masked mode the key pass above read the existing
        // topology from the same arrays.  With no valid key the zeros are the result.
        GB_CHECK_CUDA(cudaMemsetAsync(bsr_offsets, 0, sizeof(int) * (size_t)(nrow + 1), stream));
        k_run_emit<K><<<ceil_div(nnz, T), T, 0, stream>>>(kin, blk, nnz, pruned, P.colbits, nrow, bsr_offsets,
                                                          bsr_columns, tbo);
        GB_CHECK_CUDA(cudaGetLastError());
    }
    if (bsr_nnz_host) {
        GB_CHECK_CUDA(cudaMemcpyAsync(bsr_nnz_host, bsr_offsets + nrow, sizeof(int), cudaMemcpyDeviceToHost, stream));
        if (nnz_event) GB_CHECK_CUDA(cudaEventRecord(nnz_event, stream));
    }
    return GB_OK;
}

}  // namespace gb

using namespace gb;

GB_API size_t gb_bsr_from_triplets_workspace_bytes(int nnz, int nrow, int ncol)
{
    return make_plan(nnz, nrow, ncol).total;
}

// Replaces wp_bsr_matrix_from_triplets_device (warp/native/warp.h:583, sparse.cu:1168-1325).
// Same arguments and semantics, plus a caller-provided workspace (no allocation inside) and the
// stream.  bsr_nnz_host (optional) receives offsets[nrow] asynchronously; nnz_event (optional,
// a cudaEvent_t) is recorded after that copy.  tpl_block_offsets / tpl_block_indices may be
// null, in which case the workspace holds them.
GB_API int gb_bsr_matrix_from_triplets_device(int block_size, int scalar_size, int row_count, int col_count, int nnz,
                                              const int* tpl_nnz, const int* tpl_rows, const int* tpl_columns,
                                              const void* tpl_values, uint64_t scalar_zero_mask, int masked_topology,
                                              int* tpl_block_offsets, int* tpl_block_indices, int* bsr_offsets,
                                              const int* bsr_row_counts, int* bsr_columns, int* bsr_nnz_host,
                                              void* bsr_nnz_event, void* workspace, size_t workspace_bytes,
                                              cudaStream_t stream)
{
    GB_REQUIRE(row_count >= 0 && col_count >= 0 && nnz >= 0, "from_triplets: negative size");
    GB_REQUIRE(row_count < (1 << 30) && col_count < (1 << 30), "from_triplets: row/column count too large");
    GB_REQUIRE(bsr_offsets != nullptr && bsr_columns != nullptr, "from_triplets: null output arrays");
    GB_REQUIRE(nnz == 0 || (tpl_rows && tpl_columns), "from_triplets: null triplet arrays");
    if (scalar_zero_mask == 0 || tpl_values == nullptr) scalar_size = 0;
    GB_REQUIRE(scalar_size == 0 || scalar_size == 1 || scalar_size == 2 || scalar_size == 4 || scalar_size == 8,
               "from_triplets: unsupported scalar size %d", scalar_size);
    TripletPlan P = make_plan(nnz, row_count, col_count);
    GB_REQUIRE(P.bits <= 64, "from_triplets: key does not fit 64 bits");
    GB_REQUIRE(workspace_bytes >= P.total, "from_triplets: workspace too small (%zu < %zu)", workspace_bytes, P.total);
    unsigned char* ws = reinterpret_cast<unsigned char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    GB_REQUIRE(ws + (P.total - 256) <= (unsigned char*)workspace + workspace_bytes, "from_triplets: workspace alignment");
    if (P.key_bytes == 4)
        return from_triplets_impl<uint32_t>(P, block_size, scalar_size, row_count, col_count, nnz, tpl_nnz, tpl_rows,
                                            tpl_columns, tpl_values, scalar_zero_mask, masked_topology != 0,
                                            tpl_block_offsets, tpl_block_indices, bsr_offsets, bsr_row_counts,
                                            bsr_columns, bsr_nnz_host, (cudaEvent_t)bsr_nnz_event, ws, stream);
    return from_triplets_impl<uint64_t>(P, block_size, scalar_size, row_count, col_count, nnz, tpl_nnz, tpl_rows,
                                        tpl_columns, tpl_values, scalar_zero_mask, masked_topology != 0,
                                        tpl_block_offsets, tpl_block_indices, bsr_offsets, bsr_row_counts,
                                        bsr_columns, bsr_nnz_host, (cudaEvent_t)bsr_nnz_event, ws, stream);
}

// Replaces the _bsr_accumulate_triplet_values launch (warp/_src/sparse.py:1503-1515).
// dtype: GB_F32 or GB_F64.  values are [nnz_triplets, block_size] scalars; output [nnzb, block_size].
GB_API int gb_bsr_accumulate_triplet_values(int dtype, int block_size, int row_count, const int* bsr_offsets,
                                            const int* tpl_block_offsets, const int* tpl_block_indices,
                                            const void* tpl_values, void* bsr_values, int nnz_upper,
                                            cudaStream_t stream)
{
    GB_REQUIRE(block_size >= 1, "accumulate: bad block size");
    if (nnz_upper <= 0) return GB_OK;
    int grid = std::min<int64_t>(ceil_div<int64_t>((int64_t)nnz_upper * block_size, 256), (int64_t)kSmCount * 32);
    if (dtype == GB_F32) {
        k_accumulate_values<float><<<grid, 256, 0, stream>>>(row_count, bsr_offsets, tpl_block_offsets,
                                                            tpl_block_indices, (const float*)tpl_values, block_size,
                                                            (float*)bsr_values);
    } else if (dtype == GB_F64) {
        k_accumulate_values<double><<<grid, 256, 0, stream>>>(row_count, bsr_offsets, tpl_block_offsets,
                                                             tpl_block_indices, (const double*)tpl_values, block_size,
                                                             (double*)bsr_values);
    } else {
        gb::set_error("accumulate: unsupported dtype %d", dtype);
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
