// gb_spmv.cuh -- the BSR SpMV core shared by bsr_mv and the fused Krylov / refinement kernels.
//
// Persistent, warp-specialised TMA pipeline.  The matrix is cut into tiles of `rows` consecutive
// block rows; a tile's offsets slice, column indices and block values are three contiguous ranges,
// copied global -> shared by 1-D bulk copies (cp.async.bulk, completing on a "full" mbarrier).
// Each CTA owns tiles blockIdx.x, blockIdx.x + gridDim.x, ... and cycles them through a ring of
// `stages` shared-memory buffers:
//   * warp 0 (producer): waits for a buffer to be released ("empty" mbarrier), reads the tile's
//     first/last offsets (prefetched one tile ahead), issues the bulk copies (start rounded down
//     to 8 blocks so every copy is 16-byte aligned; the < 8-block / < 4-entry tails past the last
//     aligned element of an array are stored by the producer with plain loads);
//   * warps 1..16 (consumers): wait for a buffer, walk its rows with groups of G lanes per block
//     row, gather x through the read-only path (x fits the 129 MB L2 in every configuration),
//     reduce each row with shuffles, hand the row to the epilogue, release the buffer.
// Copies for the next tiles are in flight while the current one is computed, so HBM sees a
// continuous stream.  A tile whose blocks exceed the buffer is computed from global memory.
// Every mbarrier wait is bounded in wall time (gb_bulk.cuh); a timeout sets GB_DEV_WAIT_TIMEOUT.
#pragma once
#include "gb_bulk.cuh"
#include "gb_common.cuh"

namespace gb {

constexpr int SPMV_CONSUMER_WARPS = 16;
constexpr int SPMV_CONSUMERS = 32 * SPMV_CONSUMER_WARPS;  // 512 consumer threads
constexpr int SPMV_THREADS = SPMV_CONSUMERS + 32;         // + 1 producer warp
constexpr int SPMV_ALIGN = 8;       // blocks: 8 int32 columns = 32 B; 8 blocks of values = k*16 B
constexpr int SPMV_MAX_STAGES = 4;

struct SpmvShape {
    int rows;      // block rows per tile (multiple of 4)
    int G;         // lanes per block row (power of two, 1..32)
    int cap;       // staged blocks per buffer (multiple of 8; 0 = compute from global memory)
    int stages;    // ring depth (1..4)
    int grid;      // persistent CTAs
    int off_bulk;  // offsets array 16-byte aligned: its slices are bulk-copied too
    int64_t ncap;  // valid entries in the columns / values arrays
};

struct StageHeader {
    int r0, nr, a0, staged;
    int pad[4];
};

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

template <int BR, int BC, typename VT> __host__ __device__ inline size_t spmv_stage_bytes(int rows, int cap)
{
    return align16((size_t)(rows + 8) * sizeof(int)) + align16((size_t)cap * sizeof(int)) +
           align16((size_t)cap * BR * BC * sizeof(VT));
}

// mbarriers (2 x 4 x 8 B) + stage headers (4 x 32 B) + the ring
template <int BR, int BC, typename VT> __host__ __device__ inline size_t spmv_smem_bytes(int rows, int cap, int stages)
{
    return 64 + 128 + (size_t)stages * spmv_stage_bytes<BR, BC, VT>(rows, cap);
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

// Runtime-G group reduction (all 32 lanes of the warp participate).
template <typename T> __device__ __forceinline__ T group_reduce(T v, int G)
{
    for (int o = G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Select acc[i] for a runtime i without dynamic register indexing.
template <int BR, typename AT> __device__ __forceinline__ AT pick(const AT (&acc)[BR], int i)
{
    AT v = acc[0];
#pragma unroll
    for (int q = 1; q < BR; ++q)
        if (i == q) v = acc[q];
    return v;
}

// Default tile shape for a matrix (defined in gb_spmv.cu); `aligned` = columns and values are
// 16-byte aligned (staging allowed); offsets alignment is checked separately (off_bulk).
SpmvShape default_shape(int br, int bc, int val_dtype, int nrow, int64_t nnzb, int64_t ncap, bool aligned);
// Finalise a shape: round rows/cap, clamp stages and compute the persistent grid for `smem_bytes`.
void finalize_shape(SpmvShape& sh, int nrow, size_t smem_bytes, const int* offsets);
int sm_count();

// Ring layout shared by the producer and the consumers of one CTA.
struct SpmvRing {
    uint64_t* full;
    uint64_t* empty;
    StageHeader* hdr;
    unsigned char* ring;
    size_t off_bytes, col_bytes, stage_bytes;
};

template <int BR, int BC, typename VT>
__device__ __forceinline__ SpmvRing spmv_ring(unsigned char* smem, const SpmvShape& sh)
{
    SpmvRing R;
    R.full = reinterpret_cast<uint64_t*>(smem);
    R.empty = R.full + SPMV_MAX_STAGES;
    R.hdr = reinterpret_cast<StageHeader*>(smem + 64);
    R.off_bytes = align16((size_t)(sh.rows + 8) * sizeof(int));
    R.col_bytes = align16((size_t)sh.cap * sizeof(int));
    R.stage_bytes = spmv_stage_bytes<BR, BC, VT>(sh.rows, sh.cap);
    R.ring = smem + 192;
    return R;
}

// Producer lane: copy tile `tile` (block rows [r0, r0 + nr), blocks [b0, b1)) into ring slot s and
// arm its "full" barrier.  With `evict_first`, the column and value copies carry an L2 evict-first
// policy (a matrix streamed once per pass should not push the vectors out of L2).
template <int BR, int BC, typename VT>
__device__ __forceinline__ void spmv_issue(const SpmvRing& R, const SpmvShape& sh, int nrow, int s, int tile, int b0,
                                           int b1, const int* __restrict__ offsets, const int* __restrict__ columns,
                                           const VT* __restrict__ values, bool evict_first, uint64_t policy)
{
    constexpr int BB = BR * BC;
    const int r0 = tile * sh.rows;
    const int nr = min(sh.rows, nrow - r0);
    const int64_t ncap8 = sh.ncap & ~(int64_t)(SPMV_ALIGN - 1);
    unsigned char* st = R.ring + (size_t)s * R.stage_bytes;
    int* s_off = reinterpret_cast<int*>(st);
    int* s_cols = reinterpret_cast<int*>(st + R.off_bytes);
    VT* s_vals = reinterpret_cast<VT*>(st + R.off_bytes + R.col_bytes);
    const int a0 = b0 & ~(SPMV_ALIGN - 1);
    const bool staged = (sh.cap > 0) && (b1 - a0 <= sh.cap);
    // offsets slice [r0, r0 + nr]: bulk part (multiple of 4 entries inside the array)
    int n_off = sh.off_bulk ? min((nr + 1 + 3) & ~3, (nrow + 1 - r0) & ~3) : 0;
    n_off = max(n_off, 0);
    for (int k = n_off; k <= nr; ++k) s_off[k] = offsets[r0 + k];
    uint32_t bytes = (uint32_t)n_off * 4u;
    int a1 = a0, nb = 0;
    if (staged) {
        a1 = (int)min((int64_t)((b1 + SPMV_ALIGN - 1) & ~(SPMV_ALIGN - 1)), ncap8);
        a1 = max(a1, a0);
        nb = a1 - a0;
        for (int b = a1; b < b1; ++b) {
            s_cols[b - a0] = columns[b];
#pragma unroll
            for (int q = 0; q < BB; ++q) s_vals[(size_t)(b - a0) * BB + q] = values[(size_t)b * BB + q];
        }
        bytes += (uint32_t)nb * (uint32_t)(sizeof(int) + BB * sizeof(VT));
    }
    StageHeader& h = R.hdr[s];
    h.r0 = r0;
    h.nr = nr;
    h.a0 = a0;
    h.staged = staged ? 1 : 0;
    mbar_arrive_expect_tx(&R.full[s], bytes);
    if (n_off > 0) bulk_g2s(s_off, offsets + r0, (uint32_t)n_off * 4u, &R.full[s]);
    if (nb > 0) {
        if (evict_first) {
            bulk_g2s_hint(s_cols, columns + a0, (uint32_t)nb * 4u, &R.full[s], policy);
            bulk_g2s_hint(s_vals, values + (size_t)a0 * BB, (uint32_t)nb * (uint32_t)(BB * sizeof(VT)), &R.full[s],
                          policy);
        } else {
            bulk_g2s(s_cols, columns + a0, (uint32_t)nb * 4u, &R.full[s]);
            bulk_g2s(s_vals, values + (size_t)a0 * BB, (uint32_t)nb * (uint32_t)(BB * sizeof(VT)), &R.full[s]);
        }
    }
}

// Computes acc[BR] = (A x)[row] for every block row of every tile this CTA owns and calls
// epi(row, acc, lane_in_group) on the consumer lanes of the row's group (all lanes of the group
// hold the sums).  Must be called by all SPMV_THREADS threads; returns with the CTA converged
// (after a __syncthreads), so the caller may reduce block-wide afterwards.
template <int BR, int BC, typename VT, typename XT, typename AT, typename Epi>
__device__ __forceinline__ void spmv_run(int nrow, const SpmvShape sh, const int* __restrict__ offsets,
                                         const int* __restrict__ row_counts, const int* __restrict__ columns,
                                         const VT* __restrict__ values, const XT* __restrict__ x, unsigned char* smem,
                                         int* status, Epi& epi)
{
    constexpr int BB = BR * BC;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    uint64_t* empty = full + SPMV_MAX_STAGES;
    StageHeader* hdr = reinterpret_cast<StageHeader*>(smem + 64);
    const size_t off_bytes = align16((size_t)(sh.rows + 8) * sizeof(int));
    const size_t col_bytes = align16((size_t)sh.cap * sizeof(int));
    const size_t stage_bytes = spmv_stage_bytes<BR, BC, VT>(sh.rows, sh.cap);
    unsigned char* ring = smem + 192;
    const int S = sh.stages;
    const int ntiles = (nrow + sh.rows - 1) / sh.rows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], SPMV_CONSUMER_WARPS);
        }
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == 0) {
        // ------------------------------- producer ------------------------------------------
        if (lane == 0) {
            int tile = blockIdx.x;
            int nb0 = 0, nb1 = 0;
            if (tile < ntiles) {
                const int r0 = tile * sh.rows;
                nb0 = offsets[r0];
                nb1 = offsets[min(r0 + sh.rows, nrow)];
            }
            const int64_t ncap8 = sh.ncap & ~(int64_t)(SPMV_ALIGN - 1);
            bool timed_out = false;
            int issued = 0;
            for (int i = 0; tile < ntiles; ++i, tile += gridDim.x) {
                const int s = i % S;
                const uint32_t ph = (uint32_t)(i / S) & 1u;
                const int r0 = tile * sh.rows;
                const int nr = min(sh.rows, nrow - r0);
                const int b0 = nb0, b1 = nb1;
                // prefetch the next tile's range while this one is being issued / consumed
                const int ntile = tile + gridDim.x;
                if (ntile < ntiles) {
                    const int nr0 = ntile * sh.rows;
                    nb0 = offsets[nr0];
                    nb1 = offsets[min(nr0 + sh.rows, nrow)];
                }
                if (i >= S && !mbar_wait_bounded(&empty[s], ph ^ 1u)) {
                    timed_out = true;
                    break;
                }
                unsigned char* st = ring + (size_t)s * stage_bytes;
                int* s_off = reinterpret_cast<int*>(st);
                int* s_cols = reinterpret_cast<int*>(st + off_bytes);
                VT* s_vals = reinterpret_cast<VT*>(st + off_bytes + col_bytes);
                const int a0 = b0 & ~(SPMV_ALIGN - 1);
                const bool staged = (sh.cap > 0) && (b1 - a0 <= sh.cap);
                // offsets slice [r0, r0 + nr]: bulk part (multiple of 4 entries inside the array)
                int n_off = sh.off_bulk ? min((nr + 1 + 3) & ~3, (nrow + 1 - r0) & ~3) : 0;
                n_off = max(n_off, 0);
                for (int k = n_off; k <= nr; ++k) s_off[k] = offsets[r0 + k];
                uint32_t bytes = (uint32_t)n_off * 4u;
                int a1 = a0, nb = 0;
                if (staged) {
                    a1 = (int)min((int64_t)((b1 + SPMV_ALIGN - 1) & ~(SPMV_ALIGN - 1)), ncap8);
                    a1 = max(a1, a0);
                    nb = a1 - a0;
                    for (int b = a1; b < b1; ++b) {
                        s_cols[b - a0] = columns[b];
#pragma unroll
                        for (int q = 0; q < BB; ++q) s_vals[(size_t)(b - a0) * BB + q] = values[(size_t)b * BB + q];
                    }
                    bytes += (uint32_t)nb * (uint32_t)(sizeof(int) + BB * sizeof(VT));
                }
                StageHeader& h = hdr[s];
                h.r0 = r0;
                h.nr = nr;
                h.a0 = a0;
                h.staged = staged ? 1 : 0;
                mbar_arrive_expect_tx(&full[s], bytes);
                if (n_off > 0) bulk_g2s(s_off, offsets + r0, (uint32_t)n_off * 4u, &full[s]);
                if (nb > 0) {
                    bulk_g2s(s_cols, columns + a0, (uint32_t)nb * 4u, &full[s]);
                    bulk_g2s(s_vals, values + (size_t)a0 * BB, (uint32_t)nb * (uint32_t)(BB * sizeof(VT)), &full[s]);
                }
                ++issued;
            }
            if (timed_out && status) atomicOr(status, GB_DEV_WAIT_TIMEOUT);
            // drain: no bulk copy of this CTA may still be in flight when it moves on
            for (int j = max(0, issued - S); j < issued; ++j)
                mbar_wait_bounded(&full[j % S], (uint32_t)(j / S) & 1u);
        }
    } else {
        // ------------------------------- consumers -----------------------------------------
        const int ct = threadIdx.x - 32;
        const int G = sh.G;
        const int lane_g = ct & (G - 1);
        const int g = ct / G;
        const int ngroups = SPMV_CONSUMERS / G;
        int i = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
            const int s = i % S;
            const uint32_t ph = (uint32_t)(i / S) & 1u;
            const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], ph));
            if (ok) {
                const StageHeader h = hdr[s];
                unsigned char* st = ring + (size_t)s * stage_bytes;
                const int* s_off = reinterpret_cast<const int*>(st);
                const int* cbase = h.staged ? reinterpret_cast<const int*>(st + off_bytes) - h.a0 : columns;
                const VT* vbase = h.staged ? reinterpret_cast<const VT*>(st + off_bytes + col_bytes) - (size_t)h.a0 * BB
                                           : values;
                // warp-uniform trip count: rows past the tile end are inactive lanes, so the
                // full-mask shuffles below never wait on an exited lane
                for (int kb = 0; kb < h.nr; kb += ngroups) {
                    const int k = kb + g;
                    const bool active = k < h.nr;
                    int beg = 0, end = 0;
                    if (active) {
                        beg = s_off[k];
                        end = row_counts ? beg + row_counts[h.r0 + k] : s_off[k + 1];
                    }
                    AT acc[BR];
#pragma unroll
                    for (int q = 0; q < BR; ++q) acc[q] = AT(0);
                    // U blocks per lane per batch, predicated: all U gathers are issued before
                    // any is consumed, so each lane keeps U * BC loads in flight
                    constexpr int U = (BB == 1) ? 8 : 4;
                    for (int base = beg + lane_g; base < end; base += U * G) {
                        int cc[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const int bi = base + u * G;
                            cc[u] = (bi < end) ? cbase[bi] : -1;
                        }
                        AT xv[U][BC];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
#pragma unroll
                            for (int j = 0; j < BC; ++j) xv[u][j] = (cc[u] >= 0) ? ldx<AT>(x + (size_t)cc[u] * BC + j) : AT(0);
                        }
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const int bi = base + u * G;
                            if (cc[u] >= 0) {
                                const VT* vv = vbase + (size_t)bi * BB;
#pragma unroll
                                for (int q = 0; q < BR; ++q) {
#pragma unroll
                                    for (int j = 0; j < BC; ++j) acc[q] += cvt<AT>(vv[q * BC + j]) * xv[u][j];
                                }
                            }
                        }
                    }
#pragma unroll
                    for (int q = 0; q < BR; ++q) acc[q] = group_reduce(acc[q], G);
                    if (active) epi(h.r0 + k, acc, lane_g);
                }
            } else if (lane == 0 && status) {
                atomicOr(status, GB_DEV_WAIT_TIMEOUT);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
    }
    __syncthreads();
}

// Same tile walk without a product (acc = 0): for epilogues that only need the row loop.
template <int BR, typename AT, typename Epi>
__device__ __forceinline__ void rows_run(int nrow, const SpmvShape sh, Epi& epi)
{
    if (threadIdx.x >= 32) {
        const int ct = threadIdx.x - 32;
        const int G = sh.G;
        const int lane_g = ct & (G - 1);
        const int ngroups = SPMV_CONSUMERS / G;
        const int ntiles = (nrow + sh.rows - 1) / sh.rows;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const int r0 = tile * sh.rows, nr = min(sh.rows, nrow - r0);
            for (int k = ct / G; k < nr; k += ngroups) {
                AT acc[BR];
#pragma unroll
                for (int q = 0; q < BR; ++q) acc[q] = AT(0);
                epi(r0 + k, acc, lane_g);
            }
        }
    }
    __syncthreads();
}

}  // namespace gb
