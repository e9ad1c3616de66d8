// gb_scan.cu -- device-wide int32 prefix sums (reduce-then-scan, no inter-CTA waiting).
//
// Replaces the CUB scans the reference calls on this path (cub::DeviceScan::InclusiveSum at
// warp/native/sparse.cu:1305-1317 and wp_array_scan_int_device, warp/native/scan.cu).  Each
// level scans tiles of 4096 values in one CTA, writes per-tile totals, scans those totals
// recursively and adds them back; every CTA runs independently (no spin waits).
#include "gb_common.cuh"
#include "gb_scan.cuh"

namespace gb {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_IPT = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;
static_assert(SCAN_TILE == kScanTileElems, "gb_scan.cuh tile size out of date");

// Exclusive block scan of one int per thread; returns the block total in *total.
__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp, int* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < (SCAN_THREADS >> 5)) ? s_warp[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < (SCAN_THREADS >> 5)) s_warp[lane] = wi - w;
        if (lane == (SCAN_THREADS >> 5) - 1) s_warp[32] = wi;
    }
    __syncthreads();
    int excl = incl - v + s_warp[wid];
    *total = s_warp[32];
    __syncthreads();
    return excl;
}

// Scan one tile of SCAN_TILE values (striped loads through shared memory), writing the local
// scan to `out` and the tile total to tile_sums[blockIdx.x] (when non-null).
__global__ __launch_bounds__(SCAN_THREADS) void k_scan_tiles(const int* in, int* out, int64_t n, int inclusive,
                                                              int* tile_sums)
{
    __shared__ int s_data[SCAN_TILE];
    __shared__ int s_warp[33];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        int64_t i = base + k * SCAN_THREADS + threadIdx.x;
        s_data[k * SCAN_THREADS + threadIdx.x] = (i < n) ? in[i] : 0;
    }
    __syncthreads();
    int vals[SCAN_IPT];
    int sum = 0;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        vals[k] = s_data[threadIdx.x * SCAN_IPT + k];
        sum += vals[k];
    }
    int total;
    int run = block_exclusive_scan(sum, s_warp, &total);
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        int v = vals[k];
        s_data[threadIdx.x * SCAN_IPT + k] = inclusive ? run + v : run;
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        int64_t i = base + k * SCAN_THREADS + threadIdx.x;
        if (i < n) out[i] = s_data[k * SCAN_THREADS + threadIdx.x];
    }
    if (tile_sums && threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ __launch_bounds__(SCAN_THREADS) void k_scan_add(int* out, int64_t n, const int* tile_offsets)
{
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    const int add = tile_offsets[blockIdx.x];
    if (add == 0) return;
#pragma unroll
    for (int k = 0; k < SCAN_IPT; ++k) {
        int64_t i = base + k * SCAN_THREADS + threadIdx.x;
        if (i < n) out[i] += add;
    }
}

size_t scan_workspace_bytes(int64_t n)
{
    size_t bytes = 0;
    while (n > SCAN_TILE) {
        n = ceil_div<int64_t>(n, SCAN_TILE);
        bytes += (size_t)n * sizeof(int);
    }
    return bytes + 256;
}

int scan_i32(const int* in, int* out, int64_t n, bool inclusive, void* workspace, cudaStream_t stream)
{
    if (n <= 0) return GB_OK;
    if (n <= SCAN_TILE) {
        k_scan_tiles<<<1, SCAN_THREADS, 0, stream>>>(in, out, n, inclusive ? 1 : 0, nullptr);
        GB_CHECK_CUDA(cudaGetLastError());
        return GB_OK;
    }
    const int64_t ntiles = ceil_div<int64_t>(n, SCAN_TILE);
    int* tile_sums = static_cast<int*>(workspace);
    k_scan_tiles<<<(unsigned)ntiles, SCAN_THREADS, 0, stream>>>(in, out, n, inclusive ? 1 : 0, tile_sums);
    GB_CHECK_CUDA(cudaGetLastError());
    int rc = scan_i32(tile_sums, tile_sums, ntiles, false, tile_sums + ntiles, stream);
    if (rc) return rc;
    k_scan_add<<<(unsigned)ntiles, SCAN_THREADS, 0, stream>>>(out, n, tile_sums);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb

// C ABI: in-place-capable int32 scan.  Replaces wp_array_scan_int_device (warp/native/warp.h:449).
GB_API size_t gb_scan_i32_workspace_bytes(int64_t n) { return gb::scan_workspace_bytes(n); }

GB_API int gb_scan_i32(const int* in, int* out, int64_t n, int inclusive, void* workspace, size_t workspace_bytes,
                       cudaStream_t stream)
{
    GB_REQUIRE(n >= 0, "gb_scan_i32: negative length");
    GB_REQUIRE(n == 0 || (in && out), "gb_scan_i32: null array");
    GB_REQUIRE(workspace_bytes >= gb::scan_workspace_bytes(n) || n <= 4096,
               "gb_scan_i32: workspace too small (%zu < %zu)", workspace_bytes, gb::scan_workspace_bytes(n));
    return gb::scan_i32(in, out, n, inclusive != 0, workspace, stream);
}
