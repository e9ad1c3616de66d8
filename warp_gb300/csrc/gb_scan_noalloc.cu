// gb_scan_noalloc.cu -- an int32 prefix sum that allocates nothing.
//
// Who needs it: callers that must not allocate device memory at all -- a host application that
// owns every byte of device memory through its own arena and forbids libraries from allocating,
// or code that builds BSR row offsets while a stream is being captured into a CUDA graph, where a
// plain cudaMalloc is not allowed.  gb_scan_i32 asks such callers for a workspace; this variant
// instead keeps its scratch (the per-tile sums of every level of the multi-level scan) in a
// fixed, file-scope device array, so the caller passes only the input and the output.
//
// Limits and behaviour:
//   * n <= GB_SCAN_NOALLOC_MAX_N (2^28 = 268,435,456 elements); larger n is rejected with an
//     error message and nothing is launched.
//   * The array (65,600 ints, about 256 KB) is held by every GPU that loads the library until
//     the process exits.
//   * All calls share that one array.  Each call writes every scratch element it later reads, so
//     nothing has to start at zero and no earlier call's contents leak into a result; but calls
//     whose kernels overlap on the GPU (different streams, no ordering between them) race on the
//     array and may return wrong sums -- order such calls on one stream.
//   * The device address of the array is looked up once per device (cudaGetSymbolAddress with
//     that device current), on the first call made while it is current.  Make that first call
//     outside of any stream capture.
#include "gb_common.cuh"
#include "gb_scan.cuh"

#include <mutex>

namespace gb {

constexpr int64_t kScanNoAllocMaxN = (int64_t)1 << 28;
// level-1 tile sums for 2^28 elements (2^28 / 4096 = 65,536) + level 2 (16) + slack
constexpr size_t kScanNoAllocScratchInts = 65536 + 64;

static __device__ __align__(256) int g_scan_scratch[kScanNoAllocScratchInts];

constexpr int kMaxDevices = 64;
static std::mutex g_scratch_mutex;
static void* g_scratch_addr[kMaxDevices] = {nullptr};

}  // namespace gb

using namespace gb;

GB_API int64_t gb_scan_i32_noalloc_max_n(void) { return kScanNoAllocMaxN; }

// Same result as gb_scan_i32 (in-place allowed), scratch from the fixed device array above.
GB_API int gb_scan_i32_noalloc(const int* in, int* out, int64_t n, int inclusive, cudaStream_t stream)
{
    GB_REQUIRE(n >= 0, "gb_scan_i32_noalloc: negative length");
    if (n > kScanNoAllocMaxN) {
        gb::set_error("gb_scan_i32_noalloc: n = %lld exceeds the fixed scratch of this entry point "
                      "(at most %lld elements); use gb_scan_i32 with a workspace instead",
                      (long long)n, (long long)kScanNoAllocMaxN);
        return GB_ERR_CAPACITY;
    }
    if (n == 0) return GB_OK;
    GB_REQUIRE(in && out, "gb_scan_i32_noalloc: null array");
    if (scan_workspace_bytes(n) > sizeof(g_scan_scratch)) {  // cannot happen for n <= the limit
        gb::set_error("gb_scan_i32_noalloc: scratch too small for n = %lld", (long long)n);
        return GB_ERR_CAPACITY;
    }
    int dev = 0;
    GB_CHECK_CUDA(cudaGetDevice(&dev));
    GB_REQUIRE(dev >= 0 && dev < kMaxDevices, "gb_scan_i32_noalloc: device ordinal %d not supported", dev);
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void* ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_scan_scratch);
            if (e != cudaSuccess) return gb::cuda_fail(e, "cudaGetSymbolAddress(g_scan_scratch)");
            g_scratch_addr[dev] = ptr;
        }
        scratch = g_scratch_addr[dev];
    }
    return scan_i32(in, out, n, inclusive != 0, scratch, stream);
}
