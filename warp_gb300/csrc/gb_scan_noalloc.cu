// gb_scan_noalloc.cu -- an int32 prefix sum that allocates nothing.
//
// Who needs it: callers that cannot allocate device memory at all -- typically a host application
// that owns every byte of device memory through its own arena and does not let libraries call
// cudaMalloc, so it has no way to hand gb_scan_i32 the workspace it asks for.  This variant keeps
// its scratch (the per-tile sums of every level of the multi-level scan) in a fixed, file-scope
// device array instead, so the caller passes only the input and the output.
//
// Limits and behaviour:
//   * n <= gb_scan_i32_noalloc_max_n() (2^28 = 268,435,456 elements); larger n is rejected with an
//     error message and nothing is launched.  Every n up to and including the limit fits.
//   * The array (65,600 ints, about 256 KB) is held by every GPU that loads the library until
//     the process exits.
//   * All calls share that one array.  Each call writes every scratch element it later reads, so
//     nothing has to start at zero and no earlier call's contents leak into a result; but calls
//     whose kernels overlap on the GPU (different streams, no ordering between them) race on the
//     array and may return wrong sums -- order such calls on one stream.
//   * Set-up: the device address of the array is looked up (cudaGetSymbolAddress, with the device
//     current) by the first call made in a CUDA context, and cached per context; a new context on
//     the same device (after cudaDeviceReset, say) gets its own lookup.  That first call should
//     come before any stream capture.
#include "gb_common.cuh"
#include "gb_scan.cuh"

#include <cuda.h>
#include <mutex>

namespace gb {

constexpr int64_t kScanNoAllocMaxN = (int64_t)1 << 28;

// ints of tile sums that scan_i32 writes for n elements (every level above the first)
constexpr int64_t noalloc_scratch_ints(int64_t n)
{
    return n > kScanTileElems ? (n + kScanTileElems - 1) / kScanTileElems +
                                    noalloc_scratch_ints((n + kScanTileElems - 1) / kScanTileElems)
                              : 0;
}

// 65,536 + 16 for 2^28 elements, rounded up
constexpr size_t kScanNoAllocScratchInts = 65536 + 64;
static_assert(noalloc_scratch_ints(kScanNoAllocMaxN) <= (int64_t)kScanNoAllocScratchInts,
              "scratch array smaller than the documented limit needs");

static __device__ __align__(256) int g_scan_scratch[kScanNoAllocScratchInts];

// Per-context cache of the array's device address, keyed by the driver's unique context id.
typedef CUresult (*PFN_ctxGetCurrent)(CUcontext*);
typedef CUresult (*PFN_ctxGetId)(CUcontext, unsigned long long*);
constexpr int kMaxCached = 64;
static std::mutex g_scratch_mutex;
static bool g_driver_fns_looked_up = false;
static PFN_ctxGetCurrent g_ctx_get_current = nullptr;
static PFN_ctxGetId g_ctx_get_id = nullptr;
static unsigned long long g_cached_ctx[kMaxCached];
static void* g_cached_addr[kMaxCached];
static int g_ncached = 0;

// Returns the device address of g_scan_scratch in the current context, or a status.
static int scratch_address(void** out)
{
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_driver_fns_looked_up) {
        g_driver_fns_looked_up = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = (PFN_ctxGetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = (PFN_ctxGetId)f;
        cudaGetLastError();
    }
    auto current_id = [](unsigned long long* id) {
        CUcontext ctx = nullptr;
        return g_ctx_get_current && g_ctx_get_id && g_ctx_get_current(&ctx) == CUDA_SUCCESS && ctx &&
               g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
    };
    unsigned long long id = 0;
    if (current_id(&id))
        for (int i = 0; i < g_ncached; ++i)
            if (g_cached_ctx[i] == id) {
                *out = g_cached_addr[i];
                return GB_OK;
            }
    // first call in this context (the lookup also makes the runtime's primary context current)
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_scan_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_scan_scratch)");
    if (current_id(&id)) {  // without a context id every call looks the address up again
        int slot = g_ncached < kMaxCached ? g_ncached++ : (int)(id % kMaxCached);
        g_cached_ctx[slot] = id;
        g_cached_addr[slot] = ptr;
    }
    *out = ptr;
    return GB_OK;
}

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
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    return scan_i32(in, out, n, inclusive != 0, scratch, stream);
}
