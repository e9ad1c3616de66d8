// gb_capi.cu -- error reporting and library information for the warp_gb300 C ABI.
#include "gb_common.cuh"

#include <stdarg.h>
#include <string.h>

namespace gb {

static thread_local char g_last_error[1024] = {0};

void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t err, const char* what)
{
    set_error("%s failed: %s (%s)", what, cudaGetErrorName(err), cudaGetErrorString(err));
    return GB_ERR_CUDA;
}

static int g_pdl = 1;  // 0 off, 1 eager launches only, 2 eager launches and stream captures

bool pdl_enabled(bool capturing) { return capturing ? g_pdl >= 2 : g_pdl >= 1; }

}  // namespace gb

GB_API const char* gb_last_error(void) { return gb::g_last_error; }

GB_API void gb_clear_error(void) { gb::g_last_error[0] = 0; }

GB_API int gb_version(void) { return 100; }  // 1.0.0

// Programmatic dependent launch of the solver-loop kernels (multigrid transfers and smoothing,
// SpMV, Krylov updates, conv-net layers).  Mode 0: every launch uses plain stream ordering.
// Mode 1 (default): eager launches carry the programmatic-serialization attribute, launches into a
// capturing stream stay plain.  Mode 2: both eager launches and launches into a capturing stream
// carry it.  Takes effect for launches made after the call; results are identical in every mode.
GB_API int gb_set_pdl(int mode)
{
    GB_REQUIRE(mode >= 0 && mode <= 2, "set_pdl: mode must be 0, 1 or 2");
    gb::g_pdl = mode;
    return GB_OK;
}

GB_API int gb_get_pdl(void) { return gb::g_pdl; }

// Returns the compute capability (major*10+minor) of the current device, or a negative status.
GB_API int gb_device_arch(void)
{
    int dev = 0;
    GB_CHECK_CUDA(cudaGetDevice(&dev));
    int major = 0, minor = 0;
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    return major * 10 + minor;
}
