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

}  // namespace gb

GB_API const char* gb_last_error(void) { return gb::g_last_error; }

GB_API void gb_clear_error(void) { gb::g_last_error[0] = 0; }

GB_API int gb_version(void) { return 100; }  // 1.0.0

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
