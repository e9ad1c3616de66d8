// gb_scan.cuh -- internal prefix-sum interface shared by the warp_gb300 CUDA sources.
#pragma once
#include "gb_common.cuh"

namespace gb {
size_t scan_workspace_bytes(int64_t n);
int scan_i32(const int* in, int* out, int64_t n, bool inclusive, void* workspace, cudaStream_t stream);
}  // namespace gb
