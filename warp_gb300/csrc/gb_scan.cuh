// gb_scan.cuh -- internal prefix-sum interface shared by the warp_gb300 CUDA sources.
#pragma once
#include "gb_common.cuh"

namespace gb {
// elements per tile of the multi-level scan (gb_scan.cu: SCAN_TILE)
constexpr int64_t kScanTileElems = 4096;
size_t scan_workspace_bytes(int64_t n);
int scan_i32(const int* in, int* out, int64_t n, bool inclusive, void* workspace, cudaStream_t stream);
}  // namespace gb
