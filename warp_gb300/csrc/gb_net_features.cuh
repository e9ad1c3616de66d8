// gb_net_features.cuh -- input channels of the learned smoother (shared by the fp32 training kernels
// and the planar bf16 inference layout).
#pragma once
#include "gb_common.cuh"

namespace gb {

// The 16 input channels of node v.  ncomp = 1 (scalar field): ch0 = x = dinv * r, ch1..8 = x * chat[v][k]
// (normalised log-coefficient of the k-th adjacent cell, 0 outside the grid), ch9..15 = 0.
// ncomp = 3 (vec3 field, 3 interleaved components per node): ch0..2 = x_c = dinv_c * r_c, ch3 + 4c + j =
// x_c * s_j with s_0 the mean of the 8 cell values and s_1..3 their x / y / z contrasts (mean over the
// cells on the + side minus the - side), ch15 = 0.  Masked (Dirichlet) nodes are all zero.
__device__ __forceinline__ void net_node_features(int ncomp, int64_t v, const float* __restrict__ r,
                                              const float* __restrict__ dinv, const float* __restrict__ chat,
                                              const float* __restrict__ mask, float (&f)[16])
{
    const bool masked = mask && mask[v] != 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) f[k] = 0.f;
    if (ncomp == 1) {
        const float xm = masked ? 0.f : dinv[v] * r[v];
        f[0] = xm;
#pragma unroll
        for (int k = 0; k < 8; ++k) f[1 + k] = xm * chat[v * 8 + k];
        return;
    }
    float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float c = chat[v * 8 + k];
        s[0] += c;
        s[1] += (k >> 2) ? c : -c;
        s[2] += ((k >> 1) & 1) ? c : -c;
        s[3] += (k & 1) ? c : -c;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) s[j] *= 0.125f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float xc = masked ? 0.f : dinv[v * 3 + c] * r[v * 3 + c];
        f[c] = xc;
#pragma unroll
        for (int j = 0; j < 4; ++j) f[3 + 4 * c + j] = xc * s[j];
    }
}

}  // namespace gb
