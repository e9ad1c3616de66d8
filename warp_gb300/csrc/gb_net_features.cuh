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
// The values node v's channels are made of, loaded without conditions (a caller may load several nodes
// before using any).
struct NetNodeIn {
    float m;        // mask value (0: free)
    float x[3];     // dinv * r per component (component 0 only for ncomp = 1)
    float ch[8];    // chat[v][0..7]
};

__device__ __forceinline__ void net_node_load(int ncomp, int64_t v, const float* __restrict__ r,
                                              const float* __restrict__ dinv, const float* __restrict__ chat,
                                              const float* __restrict__ mask, NetNodeIn& in)
{
    in.m = mask ? mask[v] : 0.f;
    if (ncomp == 1) {
        in.x[0] = dinv[v] * r[v];
        in.x[1] = in.x[2] = 0.f;
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) in.x[c] = dinv[v * 3 + c] * r[v * 3 + c];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) in.ch[k] = chat[v * 8 + k];
}

__device__ __forceinline__ void net_node_compute(int ncomp, const NetNodeIn& in, float (&f)[16])
{
    const bool masked = in.m != 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) f[k] = 0.f;
    if (ncomp == 1) {
        const float xm = masked ? 0.f : in.x[0];
        f[0] = xm;
#pragma unroll
        for (int k = 0; k < 8; ++k) f[1 + k] = xm * in.ch[k];
        return;
    }
    float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float c = in.ch[k];
        s[0] += c;
        s[1] += (k >> 2) ? c : -c;
        s[2] += ((k >> 1) & 1) ? c : -c;
        s[3] += (k & 1) ? c : -c;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) s[j] *= 0.125f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float xc = masked ? 0.f : in.x[c];
        f[c] = xc;
#pragma unroll
        for (int j = 0; j < 4; ++j) f[3 + 4 * c + j] = xc * s[j];
    }
}

__device__ __forceinline__ void net_node_features(int ncomp, int64_t v, const float* __restrict__ r,
                                              const float* __restrict__ dinv, const float* __restrict__ chat,
                                              const float* __restrict__ mask, float (&f)[16])
{
    NetNodeIn in;
    net_node_load(ncomp, v, r, dinv, chat, mask, in);
    net_node_compute(ncomp, in, f);
}

}  // namespace gb
