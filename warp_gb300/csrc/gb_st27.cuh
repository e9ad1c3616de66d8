// gb_st27.cuh -- the node-major 27-point stencil layout shared by the multigrid stencil kernels
// (gb_stencil.cu) and the flexible solver's stencil product (gb_krylov.cu).
//
//     S[i][k],  k = (dx+1)*9 + (dy+1)*3 + (dz+1),  node i = (x*ny + y)*nz + z
//
// fp32: 27 coefficients per node; bf16 copy: 28 per node (the 27 taps and one zero, 56 bytes).  Node
// counts are padded to a multiple of 4 so that every tile copy is a multiple of 16 bytes.
#pragma once
#include "gb_common.cuh"

namespace gb {

struct St27Grid {
    int nx, ny, nz;
    int64_t n;
};

// node -> (x, y, z); node counts are below 2^31 (checked on the host), so 32-bit division suffices
__device__ __forceinline__ void st27_coords(const St27Grid& g, int64_t i, int& x, int& y, int& z)
{
    const uint32_t ui = (uint32_t)i, yz = (uint32_t)g.ny * (uint32_t)g.nz;
    const uint32_t ux = ui / yz, rem = ui - ux * yz;
    const uint32_t uy = rem / (uint32_t)g.nz;
    x = (int)ux;
    y = (int)uy;
    z = (int)(rem - uy * (uint32_t)g.nz);
}

constexpr int ST_TILE = 256;    // nodes per tile = threads per CTA
constexpr int ST_STAGES = 2;     // 2 stages x 27.6 KB (fp32) / 14.3 KB (bf16)
constexpr int ST_BF16_STRIDE = 28;  // bf16 coefficients per node (27 taps + 1 zero)

template <typename CT> struct St27Coef;
template <> struct St27Coef<float> {
    static constexpr int stride = 27;
    static constexpr int ctas_per_sm = 4;  // 2 x 27.6 KB each: 32 warps per SM
};
template <> struct St27Coef<__nv_bfloat16> {
    static constexpr int stride = ST_BF16_STRIDE;
    static constexpr int ctas_per_sm = 6;  // 2 x 14.3 KB each: 48 warps per SM
};
template <typename CT> __host__ __device__ constexpr size_t st27_stage_bytes() { return (size_t)ST_TILE * St27Coef<CT>::stride * sizeof(CT); }
template <typename CT> __host__ __device__ constexpr size_t st27_smem() { return ST_STAGES * st27_stage_bytes<CT>() + 64; }

__host__ __device__ inline int64_t st27_padded_nodes(int64_t n) { return (n + 3) / 4 * 4; }

// the 27 coefficients of this thread's node from the staged tile
__device__ __forceinline__ void st27_load_coefs(const float* c, float (&v)[27])
{
#pragma unroll
    for (int k = 0; k < 27; ++k) v[k] = c[k];
}

__device__ __forceinline__ void st27_load_coefs(const __nv_bfloat16* c, float (&v)[27])
{
    const uint2* w = reinterpret_cast<const uint2*>(c);  // 56 bytes per node: 7 aligned 8-byte words
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        const uint2 u = w[q];
        const uint32_t h[2] = {u.x, u.y};
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int k0 = q * 4 + e * 2;
            if (k0 < 27) v[k0] = __uint_as_float(h[e] << 16);
            if (k0 + 1 < 27) v[k0 + 1] = __uint_as_float(h[e] & 0xFFFF0000u);
        }
    }
}

}  // namespace gb
