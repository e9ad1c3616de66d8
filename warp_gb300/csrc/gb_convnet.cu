// gb_convnet.cu -- the learned smoother: a 4-layer 3x3x3 convolutional network on the Q1 node grid.
//
// No reference counterpart (Warp's preconditioners are Jacobi only).  Layout: activations are
// channels-last over the node grid, act[v][C] with v = (x * ny + y) * nz + z and C = 16; taps
// t = (dx+1)*9 + (dy+1)*3 + (dz+1) for dx, dy, dz in {-1, 0, 1}; neighbours outside the grid read
// as zero; weights W[t][ci][co]:
//     out[v][co] = sum_t sum_ci W[t][ci][co] * in[v + off(t)][ci]        (no bias: the network is
// positively homogeneous, N(c x) = c N(x) for c > 0, so no residual normalisation is needed).
//
// Training (fp32, CUDA cores): k_conv_fwd_f32, k_conv_bwd_data_f32 (gradient w.r.t. the input =
// correlation with the flipped, transposed kernel), k_conv_bwd_weight_f32 (per-CTA partial sums
// reduced in a fixed order: deterministic), ReLU backward and Adam.  Inference runs on the tcgen05
// tensor cores (gb_conv_tc.cu).
#include "gb_common.cuh"
#include "gb_net_features.cuh"

namespace gb {

constexpr int CN = 16;  // channels of the hidden layers (and of the padded input)

struct Grid3 {
    int nx, ny, nz;
};

__device__ __forceinline__ bool tap_neighbor(const Grid3& g, int x, int y, int z, int t, int64_t& nb)
{
    const int dx = t / 9 - 1, dy = (t / 3) % 3 - 1, dz = t % 3 - 1;
    const int xx = x + dx, yy = y + dy, zz = z + dz;
    if (xx < 0 || yy < 0 || zz < 0 || xx >= g.nx || yy >= g.ny || zz >= g.nz) return false;
    nb = ((int64_t)xx * g.ny + yy) * g.nz + zz;
    return true;
}

__device__ __forceinline__ void decode(const Grid3& g, int64_t v, int& x, int& y, int& z)
{
    x = (int)(v / ((int64_t)g.ny * g.nz));
    y = (int)((v / g.nz) % g.ny);
    z = (int)(v % g.nz);
}

// ---------------------------------------------------------------------------------------------
// fp32 training kernels
// ---------------------------------------------------------------------------------------------
// out[v][co] = sum W * in ; cin, cout <= 16; relu: out = max(out, 0)
__global__ __launch_bounds__(256) void k_conv_fwd_f32(Grid3 g, int cin, int cout, const float* __restrict__ in,
                                                      const float* __restrict__ W, int relu, float* __restrict__ out)
{
    __shared__ float s_w[27 * CN * CN];
    for (int i = threadIdx.x; i < 27 * cin * cout; i += blockDim.x) s_w[i] = W[i];
    __syncthreads();
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    int x, y, z;
    decode(g, v, x, y, z);
    float acc[CN];
#pragma unroll
    for (int c = 0; c < CN; ++c) acc[c] = 0.f;
    for (int t = 0; t < 27; ++t) {
        int64_t nb;
        if (!tap_neighbor(g, x, y, z, t, nb)) continue;
        const float* src = in + nb * cin;
        for (int ci = 0; ci < cin; ++ci) {
            const float a = src[ci];
            const float* w = s_w + (t * cin + ci) * cout;
#pragma unroll
            for (int co = 0; co < CN; ++co)
                if (co < cout) acc[co] += a * w[co];
        }
    }
#pragma unroll
    for (int co = 0; co < CN; ++co)
        if (co < cout) out[v * cout + co] = relu ? fmaxf(acc[co], 0.f) : acc[co];
}

// gin[v][ci] = sum_t sum_co W[t][ci][co] * gout[v - off(t)][co]
__global__ __launch_bounds__(256) void k_conv_bwd_data_f32(Grid3 g, int cin, int cout, const float* __restrict__ gout,
                                                           const float* __restrict__ W, float* __restrict__ gin)
{
    __shared__ float s_w[27 * CN * CN];
    for (int i = threadIdx.x; i < 27 * cin * cout; i += blockDim.x) s_w[i] = W[i];
    __syncthreads();
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    int x, y, z;
    decode(g, v, x, y, z);
    float acc[CN];
#pragma unroll
    for (int c = 0; c < CN; ++c) acc[c] = 0.f;
    for (int t = 0; t < 27; ++t) {
        int64_t nb;
        if (!tap_neighbor(g, x, y, z, 26 - t, nb)) continue;  // v - off(t) = v + off(26 - t)
        const float* src = gout + nb * cout;
        for (int co = 0; co < cout; ++co) {
            const float gv = src[co];
#pragma unroll
            for (int ci = 0; ci < CN; ++ci)
                if (ci < cin) acc[ci] += gv * s_w[(t * cin + ci) * cout + co];
        }
    }
#pragma unroll
    for (int ci = 0; ci < CN; ++ci)
        if (ci < cin) gin[v * cin + ci] = acc[ci];
}

// partial[cta][t][ci][co] = sum over the CTA's voxels v of in[v + off(t)][ci] * gout[v][co].
// Persistent CTAs walk tiles of WG_VOX voxels; thread (ci, co) keeps the 27 tap sums in registers; the
// tile's neighbour table and output gradients are staged in shared memory.
constexpr int WG_VOX = 64;
constexpr int WG_CTAS = 2 * kSmCount;
__global__ __launch_bounds__(256) void k_conv_bwd_weight_f32(Grid3 g, int cin, int cout, const float* __restrict__ in,
                                                             const float* __restrict__ gout,
                                                             float* __restrict__ partial)
{
    __shared__ float s_g[WG_VOX * CN];
    __shared__ int64_t s_nb[WG_VOX * 27];
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t ntiles = ceil_div<int64_t>(n, WG_VOX);
    const int ci = threadIdx.x / cout, co = threadIdx.x % cout;
    const bool active = threadIdx.x < cin * cout;
    float acc[27];
#pragma unroll
    for (int t = 0; t < 27; ++t) acc[t] = 0.f;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t v0 = tile * WG_VOX;
        __syncthreads();
        for (int i = threadIdx.x; i < WG_VOX * cout; i += blockDim.x) {
            const int64_t v = v0 + i / cout;
            s_g[i] = (v < n) ? gout[v * cout + (i % cout)] : 0.f;
        }
        for (int i = threadIdx.x; i < WG_VOX * 27; i += blockDim.x) {
            const int64_t v = v0 + i / 27;
            int64_t nb = -1;
            if (v < n) {
                int x, y, z;
                decode(g, v, x, y, z);
                if (!tap_neighbor(g, x, y, z, i % 27, nb)) nb = -1;
            }
            s_nb[i] = nb;
        }
        __syncthreads();
        if (!active) continue;
        for (int j = 0; j < WG_VOX; ++j) {
            const float gv = s_g[j * cout + co];
#pragma unroll
            for (int t = 0; t < 27; ++t) {
                const int64_t nb = s_nb[j * 27 + t];
                if (nb >= 0) acc[t] += __ldg(in + nb * cin + ci) * gv;
            }
        }
    }
    if (active) {
        const int nw = 27 * cin * cout;
#pragma unroll
        for (int t = 0; t < 27; ++t) partial[(int64_t)blockIdx.x * nw + (t * cin + ci) * cout + co] = acc[t];
    }
}

// gW[k] += sum_cta partial[cta][k]  (fixed order)
__global__ void k_reduce_partials(int nparts, int nw, const float* __restrict__ partial, float* __restrict__ gW)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nw) return;
    float s = 0.f;
    for (int p = 0; p < nparts; ++p) s += partial[(int64_t)p * nw + k];
    gW[k] += s;
}

// g *= (out > 0)
__global__ void k_relu_bwd(int64_t n, const float* __restrict__ out, float* __restrict__ g)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (out[i] <= 0.f) g[i] = 0.f;
}

// Adam (Kingma & Ba): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2; w -= lr mhat / (sqrt(vhat) + eps);
// also writes the bf16 copy used by the tensor-core forward.
__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ wb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
}

// Input features: ch0 = x = dinv * r; ch1..8 = x * chat[v][k] (normalised log-coefficient of the
// k-th adjacent cell, 0 outside the grid); ch9..15 = 0; masked (Dirichlet) nodes are all zero.
// fp32 (training) or bf16 (inference) output.
// fp32 (training) or bf16 (inference) output, channels-last [n][16].
template <typename OT>
__global__ void k_features(int ncomp, int64_t n, const float* __restrict__ r, const float* __restrict__ dinv,
                           const float* __restrict__ chat, const float* __restrict__ mask, OT* __restrict__ out)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        float f[CN];
        net_node_features(ncomp, v, r, dinv, chat, mask, f);
        if constexpr (sizeof(OT) == 2) {
            __nv_bfloat162* o = reinterpret_cast<__nv_bfloat162*>(out + v * CN);
#pragma unroll
            for (int k = 0; k < CN / 2; ++k) o[k] = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
        } else {
#pragma unroll
            for (int k = 0; k < CN; ++k) out[v * CN + k] = f[k];
        }
    }
}

// per-node normalised log-coefficients of the 8 adjacent cells (set-up)
__global__ void k_cell_features(Grid3 g, const float* __restrict__ cell_coef, float mean_log, float inv_std,
                                float* __restrict__ chat)
{
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    int x, y, z;
    decode(g, v, x, y, z);
    const int cx = g.nx - 1, cy = g.ny - 1, cz = g.nz - 1;
    for (int k = 0; k < 8; ++k) {
        const int ax = x - 1 + (k >> 2), ay = y - 1 + ((k >> 1) & 1), az = z - 1 + (k & 1);
        float val = 0.f;
        if (ax >= 0 && ay >= 0 && az >= 0 && ax < cx && ay < cy && az < cz)
            val = (logf(cell_coef[((int64_t)ax * cy + ay) * cz + az]) - mean_log) * inv_std;
        chat[v * 8 + k] = val;
    }
}

// out[i] = omega * dinv[i] * r[i] + (mask[node] ? 0 : act[node][c]) for dof i = node * ncomp + c: the Jacobi
// step plus the network's output channel c (dinv may be null: network only).
template <typename T>
__global__ void k_net_combine(int ncomp, int64_t n, int stride, const T* __restrict__ act,
                              const float* __restrict__ mask, float omega, const float* __restrict__ dinv,
                              const float* __restrict__ r, float* __restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = i / ncomp;
        const int c = (int)(i - v * ncomp);
        float a;
        if constexpr (sizeof(T) == 2) a = __bfloat162float(act[v * stride + c]); else a = act[v * stride + c];
        if (mask && mask[v] != 0.f) a = 0.f;
        if (dinv) a += omega * dinv[i] * r[i];
        out[i] = a;
    }
}

static int g1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 16)); }

}  // namespace gb

using namespace gb;

GB_API int gb_conv3_fwd_f32(int nx, int ny, int nz, int cin, int cout, const float* in, const float* W, int relu,
                            float* out, cudaStream_t stream)
{
    GB_REQUIRE(cin >= 1 && cin <= CN && cout >= 1 && cout <= CN, "conv3_fwd_f32: channels must be 1..16");
    Grid3 g{nx, ny, nz};
    const int64_t n = (int64_t)nx * ny * nz;
    k_conv_fwd_f32<<<(int)ceil_div<int64_t>(n, 256), 256, 0, stream>>>(g, cin, cout, in, W, relu, out);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_conv3_bwd_data_f32(int nx, int ny, int nz, int cin, int cout, const float* gout, const float* W,
                                 float* gin, cudaStream_t stream)
{
    GB_REQUIRE(cin >= 1 && cin <= CN && cout >= 1 && cout <= CN, "conv3_bwd_data: channels must be 1..16");
    Grid3 g{nx, ny, nz};
    const int64_t n = (int64_t)nx * ny * nz;
    k_conv_bwd_data_f32<<<(int)ceil_div<int64_t>(n, 256), 256, 0, stream>>>(g, cin, cout, gout, W, gin);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

static int bwd_weight_ctas(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, WG_VOX), WG_CTAS)); }

GB_API size_t gb_conv3_bwd_weight_workspace_bytes(int nx, int ny, int nz, int cin, int cout)
{
    const int64_t n = (int64_t)nx * ny * nz;
    return sizeof(float) * (size_t)bwd_weight_ctas(n) * 27 * cin * cout;
}

// gW += dL/dW (accumulates, so several samples can be summed before an optimiser step)
GB_API int gb_conv3_bwd_weight_f32(int nx, int ny, int nz, int cin, int cout, const float* in, const float* gout,
                                   float* gW, void* workspace, size_t workspace_bytes, cudaStream_t stream)
{
    GB_REQUIRE(cin >= 1 && cin <= CN && cout >= 1 && cout <= CN, "conv3_bwd_weight: channels must be 1..16");
    GB_REQUIRE(workspace_bytes >= gb_conv3_bwd_weight_workspace_bytes(nx, ny, nz, cin, cout),
               "conv3_bwd_weight: workspace too small");
    Grid3 g{nx, ny, nz};
    const int64_t n = (int64_t)nx * ny * nz;
    const int parts = bwd_weight_ctas(n);
    float* partial = static_cast<float*>(workspace);
    k_conv_bwd_weight_f32<<<parts, 256, 0, stream>>>(g, cin, cout, in, gout, partial);
    const int nw = 27 * cin * cout;
    k_reduce_partials<<<ceil_div(nw, 256), 256, 0, stream>>>(parts, nw, partial, gW);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_relu_bwd(int64_t n, const float* out, float* g, cudaStream_t stream)
{
    if (n <= 0) return GB_OK;
    k_relu_bwd<<<g1(n), 256, 0, stream>>>(n, out, g);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_adam_step(int n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                        int step, void* w_bf16, cudaStream_t stream)
{
    GB_REQUIRE(n > 0 && step >= 1, "adam: bad arguments");
    const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    k_adam<<<ceil_div(n, 256), 256, 0, stream>>>(n, w, g, m, v, lr, b1, b2, eps, c1, c2,
                                                 static_cast<__nv_bfloat16*>(w_bf16));
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// features: dtype GB_F32 -> fp32 [n][16], GB_BF16 -> bf16 [n][16]; n nodes of ncomp components
GB_API int gb_net_features(int dtype, int ncomp, int64_t n, const float* r, const float* dinv, const float* chat,
                           const float* mask, void* out, cudaStream_t stream)
{
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "net_features: ncomp must be 1 or 3");
    if (n <= 0) return GB_OK;
    if (dtype == GB_F32)
        k_features<float><<<g1(n), 256, 0, stream>>>(ncomp, n, r, dinv, chat, mask, static_cast<float*>(out));
    else if (dtype == GB_BF16)
        k_features<__nv_bfloat16><<<g1(n), 256, 0, stream>>>(ncomp, n, r, dinv, chat, mask,
                                                             static_cast<__nv_bfloat16*>(out));
    else {
        gb::set_error("net_features: dtype must be f32 or bf16");
        return GB_ERR_UNSUPPORTED;
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_net_cell_features(int nx, int ny, int nz, const float* cell_coef, float mean_log, float inv_std,
                                float* chat, cudaStream_t stream)
{
    Grid3 g{nx, ny, nz};
    const int64_t n = (int64_t)nx * ny * nz;
    k_cell_features<<<(int)ceil_div<int64_t>(n, 256), 256, 0, stream>>>(g, cell_coef, mean_log, inv_std, chat);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_net_combine(int dtype, int ncomp, int64_t n, int stride, const void* act, const float* mask, float omega,
                          const float* dinv, const float* r, float* out, cudaStream_t stream)
{
    GB_REQUIRE(ncomp >= 1 && ncomp <= stride, "net_combine: 1 <= ncomp <= stride");
    if (n <= 0) return GB_OK;
    const int64_t nd = n * ncomp;
    if (dtype == GB_F32)
        k_net_combine<float><<<g1(nd), 256, 0, stream>>>(ncomp, nd, stride, static_cast<const float*>(act), mask, omega,
                                                         dinv, r, out);
    else
        k_net_combine<__nv_bfloat16><<<g1(nd), 256, 0, stream>>>(ncomp, nd, stride,
                                                                 static_cast<const __nv_bfloat16*>(act), mask, omega,
                                                                 dinv, r, out);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
