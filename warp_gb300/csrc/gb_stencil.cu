// gb_stencil.cu -- 27-point stencil form of the multigrid levels' operators.
//
// No reference counterpart: Warp's solvers apply CSR/BSR matrices only.  The multigrid levels of
// the flexible-CG preconditioner are Q1 operators on structured node grids, so every row has at most
// the 27 neighbours (dx, dy, dz) in {-1, 0, 1}^3 of its node.  Storing the coefficients node-major,
//     S[i][k],  k = (dx+1)*9 + (dy+1)*3 + (dz+1),  node i = (x*ny + y)*nz + z
// (n rounded up to a multiple of 4 nodes, so every tile is a multiple of 16 bytes) drops the column
// indices and row offsets of the CSR form: a smoothing or residual pass reads 108 bytes of
// coefficients per row plus the vectors, against 27*8 + 4 for CSR.  Coefficients that the CSR row
// does not hold are stored as zero, so the product is the CSR product (summed in tap order).
// Neighbours outside the grid are skipped.
//
// The apply kernel is persistent: per 256-node tile one thread issues a 1-D bulk copy of the tile's
// 27.6 KB of coefficients into a 2-stage shared-memory ring (one contiguous stream per CTA, as the
// CSR kernel's staging), four CTAs per SM; each thread reads its node's 27 coefficients from shared
// memory (word stride 27, odd: no bank conflicts) and its neighbours' vector entries through the
// read-only path.  Measured at 97^3 (GB300): 22-24 us per pass (~5 TB/s); 3 stages x 2 CTAs per SM
// (16 warps) was latency-bound at 31 us, and a planar S[k][i] layout read with 27 plain loads per
// thread ran 1.5-2x slower than the CSR kernel (27 concurrent streams per warp).
//
// A bf16 copy of S (28 values per node: the 27 taps and one zero, 56 bytes, read as 7 eight-byte words)
// halves the coefficient stream for the fine level of a V-cycle that only has to be an approximate
// inverse; products still accumulate in fp32.
//
// Kernels:
//   gb_st27_to_bf16  S -> bf16 copy (gb_st27_bytes_bf16)
//   gb_st27_build  CSR (1x1 fp32, compact) -> S; an entry outside the 27-neighbourhood sets
//                  status bit 1 (the caller keeps the CSR form then)
//   gb_st27_apply  mode 0: t = r - A w
//                  mode 1: w = omega D^-1 r (written), t = r - A w   (first Jacobi step + residual)
//                  mode 2: z = w + omega D^-1 (r - A w)               (Jacobi step fused with residual)
#include "gb_bulk.cuh"
#include "gb_common.cuh"
#include "gb_spmv.cuh"  // sm_count()
#include "gb_st27.cuh"
#include "gb_df32.cuh"

namespace gb {

__global__ void k_st27_build(St27Grid g, const int* __restrict__ offsets, const int* __restrict__ columns,
                             const float* __restrict__ values, float* __restrict__ S, int* status)
{
    pdl_enter();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += stride) {
        int x, y, z;
        st27_coords(g, i, x, y, z);
        float s[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) s[k] = 0.f;
        bool bad = false;
        for (int e = offsets[i]; e < offsets[i + 1]; ++e) {
            int cx, cy, cz;
            st27_coords(g, columns[e], cx, cy, cz);
            const int dx = cx - x, dy = cy - y, dz = cz - z;
            if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1 || columns[e] < 0 ||
                (int64_t)columns[e] >= g.n) {
                bad = true;
                continue;
            }
            const int k = (dx + 1) * 9 + (dy + 1) * 3 + (dz + 1);
            // a compact row holds each column once; a repeated one would be summed by the CSR product
#pragma unroll
            for (int q = 0; q < 27; ++q)
                if (q == k) s[q] += values[e];
        }
        if (bad) atomicOr(status, 1);
#pragma unroll
        for (int k = 0; k < 27; ++k) S[i * 27 + k] = s[k];
    }
}

template <int MODE, typename CT>
__global__ void __launch_bounds__(ST_TILE) k_st27_apply(St27Grid g, const CT* __restrict__ S, const float* w,
                                                         const float* __restrict__ r, const float* __restrict__ dinv,
                                                         float omega, float* w_out, float* out, int* status)
{
    constexpr int STRIDE = St27Coef<CT>::stride;
    constexpr size_t STAGE = st27_stage_bytes<CT>();
    extern __shared__ __align__(16) unsigned char smem[];
    pdl_enter();
    CT* ring = reinterpret_cast<CT*>(smem);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST_STAGES * STAGE);
    const int64_t ntiles = (g.n + ST_TILE - 1) / ST_TILE;
    const int64_t npad = st27_padded_nodes(g.n);
    // copy of tile `tile` into stage s: its nodes rounded up to 4 (the padded tail of S)
    auto issue = [&](int64_t tile, int s) {
        const int64_t i0 = tile * ST_TILE;
        const int64_t cnt = npad - i0 < ST_TILE ? npad - i0 : ST_TILE;
        const uint32_t bytes = (uint32_t)(cnt * STRIDE * sizeof(CT));
        mbar_arrive_expect_tx(&full[s], bytes);
        bulk_g2s(ring + (size_t)s * ST_TILE * STRIDE, S + i0 * STRIDE, bytes, &full[s]);
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < ST_STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        for (int s = 0; s < ST_STAGES; ++s)
            if (blockIdx.x + (int64_t)s * gridDim.x < ntiles) issue(blockIdx.x + (int64_t)s * gridDim.x, s);
    }
    __syncthreads();
    const int64_t yz = (int64_t)g.ny * g.nz;
    int it = 0;
    int64_t tile = blockIdx.x;
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const int s = it % ST_STAGES;
        // every thread waits (bounded); the CTA leaves together if any wait gave up
        if (!__syncthreads_and(mbar_wait_bounded(&full[s], (uint32_t)(it / ST_STAGES) & 1u))) break;
        const int64_t i = tile * ST_TILE + threadIdx.x;
        if (i < g.n) {
            float c[27];
            st27_load_coefs(ring + (size_t)s * ST_TILE * STRIDE + threadIdx.x * STRIDE, c);
            int x, y, z;
            st27_coords(g, i, x, y, z);
            const bool okx[3] = {x > 0, true, x < g.nx - 1};
            const bool oky[3] = {y > 0, true, y < g.ny - 1};
            const bool okz[3] = {z > 0, true, z < g.nz - 1};
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
                if (okx[dx + 1] && oky[dy + 1] && okz[dz + 1]) {
                    const int64_t j = i + dx * yz + (int64_t)dy * g.nz + dz;
                    // MODE 1: the first Jacobi iterate w = omega D^-1 r, formed on the fly
                    const float wj = MODE == 1 ? omega * __ldg(dinv + j) * __ldg(r + j) : w[j];
                    acc = fmaf(c[k], wj, acc);
                }
            }
            const float ri = r[i];
            if (MODE == 0) {
                out[i] = ri - acc;
            } else if (MODE == 1) {
                w_out[i] = omega * dinv[i] * ri;
                out[i] = ri - acc;
            } else {
                out[i] = w[i] + omega * dinv[i] * (ri - acc);
            }
        }
        __syncthreads();  // stage s is read: refill it
        if (threadIdx.x == 0 && tile + (int64_t)ST_STAGES * gridDim.x < ntiles)
            issue(tile + (int64_t)ST_STAGES * gridDim.x, s);
    }
    if (tile < ntiles) {
        // a wait gave up: drain the copies still in flight (bounded) before shared memory goes away
        if (threadIdx.x == 0) {
            for (int q = 0; q < ST_STAGES; ++q) {
                const int64_t tq = tile + (int64_t)q * gridDim.x;
                if (tq < ntiles) mbar_wait_bounded(&full[(it + q) % ST_STAGES], (uint32_t)((it + q) / ST_STAGES) & 1u);
            }
            atomicOr(status, GB_DEV_WAIT_TIMEOUT);
        }
        __syncthreads();
    }
}

// The refinement's true residual on the stencil form: r = b - A x with x given as (hi, lo) fp32
// pairs and double-float products and sums (the arithmetic of gb_refine.cu's k_resid_df), r32 = the
// residual rounded to fp32 (and r64 in FP64, if asked), norms = ||r||^2, ||b||^2.  Staging as
// k_st27_apply.
__global__ void __launch_bounds__(ST_TILE) k_st27_resid_df(St27Grid g, const float* __restrict__ S,
                                                           const float2* __restrict__ x2, const float* __restrict__ b,
                                                           double* r64, float* r32, double* norms, double* partials,
                                                           unsigned int* counter, int* status)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[64];
    pdl_enter();
    constexpr size_t STAGE = st27_stage_bytes<float>();
    float* ring = reinterpret_cast<float*>(smem);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST_STAGES * STAGE);
    const int64_t ntiles = (g.n + ST_TILE - 1) / ST_TILE;
    const int64_t npad = st27_padded_nodes(g.n);
    auto issue = [&](int64_t tile, int s) {
        const int64_t i0 = tile * ST_TILE;
        const int64_t cnt = npad - i0 < ST_TILE ? npad - i0 : ST_TILE;
        const uint32_t bytes = (uint32_t)(cnt * 27 * sizeof(float));
        mbar_arrive_expect_tx(&full[s], bytes);
        bulk_g2s(ring + (size_t)s * ST_TILE * 27, S + i0 * 27, bytes, &full[s]);
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < ST_STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        for (int s = 0; s < ST_STAGES; ++s)
            if (blockIdx.x + (int64_t)s * gridDim.x < ntiles) issue(blockIdx.x + (int64_t)s * gridDim.x, s);
    }
    __syncthreads();
    const int64_t yz = (int64_t)g.ny * g.nz;
    float rr = 0.f, bb = 0.f;
    int it = 0;
    int64_t tile = blockIdx.x;
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const int s = it % ST_STAGES;
        if (!__syncthreads_and(mbar_wait_bounded(&full[s], (uint32_t)(it / ST_STAGES) & 1u))) break;
        const int64_t i = tile * ST_TILE + threadIdx.x;
        if (i < g.n) {
            float c[27];
            st27_load_coefs(ring + (size_t)s * ST_TILE * 27 + threadIdx.x * 27, c);
            int x, y, z;
            st27_coords(g, i, x, y, z);
            const bool okx[3] = {x > 0, true, x < g.nx - 1};
            const bool oky[3] = {y > 0, true, y < g.ny - 1};
            const bool okz[3] = {z > 0, true, z < g.nz - 1};
            df32 acc;
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
                if (okx[dx + 1] && oky[dy + 1] && okz[dz + 1]) {
                    const float2 xv = __ldg(x2 + i + dx * yz + (int64_t)dy * g.nz + dz);
                    acc += df32(c[k], 0.f) * df32(xv.x, xv.y);
                }
            }
            const float bi = b[i];
            const df32 ri = df32(bi, 0.f) + (-acc);
            const float r = ri.hi + ri.lo;
            if (r64) r64[i] = (double)ri.hi + (double)ri.lo;
            if (r32) r32[i] = r;
            rr += r * r;
            bb += bi * bi;
        }
        __syncthreads();  // stage s is read: refill it
        if (threadIdx.x == 0 && tile + (int64_t)ST_STAGES * gridDim.x < ntiles)
            issue(tile + (int64_t)ST_STAGES * gridDim.x, s);
    }
    if (tile < ntiles) {
        if (threadIdx.x == 0) {
            for (int q = 0; q < ST_STAGES; ++q) {
                const int64_t tq = tile + (int64_t)q * gridDim.x;
                if (tq < ntiles) mbar_wait_bounded(&full[(it + q) % ST_STAGES], (uint32_t)((it + q) / ST_STAGES) & 1u);
            }
            atomicOr(status, GB_DEV_WAIT_TIMEOUT);
        }
        __syncthreads();
    }
    float v[2] = {rr, bb};
    grid_reduce_df<2>(v, partials, counter, s_red, [&](const double (&t)[2]) {
        norms[0] = t[0];
        norms[1] = t[1];
    });
}

// S (fp32, 27 per node) -> Sb (bf16, 28 per node, the 28th zero), round to nearest even
__global__ void k_st27_to_bf16(int64_t npad, const float* __restrict__ S, __nv_bfloat16* __restrict__ Sb)
{
    pdl_enter();
    const int64_t total = npad * ST_BF16_STRIDE;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / ST_BF16_STRIDE;
        const int k = (int)(e - i * ST_BF16_STRIDE);
        Sb[e] = __float2bfloat16_rn(k < 27 ? S[i * 27 + k] : 0.f);
    }
}

static int st27_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 8)); }

template <typename CT> static int st27_apply_grid(int64_t n)
{
    return (int)std::max<int64_t>(
        1, std::min<int64_t>(ceil_div<int64_t>(n, ST_TILE), (int64_t)sm_count() * St27Coef<CT>::ctas_per_sm));
}

template <typename CT>
static int st27_apply_t(int mode, const St27Grid& g, const CT* S, const float* w, const float* r, const float* dinv,
                        float omega, float* w_out, float* out, int* status, cudaStream_t stream)
{
    const int grid = st27_apply_grid<CT>(g.n);
    constexpr size_t smem = st27_smem<CT>();
    static bool attr_set = false;  // one-time per process and coefficient type
    if (!attr_set) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_st27_apply<0, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_st27_apply<1, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_st27_apply<2, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    if (mode == 0) {
        GB_CHECK_CUDA(launch_pdl(k_st27_apply<0, CT>, grid, ST_TILE, smem, stream, g, S, w, r, dinv, omega, w_out, out,
                                 status));
    } else if (mode == 1) {
        GB_CHECK_CUDA(launch_pdl(k_st27_apply<1, CT>, grid, ST_TILE, smem, stream, g, S, w, r, dinv, omega, w_out, out,
                                 status));
    } else if (mode == 2) {
        GB_CHECK_CUDA(launch_pdl(k_st27_apply<2, CT>, grid, ST_TILE, smem, stream, g, S, w, r, dinv, omega, w_out, out,
                                 status));
    } else {
        gb::set_error("st27_apply: mode must be 0, 1 or 2");
        return GB_ERR_INVALID;
    }
    return GB_OK;
}

}  // namespace gb

using namespace gb;

GB_API size_t gb_st27_bytes(int nx, int ny, int nz)
{
    return (size_t)27 * st27_padded_nodes((int64_t)nx * ny * nz) * sizeof(float);
}

// CSR (1x1 fp32, compact rows) on an nx x ny x nz node grid -> node-major coefficients S
// (gb_st27_bytes; 16-byte aligned; the padded tail is not read back into results).
// status bit 1: an entry lies outside the 27-neighbourhood (S is then incomplete).
GB_API int gb_st27_build(int nx, int ny, int nz, const int* offsets, const int* columns, const float* values,
                         float* S, int* status, cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1 && offsets && columns && values && S && status, "st27_build: bad arguments");
    const St27Grid g{nx, ny, nz, (int64_t)nx * ny * nz};
    GB_REQUIRE(g.n < (int64_t(1) << 31), "st27_build: grid too large");
    GB_REQUIRE((uintptr_t)S % 16 == 0, "st27_build: S must be 16-byte aligned");
    GB_CHECK_CUDA(launch_pdl(k_st27_build, st27_grid(g.n), 256, 0, stream, g, offsets, columns, values, S, status));
    return GB_OK;
}

// mode 0: out = r - A w;  mode 1: w_out = omega D^-1 r, out = r - A w_out;  mode 2: out = w + omega D^-1 (r - A w).
// out must not alias w, r or w_out.  status: GB_DEV_WAIT_TIMEOUT if a staging wait gave up.
GB_API int gb_st27_apply(int mode, int nx, int ny, int nz, const float* S, const float* w, const float* r,
                         const float* dinv, float omega, float* w_out, float* out, int* status, cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1 && S && r && out && status, "st27_apply: bad arguments");
    GB_REQUIRE((uintptr_t)S % 16 == 0, "st27_apply: S must be 16-byte aligned");
    GB_REQUIRE(mode == 1 ? (dinv && w_out) : (w != nullptr && (mode == 0 || dinv != nullptr)),
               "st27_apply: missing operand for mode");
    GB_REQUIRE(out != w && out != r && out != w_out, "st27_apply: out must not alias an input");
    const St27Grid g{nx, ny, nz, (int64_t)nx * ny * nz};
    GB_REQUIRE(g.n < (int64_t(1) << 31), "st27_apply: grid too large");
    return st27_apply_t<float>(mode, g, S, w, r, dinv, omega, w_out, out, status, stream);
}

GB_API size_t gb_st27_bytes_bf16(int nx, int ny, int nz)
{
    return (size_t)ST_BF16_STRIDE * st27_padded_nodes((int64_t)nx * ny * nz) * sizeof(__nv_bfloat16);
}

// bf16 copy of the node-major coefficients S (gb_st27_bytes_bf16; 16-byte aligned).
GB_API int gb_st27_to_bf16(int nx, int ny, int nz, const float* S, void* Sb, cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1 && S && Sb, "st27_to_bf16: bad arguments");
    GB_REQUIRE((uintptr_t)Sb % 16 == 0, "st27_to_bf16: Sb must be 16-byte aligned");
    const int64_t npad = st27_padded_nodes((int64_t)nx * ny * nz);
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(npad * ST_BF16_STRIDE, 256),
                                                                 kSmCount * 8));
    GB_CHECK_CUDA(launch_pdl(k_st27_to_bf16, grid, 256, 0, stream, npad, S, static_cast<__nv_bfloat16*>(Sb)));
    return GB_OK;
}

// gb_st27_apply with the bf16 coefficient copy (products accumulate in fp32).
GB_API int gb_st27_apply_bf16(int mode, int nx, int ny, int nz, const void* Sb, const float* w, const float* r,
                              const float* dinv, float omega, float* w_out, float* out, int* status,
                              cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1 && Sb && r && out && status, "st27_apply_bf16: bad arguments");
    GB_REQUIRE((uintptr_t)Sb % 16 == 0, "st27_apply_bf16: Sb must be 16-byte aligned");
    GB_REQUIRE(mode == 1 ? (dinv && w_out) : (w != nullptr && (mode == 0 || dinv != nullptr)),
               "st27_apply_bf16: missing operand for mode");
    GB_REQUIRE(out != w && out != r && out != w_out, "st27_apply_bf16: out must not alias an input");
    const St27Grid g{nx, ny, nz, (int64_t)nx * ny * nz};
    GB_REQUIRE(g.n < (int64_t(1) << 31), "st27_apply_bf16: grid too large");
    return st27_apply_t<__nv_bfloat16>(mode, g, static_cast<const __nv_bfloat16*>(Sb), w, r, dinv, omega, w_out, out,
                                       status, stream);
}

// r = b - A x on the stencil form S (fp32, gb_st27_build) of a 1x1 matrix on an nx x ny x nz node
// grid, x given as interleaved (hi, lo) fp32 pairs, double-float arithmetic: the stencil counterpart of
// gb_residual_df (same outputs; the workspace of gb_residual_f64_workspace_bytes, first 256 bytes the
// arrival counter, zero before the first call and left zero).
GB_API int gb_residual_df_st27(int nx, int ny, int nz, const float* S, const void* x2, const float* b, double* r64,
                               float* r32, double* norms, void* workspace, size_t workspace_bytes, int* status,
                               cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1 && S && x2 && b && norms && workspace && status,
               "residual_df_st27: null argument");
    GB_REQUIRE((uintptr_t)S % 16 == 0, "residual_df_st27: S must be 16-byte aligned");
    const St27Grid g{nx, ny, nz, (int64_t)nx * ny * nz};
    GB_REQUIRE(g.n < (int64_t(1) << 31), "residual_df_st27: grid too large");
    const int grid = st27_apply_grid<float>(g.n);
    GB_REQUIRE(workspace_bytes >= 256 + sizeof(double) * 2 * (size_t)grid, "residual_df_st27: workspace too small");
    static bool attr_set = false;
    if (!attr_set) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_st27_resid_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)st27_smem<float>()));
        attr_set = true;
    }
    unsigned int* counter = static_cast<unsigned int*>(workspace);
    double* partials = reinterpret_cast<double*>(static_cast<unsigned char*>(workspace) + 256);
    GB_CHECK_CUDA(launch_pdl(k_st27_resid_df, grid, ST_TILE, st27_smem<float>(), stream, g, S,
                             static_cast<const float2*>(x2), b, r64, r32, norms, partials, counter, status));
    return GB_OK;
}
