// gb_mg.cu -- geometric multigrid pieces for the flexible-CG preconditioner on Q1 grids.
//
// No reference counterpart: Warp's solvers offer only the Jacobi preconditioner
// (warp/_src/optim/linear.py:236-329).  These kernels build the hierarchy that carries the
// learned preconditioner: vertex-centred 2:1 coarsening of Q1 node grids (fine node 2I is coarse
// node I), trilinear prolongation P and its transpose R = P^T (full weighting), damped Jacobi
// steps, and the per-cell coefficient coarsening used to rediscretise the coarse operators
// (for a coefficient constant on coarse cells the rediscretised Q1 operator equals the Galerkin
// product P^T A P, since coarse Q1 functions are fine Q1 functions).  Dirichlet nodes are masked:
// their restricted residuals are zeroed and prolongation never writes them.
#include "gb_common.cuh"

namespace gb {

struct NodeGrid {
    int nx, ny, nz;  // nodes per axis (cells + 1)
};

__device__ __forceinline__ int64_t nidx(const NodeGrid& g, int x, int y, int z)
{
    return ((int64_t)x * g.ny + y) * g.nz + z;
}

// rc[I] = mask_c[I] * sum_{d in {-1,0,1}^3} w(d) r[2I + d],  w = prod (1 if d=0 else 1/2); fine
// nodes outside the grid or masked (Dirichlet) contribute nothing.  Branch-free: every tap loads from
// a clamped in-grid index and adds a zero when it does not count, so all 54 loads can be in flight
// at once (the sum over the counted taps, in tap order, is unchanged).
// Vectors hold C interleaved components per node (value of component c at node i: [i*C + c]); the
// masks are per node.
template <int C>
__global__ void k_restrict_fw(NodeGrid fg, NodeGrid cg, const float* __restrict__ r, const float* __restrict__ fmask,
                              const float* __restrict__ cmask, float* __restrict__ rc)
{
    pdl_enter();
    // 3-D launch (tgrid3): no index division
    const int Z = (int)(blockIdx.x * blockDim.x + threadIdx.x), Y = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int X = (int)blockIdx.z;
    if (Z >= cg.nz || Y >= cg.ny) return;
    const int64_t I = nidx(cg, X, Y, Z);
    const bool cmasked = cmask && __ldg(cmask + I) != 0.f;
    float s[C];
#pragma unroll
    for (int c = 0; c < C; ++c) s[c] = 0.f;
#pragma unroll
    for (int dx = -1; dx <= 1; ++dx) {
        const int x = 2 * X + dx;
        const bool vx = x >= 0 && x < fg.nx;
        const int xc = min(max(x, 0), fg.nx - 1);
        const float wx = dx == 0 ? 1.f : 0.5f;
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = 2 * Y + dy;
            const bool vy = y >= 0 && y < fg.ny;
            const int yc = min(max(y, 0), fg.ny - 1);
            const float wy = dy == 0 ? 1.f : 0.5f;
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz) {
                const int z = 2 * Z + dz;
                const bool vz = z >= 0 && z < fg.nz;
                const int zc = min(max(z, 0), fg.nz - 1);
                const int64_t i = nidx(fg, xc, yc, zc);
                const bool keep = vx && vy && vz && !(fmask && __ldg(fmask + i) != 0.f);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const float rv = __ldg(r + i * C + c);
                    s[c] += keep ? wx * wy * (dz == 0 ? 1.f : 0.5f) * rv : 0.f;
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c) rc[I * C + c] = cmasked ? 0.f : s[c];
}

// z[i] += scale * sum_parents w * zc[parent]   (trilinear interpolation; masked fine nodes kept).
// Branch-free as the restriction: the 8 candidate parents are loaded from clamped indices and only
// the real ones (1, 2, 4 or 8 of them, in the same order) are summed.
template <int C>
__global__ void k_prolong_add(NodeGrid fg, NodeGrid cg, const float* __restrict__ zc, const float* __restrict__ fmask,
                              float scale, float* __restrict__ z)
{
    pdl_enter();
    // 3-D launch (tgrid3): no index division
    const int zz = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int x = (int)blockIdx.z;
    if (zz >= fg.nz || y >= fg.ny) return;
    const int64_t i = nidx(fg, x, y, zz);
    const bool masked = fmask && __ldg(fmask + i) != 0.f;
    const int xs[2] = {x >> 1, min((x + 1) >> 1, cg.nx - 1)};
    const int ys[2] = {y >> 1, min((y + 1) >> 1, cg.ny - 1)};
    const int zs[2] = {zz >> 1, min((zz + 1) >> 1, cg.nz - 1)};
    const float wx = (x & 1) ? 0.5f : 1.f, wy = (y & 1) ? 0.5f : 1.f, wz = (zz & 1) ? 0.5f : 1.f;
    const int nxp = (x & 1) ? 2 : 1, nyp = (y & 1) ? 2 : 1, nzp = (zz & 1) ? 2 : 1;
    float s[C];
#pragma unroll
    for (int q = 0; q < C; ++q) s[q] = 0.f;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const int64_t j = nidx(cg, xs[a], ys[b], zs[c]);
                const bool real = a < nxp && b < nyp && c < nzp;
#pragma unroll
                for (int q = 0; q < C; ++q) {
                    const float v = __ldg(zc + j * C + q);
                    s[q] += real ? v : 0.f;
                }
            }
    if (!masked) {
#pragma unroll
        for (int q = 0; q < C; ++q) z[i * C + q] += scale * wx * wy * wz * s[q];
    }
}

// z = omega * dinv * r   (first damped Jacobi step from z = 0)
__global__ void k_jacobi0(int64_t n, float omega, const float* __restrict__ dinv, const float* __restrict__ r,
                          float* __restrict__ z)
{
    pdl_enter();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = omega * dinv[i] * r[i];
}

// z_i = omega * Dinv_i r_i per node (3x3 blocks, 9 floats per node): the first block-Jacobi step
__global__ void k_block_jacobi0(int64_t nodes, float omega, const float* __restrict__ dinv, const float* __restrict__ r,
                                float* __restrict__ z)
{
    pdl_enter();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nodes; i += (int64_t)gridDim.x * blockDim.x) {
        const float* d = dinv + i * 9;
        const float r0 = r[3 * i], r1 = r[3 * i + 1], r2 = r[3 * i + 2];
#pragma unroll
        for (int c = 0; c < 3; ++c) z[3 * i + c] = omega * (d[3 * c] * r0 + d[3 * c + 1] * r1 + d[3 * c + 2] * r2);
    }
}

// cell coefficient of coarse cell (X,Y,Z) = exp(mean log of its 2x2x2 fine cells)
__global__ void k_coarsen_cells(int fx, int fy, int fz, const float* __restrict__ a, float* __restrict__ ac)
{
    const int cx = fx / 2, cy = fy / 2, cz = fz / 2;
    const int64_t n = (int64_t)cx * cy * cz;
    const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= n) return;
    const int X = (int)(I / ((int64_t)cy * cz));
    const int Y = (int)((I / cz) % cy);
    const int Z = (int)(I % cz);
    float s = 0.f;
    for (int d = 0; d < 8; ++d) {
        const int x = 2 * X + (d >> 2), y = 2 * Y + ((d >> 1) & 1), z = 2 * Z + (d & 1);
        s += logf(a[((int64_t)x * fy + y) * fz + z]);
    }
    ac[I] = expf(s * 0.125f);
}

static int grid1(int64_t n) { return (int)std::max<int64_t>(1, ceil_div<int64_t>(n, 256)); }

// 3-D launch over an nx x ny x nz node grid: 32 z-consecutive nodes x 8 y-rows per block, one x-plane
// per grid z index (coalesced along z, no division for the coordinates)
constexpr int TG3_Z = 32, TG3_Y = 8;
static dim3 tgrid3(const NodeGrid& g) { return dim3(ceil_div(g.nz, TG3_Z), ceil_div(g.ny, TG3_Y), g.nx); }
static dim3 tblock3() { return dim3(TG3_Z, TG3_Y, 1); }

}  // namespace gb

using namespace gb;

// Multigrid transfer and smoothing kernels (no reference counterpart; see the file comment).
// Node grids are given as nodes per axis.  Masks (1 = Dirichlet node) may be null.
GB_API int gb_mg_restrict_c(int ncomp, int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* r,
                            const float* fmask, const float* cmask, float* rc, cudaStream_t stream)
{
    GB_REQUIRE(cnx == (fnx + 1) / 2 && cny == (fny + 1) / 2 && cnz == (fnz + 1) / 2, "mg_restrict: grid mismatch");
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "mg_restrict: 1 or 3 components");
    NodeGrid fg{fnx, fny, fnz}, cg{cnx, cny, cnz};
    GB_REQUIRE(cnx <= 65535, "mg_restrict: grid too long in x");
    if (ncomp == 1)
        GB_CHECK_CUDA(launch_pdl(k_restrict_fw<1>, tgrid3(cg), tblock3(), 0, stream, fg, cg, r, fmask, cmask, rc));
    else
        GB_CHECK_CUDA(launch_pdl(k_restrict_fw<3>, tgrid3(cg), tblock3(), 0, stream, fg, cg, r, fmask, cmask, rc));
    return GB_OK;
}

GB_API int gb_mg_prolong_add_c(int ncomp, int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* zc,
                               const float* fmask, float scale, float* z, cudaStream_t stream)
{
    GB_REQUIRE(cnx == (fnx + 1) / 2 && cny == (fny + 1) / 2 && cnz == (fnz + 1) / 2, "mg_prolong: grid mismatch");
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "mg_prolong: 1 or 3 components");
    NodeGrid fg{fnx, fny, fnz}, cg{cnx, cny, cnz};
    GB_REQUIRE(fnx <= 65535, "mg_prolong: grid too long in x");
    if (ncomp == 1)
        GB_CHECK_CUDA(launch_pdl(k_prolong_add<1>, tgrid3(fg), tblock3(), 0, stream, fg, cg, zc, fmask, scale, z));
    else
        GB_CHECK_CUDA(launch_pdl(k_prolong_add<3>, tgrid3(fg), tblock3(), 0, stream, fg, cg, zc, fmask, scale, z));
    return GB_OK;
}

GB_API int gb_mg_restrict(int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* r, const float* fmask,
                          const float* cmask, float* rc, cudaStream_t stream)
{
    return gb_mg_restrict_c(1, fnx, fny, fnz, cnx, cny, cnz, r, fmask, cmask, rc, stream);
}

GB_API int gb_mg_prolong_add(int fnx, int fny, int fnz, int cnx, int cny, int cnz, const float* zc,
                             const float* fmask, float scale, float* z, cudaStream_t stream)
{
    return gb_mg_prolong_add_c(1, fnx, fny, fnz, cnx, cny, cnz, zc, fmask, scale, z, stream);
}

GB_API int gb_mg_jacobi0(int64_t n, float omega, const float* dinv, const float* r, float* z, cudaStream_t stream)
{
    if (n <= 0) return GB_OK;
    GB_CHECK_CUDA(launch_pdl(k_jacobi0, (int)std::min<int64_t>(grid1(n), kSmCount * 8), 256, 0, stream, n, omega, dinv, r, z));
    return GB_OK;
}

GB_API int gb_mg_block_jacobi0(int64_t nodes, float omega, const float* dinv, const float* r, float* z,
                               cudaStream_t stream)
{
    if (nodes <= 0) return GB_OK;
    GB_REQUIRE(dinv && r && z && r != z, "mg_block_jacobi0: bad arguments");
    GB_CHECK_CUDA(launch_pdl(k_block_jacobi0, (int)std::min<int64_t>(grid1(nodes), kSmCount * 8), 256, 0, stream, nodes,
                             omega, dinv, r, z));
    return GB_OK;
}

GB_API int gb_mg_coarsen_cells(int fx, int fy, int fz, const float* a, float* ac, cudaStream_t stream)
{
    GB_REQUIRE(fx % 2 == 0 && fy % 2 == 0 && fz % 2 == 0, "mg_coarsen_cells: cell counts must be even");
    k_coarsen_cells<<<grid1((int64_t)(fx / 2) * (fy / 2) * (fz / 2)), 256, 0, stream>>>(fx, fy, fz, a, ac);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
