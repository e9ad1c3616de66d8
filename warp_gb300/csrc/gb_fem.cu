// gb_fem.cu -- Q1 finite-element assembly on regular Grid2D / Grid3D for the solve path.
//
// Replaces, for Q1 (bi/trilinear) nodal spaces on Grid2D/Grid3D, the bilinear-form assembly of
// warp.fem.integrate with the "dispatch" strategy (warp/_src/fem/integrate.py:1627-1878; local
// kernel :1108-1159; dispatch kernel warp/_src/fem/field/virtual.py:884-1116), the linear-form
// assembly of a nodal right-hand side, and the Dirichlet projection of
// warp/_src/fem/dirichlet.py:69-124.
//
// Triplet layout is the reference's: triplet index = (node-element pair) * NODES_PER_ELEMENT +
// trial node, where node-element pairs are ordered by test node and, for each node, by ascending
// element index (the space restriction's node->element map, warp/_src/fem/space/restriction.py);
// so bsr_set_from_triplets sums each block's element contributions in the reference's order.
// Node numbering x*(ny+1)*(nz+1) + y*(nz+1) + z (grid_3d_function_space.py:202-204), cell
// numbering x*ny*nz + y*nz + z (grid_3d.py:269-271), element-local node i*4 + j*2 + k
// (cube_shape_function.py:103-113); the 2-D forms drop the z axis.
//
// Element matrices of the unit cell are computed once on the host in FP64 (Gauss-Legendre,
// 2 points per axis, exact for Q1 products) and scaled here by the per-cell coefficient; values
// are rounded to fp32 once, like the reference's fp64-accumulated dispatch kernel.
#include "gb_common.cuh"

namespace gb {

// Number of cells adjacent to node coordinate i along an axis with n cells, and the count of
// (node, adjacent cell) pairs for all nodes before coordinate i.
__device__ __forceinline__ int axis_count(int i, int n) { return (i == 0 || i == n) ? 1 : 2; }
__device__ __forceinline__ int64_t axis_prefix(int i, int n) { return (i == 0) ? 0 : (int64_t)(2 * i - 1); }

struct Grid {
    int dim;
    int nx, ny, nz;  // cells per axis (nz = 0 for 2-D)
};

// Pair index of the first (node, element) pair of node (x, y, z).
__device__ __forceinline__ int64_t pair_start(const Grid& g, int x, int y, int z)
{
    if (g.dim == 2) {
        const int64_t Cy = 2 * (int64_t)g.ny;
        return axis_prefix(x, g.nx) * Cy + axis_count(x, g.nx) * axis_prefix(y, g.ny);
    }
    const int64_t Cy = 2 * (int64_t)g.ny, Cz = 2 * (int64_t)g.nz;
    return axis_prefix(x, g.nx) * Cy * Cz + axis_count(x, g.nx) * (axis_prefix(y, g.ny) * Cz +
                                                                    axis_count(y, g.ny) * axis_prefix(z, g.nz));
}

// s-th adjacent cell of node (x,y,z) in ascending cell index; returns false if s >= count.
__device__ __forceinline__ bool nth_cell(const Grid& g, int x, int y, int z, int s, int& cx, int& cy, int& cz)
{
    int lo[3] = {x - 1, y - 1, z - 1};
    int cnt[3];
    const int n[3] = {g.nx, g.ny, g.nz};
    const int c[3] = {x, y, z};
    for (int d = 0; d < 3; ++d) {
        if (d >= g.dim) {
            lo[d] = 0;
            cnt[d] = 1;
            continue;
        }
        int first = max(c[d] - 1, 0), last = min(c[d], n[d] - 1);
        lo[d] = first;
        cnt[d] = last - first + 1;
    }
    if (s >= cnt[0] * cnt[1] * cnt[2]) return false;
    const int sz = s % cnt[2];
    const int sy = (s / cnt[2]) % cnt[1];
    const int sx = s / (cnt[2] * cnt[1]);
    cx = lo[0] + sx;
    cy = lo[1] + sy;
    cz = lo[2] + sz;
    return true;
}

__device__ __forceinline__ int node_index(const Grid& g, int x, int y, int z)
{
    if (g.dim == 2) return x * (g.ny + 1) + y;
    return (x * (g.ny + 1) + y) * (g.nz + 1) + z;
}

__device__ __forceinline__ int cell_index(const Grid& g, int cx, int cy, int cz)
{
    if (g.dim == 2) return cx * g.ny + cy;
    return (cx * g.ny + cy) * g.nz + cz;
}

// element-local node index and its grid offsets
__device__ __forceinline__ void local_node(const Grid& g, int a, int& i, int& j, int& k)
{
    if (g.dim == 2) {
        i = a >> 1;
        j = a & 1;
        k = 0;
    } else {
        i = a >> 2;
        j = (a >> 1) & 1;
        k = a & 1;
    }
}

// One thread per (node, adjacent-cell slot): writes that pair's NPE triplets (trial nodes).
// ncomp = 1: scalar diffusion, value = coef[cell] * K[a][b] (K: NPE x NPE)
// ncomp = 3: linear elasticity, block(i,j) = lam[cell] * KL[(a,i),(b,j)] + mu[cell] * KM[(a,i),(b,j)]
template <int NCOMP>
__global__ void k_q1_triplets(Grid g, const double* __restrict__ K0, const double* __restrict__ K1,
                              const float* __restrict__ coef0, float coef0_const, const float* __restrict__ coef1,
                              float coef1_const, int* __restrict__ rows, int* __restrict__ cols,
                              float* __restrict__ vals)
{
    const int npe = (g.dim == 2) ? 4 : 8;
    const int64_t nnodes = (int64_t)(g.nx + 1) * (g.ny + 1) * (g.dim == 3 ? g.nz + 1 : 1);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * npe) return;
    const int s = (int)(t % npe);
    const int64_t node = t / npe;
    int x, y, z;
    if (g.dim == 2) {
        x = (int)(node / (g.ny + 1));
        y = (int)(node % (g.ny + 1));
        z = 0;
    } else {
        const int64_t pitch_x = (int64_t)(g.ny + 1) * (g.nz + 1);
        x = (int)(node / pitch_x);
        const int64_t rem = node - x * pitch_x;
        y = (int)(rem / (g.nz + 1));
        z = (int)(rem % (g.nz + 1));
    }
    int cx, cy, cz;
    if (!nth_cell(g, x, y, z, s, cx, cy, cz)) return;
    const int64_t pair = pair_start(g, x, y, z) + s;
    const int cell = cell_index(g, cx, cy, cz);
    const int a = (g.dim == 2) ? ((x - cx) * 2 + (y - cy)) : ((x - cx) * 4 + (y - cy) * 2 + (z - cz));
    const double c0 = coef0 ? (double)coef0[cell] : (double)coef0_const;
    const double c1 = coef1 ? (double)coef1[cell] : (double)coef1_const;
    const int nd = npe * NCOMP;  // element matrix dimension
    for (int b = 0; b < npe; ++b) {
        int bi, bj, bk;
        local_node(g, b, bi, bj, bk);
        const int64_t tri = pair * npe + b;
        rows[tri] = (int)node;
        cols[tri] = node_index(g, cx + bi, cy + bj, cz + bk);
#pragma unroll
        for (int i = 0; i < NCOMP; ++i) {
#pragma unroll
            for (int j = 0; j < NCOMP; ++j) {
                const int r = a * NCOMP + i, c = b * NCOMP + j;
                double v = c0 * K0[r * nd + c];
                if (NCOMP == 3) v += c1 * K1[r * nd + c];
                vals[tri * NCOMP * NCOMP + i * NCOMP + j] = (float)v;
            }
        }
    }
}

// b[node*ncomp + c] = sum_{cells e of node} sum_b M[a][b] * f[node(e,b)*ncomp + c]  (nodal f), or
// f_const[c] * sum_e sum_b M[a][b] when f is null (uniform body force).  Accumulated in fp64.
__global__ void k_q1_rhs(Grid g, int ncomp, const double* __restrict__ M, const float* __restrict__ f,
                         float f0, float f1, float f2, float* __restrict__ out)
{
    const int npe = (g.dim == 2) ? 4 : 8;
    const int64_t nnodes = (int64_t)(g.nx + 1) * (g.ny + 1) * (g.dim == 3 ? g.nz + 1 : 1);
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nnodes) return;
    int x, y, z;
    if (g.dim == 2) {
        x = (int)(node / (g.ny + 1));
        y = (int)(node % (g.ny + 1));
        z = 0;
    } else {
        const int64_t pitch_x = (int64_t)(g.ny + 1) * (g.nz + 1);
        x = (int)(node / pitch_x);
        const int64_t rem = node - x * pitch_x;
        y = (int)(rem / (g.nz + 1));
        z = (int)(rem % (g.nz + 1));
    }
    double acc[3] = {0, 0, 0};
    const float fc[3] = {f0, f1, f2};
    for (int s = 0; s < 8; ++s) {
        int cx, cy, cz;
        if (!nth_cell(g, x, y, z, s, cx, cy, cz)) break;
        const int a = (g.dim == 2) ? ((x - cx) * 2 + (y - cy)) : ((x - cx) * 4 + (y - cy) * 2 + (z - cz));
        for (int b = 0; b < npe; ++b) {
            const double m = M[a * npe + b];
            if (f) {
                int bi, bj, bk;
                local_node(g, b, bi, bj, bk);
                const int nb = node_index(g, cx + bi, cy + bj, cz + bk);
                for (int c = 0; c < ncomp; ++c) acc[c] += m * (double)f[(size_t)nb * ncomp + c];
            } else {
                for (int c = 0; c < ncomp; ++c) acc[c] += m * (double)fc[c];
            }
        }
    }
    for (int c = 0; c < ncomp; ++c) out[(size_t)node * ncomp + c] = (float)acc[c];
}

// Per-dof Dirichlet mask on the grid boundary.  face_bits: bit 2d = the low face of axis d,
// bit 2d+1 = the high face; comp_mask: which of the ncomp components are constrained.
__global__ void k_grid_boundary_mask(Grid g, int face_bits, int ncomp, int comp_mask, float* __restrict__ mask)
{
    const int64_t nnodes = (int64_t)(g.nx + 1) * (g.ny + 1) * (g.dim == 3 ? g.nz + 1 : 1);
    const int64_t node = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= nnodes) return;
    int c[3];
    if (g.dim == 2) {
        c[0] = (int)(node / (g.ny + 1));
        c[1] = (int)(node % (g.ny + 1));
        c[2] = 0;
    } else {
        const int64_t pitch_x = (int64_t)(g.ny + 1) * (g.nz + 1);
        c[0] = (int)(node / pitch_x);
        const int64_t rem = node - c[0] * pitch_x;
        c[1] = (int)(rem / (g.nz + 1));
        c[2] = (int)(rem % (g.nz + 1));
    }
    const int n[3] = {g.nx, g.ny, g.nz};
    bool on = false;
    for (int d = 0; d < g.dim; ++d) {
        if ((face_bits >> (2 * d)) & 1) on |= (c[d] == 0);
        if ((face_bits >> (2 * d + 1)) & 1) on |= (c[d] == n[d]);
    }
    for (int k = 0; k < ncomp; ++k) mask[(size_t)node * ncomp + k] = (on && ((comp_mask >> k) & 1)) ? 1.f : 0.f;
}

// A <- (I - P) A (I - P) + P for a diagonal projector P = diag(mask) (mask per scalar dof,
// 0 or 1), keeping A's structure (explicit zeros stay).  Block row per thread.
template <int B>
__global__ void k_project_matrix(int nrow, const int* __restrict__ offsets, const int* __restrict__ columns,
                                 float* __restrict__ values, const float* __restrict__ mask)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= nrow) return;
    float mr[B];
#pragma unroll
    for (int i = 0; i < B; ++i) mr[i] = mask[(size_t)row * B + i];
    for (int k = offsets[row]; k < offsets[row + 1]; ++k) {
        const int col = columns[k];
#pragma unroll
        for (int i = 0; i < B; ++i) {
#pragma unroll
            for (int j = 0; j < B; ++j) {
                const float mc = mask[(size_t)col * B + j];
                float v = values[((size_t)k * B + i) * B + j];
                v = (1.f - mr[i]) * (1.f - mc) * v;
                if (col == row && i == j) v += mr[i];
                values[((size_t)k * B + i) * B + j] = v;
            }
        }
    }
}

// b <- (I - P) b + P f   (the reference's (I-P)(b - A P f) + P f once b already holds b - A P f)
__global__ void k_project_rhs(int64_t n, const float* __restrict__ mask, const float* __restrict__ fixed,
                              float* __restrict__ b)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float m = mask[i];
        b[i] = (1.f - m) * b[i] + (fixed ? m * fixed[i] : 0.f);
    }
}

// t = P f  (mask * f)
__global__ void k_mask_mul(int64_t n, const float* __restrict__ mask, const float* __restrict__ f, float* __restrict__ t)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        t[i] = mask[i] * f[i];
}

}  // namespace gb

using namespace gb;

int gb_bsr_mv_internal(int bdim, int nrow, const int* offsets, const int* columns, const float* values,
                       const float* x, float* y, cudaStream_t stream);

static int64_t grid_nodes(int dim, int nx, int ny, int nz)
{
    return (int64_t)(nx + 1) * (ny + 1) * (dim == 3 ? (nz + 1) : 1);
}

// Number of triplets the Q1 bilinear assembly writes: cells * NPE^2 (reference integrate.py:1637).
GB_API int64_t gb_q1_triplet_count(int dim, int nx, int ny, int nz)
{
    const int64_t cells = (int64_t)nx * ny * (dim == 3 ? nz : 1);
    const int npe = dim == 3 ? 8 : 4;
    return cells * npe * npe;
}

// Q1 bilinear-form triplets.  ncomp = 1: K0 = unit-coefficient stiffness (NPE x NPE), coefficient
// per cell (coef0) or constant.  ncomp = 3: K0 = lambda part, K1 = mu part (3NPE x 3NPE).
GB_API int gb_q1_assemble_triplets(int dim, int nx, int ny, int nz, int ncomp, const double* K0, const double* K1,
                                   const float* coef0, float coef0_const, const float* coef1, float coef1_const,
                                   int* rows, int* cols, float* vals, cudaStream_t stream)
{
    GB_REQUIRE(dim == 2 || dim == 3, "q1_assemble: dim must be 2 or 3");
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "q1_assemble: ncomp must be 1 or 3");
    GB_REQUIRE(nx > 0 && ny > 0 && (dim == 2 || nz > 0), "q1_assemble: empty grid");
    GB_REQUIRE(K0 && rows && cols && vals && (ncomp == 1 || K1), "q1_assemble: null argument");
    Grid g{dim, nx, ny, dim == 3 ? nz : 0};
    const int npe = dim == 3 ? 8 : 4;
    const int64_t nthreads = grid_nodes(dim, nx, ny, nz) * npe;
    const int grid = (int)ceil_div<int64_t>(nthreads, 256);
    if (ncomp == 1)
        k_q1_triplets<1><<<grid, 256, 0, stream>>>(g, K0, K1, coef0, coef0_const, coef1, coef1_const, rows, cols, vals);
    else
        k_q1_triplets<3><<<grid, 256, 0, stream>>>(g, K0, K1, coef0, coef0_const, coef1, coef1_const, rows, cols, vals);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// Q1 linear form with the consistent mass matrix M (NPE x NPE, device fp64): nodal f
// ([nodes * ncomp]) or a constant vector (f null, f0..f2).
GB_API int gb_q1_assemble_rhs(int dim, int nx, int ny, int nz, int ncomp, const double* M, const float* f, float f0,
                              float f1, float f2, float* out, cudaStream_t stream)
{
    GB_REQUIRE(dim == 2 || dim == 3, "q1_rhs: dim must be 2 or 3");
    GB_REQUIRE(ncomp >= 1 && ncomp <= 3, "q1_rhs: ncomp must be 1..3");
    Grid g{dim, nx, ny, dim == 3 ? nz : 0};
    const int64_t nn = grid_nodes(dim, nx, ny, nz);
    k_q1_rhs<<<(int)ceil_div<int64_t>(nn, 256), 256, 0, stream>>>(g, ncomp, M, f, f0, f1, f2, out);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

GB_API int gb_grid_boundary_mask(int dim, int nx, int ny, int nz, int face_bits, int ncomp, int comp_mask, float* mask,
                                 cudaStream_t stream)
{
    GB_REQUIRE(dim == 2 || dim == 3, "boundary_mask: dim must be 2 or 3");
    Grid g{dim, nx, ny, dim == 3 ? nz : 0};
    const int64_t nn = grid_nodes(dim, nx, ny, nz);
    k_grid_boundary_mask<<<(int)ceil_div<int64_t>(nn, 256), 256, 0, stream>>>(g, face_bits, ncomp, comp_mask, mask);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// Dirichlet projection of a compact BSR system (reference: project_linear_system,
// warp/_src/fem/dirichlet.py:107-124, with a normalised diagonal projector given as a 0/1 mask
// per scalar dof).  rhs: b <- (I-P)(b - A P f) + P f; matrix: A <- (I-P) A (I-P) + P.
// `tmp` is an n-float scratch vector used only when fixed != null.
GB_API int gb_dirichlet_project(int bdim, int nrow, const int* offsets, const int* columns, float* values,
                                const float* mask, float* rhs, const float* fixed, float* tmp, int project_matrix,
                                cudaStream_t stream)
{
    GB_REQUIRE(bdim == 1 || bdim == 3, "dirichlet_project: block dim must be 1 or 3");
    const int64_t n = (int64_t)nrow * bdim;
    const int vg = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 8));
    if (rhs) {
        if (fixed) {
            GB_REQUIRE(tmp != nullptr, "dirichlet_project: scratch vector required with fixed values");
            k_mask_mul<<<vg, 256, 0, stream>>>(n, mask, fixed, tmp);
            // b -= A (P f): generic product through the exported SpMV
            int rc = gb_bsr_mv_internal(bdim, nrow, offsets, columns, values, tmp, rhs, stream);
            if (rc) return rc;
        }
        k_project_rhs<<<vg, 256, 0, stream>>>(n, mask, fixed, rhs);
        GB_CHECK_CUDA(cudaGetLastError());
    }
    if (project_matrix) {
        const int grid = ceil_div(nrow, 128);
        if (bdim == 1)
            k_project_matrix<1><<<grid, 128, 0, stream>>>(nrow, offsets, columns, values, mask);
        else
            k_project_matrix<3><<<grid, 128, 0, stream>>>(nrow, offsets, columns, values, mask);
        GB_CHECK_CUDA(cudaGetLastError());
    }
    return GB_OK;
}
