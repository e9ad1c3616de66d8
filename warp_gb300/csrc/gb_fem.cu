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
#include "gb_scan.cuh"

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
// Value of scalar (i, j) of the triplet (test node a, trial node b) of a cell: the fp32 element
// tables (rounded once from the FP64 integrals) scaled by the cell's coefficients in fp32, with a
// fixed operation order so every assembly route produces the same bits.
template <int NCOMP>
__device__ __forceinline__ float q1_entry(const float* __restrict__ K0, const float* __restrict__ K1, int nd, int r,
                                          int c, float c0, float c1)
{
    const float v = __fmul_rn(c0, K0[r * nd + c]);
    return NCOMP == 3 ? __fmaf_rn(c1, K1[r * nd + c], v) : v;
}

template <int NCOMP>
__global__ void k_q1_triplets(Grid g, const float* __restrict__ K0, const float* __restrict__ K1,
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
    const float c0 = coef0 ? coef0[cell] : coef0_const;
    const float c1 = coef1 ? coef1[cell] : coef1_const;
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
            for (int j = 0; j < NCOMP; ++j)
                vals[tri * NCOMP * NCOMP + i * NCOMP + j] =
                    q1_entry<NCOMP>(K0, K1, nd, a * NCOMP + i, b * NCOMP + j, c0, c1);
        }
    }
}

// Direct assembly of the Q1 bilinear form into compact BSR (no triplets, no sort).  Produces exactly
// what k_q1_triplets + bsr_set_from_triplets + the run sums produce: row = test node; its candidate
// blocks are generated in triplet order (adjacent cells in ascending cell index, then trial nodes in
// element-local order), a triplet whose scalars are all zero is dropped when pruning (bits & 0x7FFFFFFF),
// each block is the fp32 sum of its remaining triplets in that order (starting from the first one),
// and blocks are stored in ascending column (node) order.  Thread layout: NCOMP = 1, one thread per
// row; NCOMP = 3, a group of 4 lanes per block row (lanes 0..2 hold component rows i = 0..2, lane 3
// mirrors lane 0 and writes nothing) that agree on each triplet's zero test with two shuffles.
// Cells are visited by their offset (ox, oy, oz) in {-1, 0}^3 from the node, so every index is a
// compile-time constant and the 27 (9 in 2-D) block accumulators live in registers.
// FILL = false: counts[row] = number of blocks; FILL = true: write columns / values at offsets[row].
constexpr int Q1_BSR_THREADS = 128;

template <int DIM, int NCOMP, bool FILL>
__device__ __forceinline__ void q1_bsr_row(Grid g, const float* __restrict__ K0, const float* __restrict__ K1,
                                           const float* __restrict__ coef0, float coef0_const,
                                           const float* __restrict__ coef1, float coef1_const, int prune,
                                           int* __restrict__ counts, const int* __restrict__ offsets, int* s_cols,
                                           float* s_vals)
{
    constexpr int NPE = DIM == 3 ? 8 : 4;
    constexpr int ND = NPE * NCOMP;
    constexpr int NNB = DIM == 3 ? 27 : 9;
    constexpr int LPR = NCOMP == 3 ? 4 : 1;  // lanes per block row
    const int64_t nnodes = (int64_t)(g.nx + 1) * (g.ny + 1) * (DIM == 3 ? g.nz + 1 : 1);
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t node = t / LPR;
    const int comp = (int)(t % LPR);
    if (node >= nnodes) return;  // whole 4-lane groups leave together
    const int ci = comp < NCOMP ? comp : 0;
    const unsigned gmask = NCOMP == 3 ? (0xFu << (threadIdx.x & 28)) : 0u;
    int x, y, z = 0;
    if (DIM == 2) {
        x = (int)(node / (g.ny + 1));
        y = (int)(node % (g.ny + 1));
    } else {
        const int64_t pitch_x = (int64_t)(g.ny + 1) * (g.nz + 1);
        x = (int)(node / pitch_x);
        const int64_t rem = node - x * pitch_x;
        y = (int)(rem / (g.nz + 1));
        z = (int)(rem % (g.nz + 1));
    }
    float acc[NNB][NCOMP];
    uint32_t has = 0;
#pragma unroll
    for (int k = 0; k < NNB; ++k)
#pragma unroll
        for (int j = 0; j < NCOMP; ++j) acc[k][j] = 0.f;
#pragma unroll
    for (int oc = 0; oc < (1 << DIM); ++oc) {
        // cell offset from the node, ascending cell index: ox outermost, each -1 before 0
        const int ox = (oc >> (DIM - 1)) - 1;
        const int oy = DIM == 3 ? ((oc >> 1) & 1) - 1 : (oc & 1) - 1;
        const int oz = DIM == 3 ? (oc & 1) - 1 : 0;
        const int cx = x + ox, cy = y + oy, cz = z + oz;
        const bool inside = cx >= 0 && cx < g.nx && cy >= 0 && cy < g.ny && (DIM == 2 || (cz >= 0 && cz < g.nz));
        if (!inside) continue;  // uniform inside a lane group (same node)
        const int cell = DIM == 2 ? cx * g.ny + cy : (cx * g.ny + cy) * g.nz + cz;
        const float c0 = coef0 ? coef0[cell] : coef0_const;
        const float c1 = coef1 ? coef1[cell] : coef1_const;
        const int a = DIM == 2 ? (-ox) * 2 + (-oy) : (-ox) * 4 + (-oy) * 2 + (-oz);
#pragma unroll
        for (int b = 0; b < NPE; ++b) {
            const int bi = DIM == 2 ? (b >> 1) : (b >> 2);
            const int bj = DIM == 2 ? (b & 1) : ((b >> 1) & 1);
            const int bk = DIM == 2 ? 0 : (b & 1);
            const int k = DIM == 2 ? 3 * (ox + bi + 1) + (oy + bj + 1)
                                   : 9 * (ox + bi + 1) + 3 * (oy + bj + 1) + (oz + bk + 1);
            float v[NCOMP];
            uint32_t nzbits = 0;
#pragma unroll
            for (int j = 0; j < NCOMP; ++j) {
                v[j] = q1_entry<NCOMP>(K0, K1, ND, a * NCOMP + ci, b * NCOMP + j, c0, c1);
                nzbits |= __float_as_uint(v[j]) & 0x7FFFFFFFu;
            }
            if (NCOMP == 3) {
                nzbits = comp < NCOMP ? nzbits : 0u;
                nzbits |= __shfl_xor_sync(gmask, nzbits, 1);
                nzbits |= __shfl_xor_sync(gmask, nzbits, 2);
            }
            if (!prune || nzbits != 0u) {
                const bool first = !(has & (1u << k));
#pragma unroll
                for (int j = 0; j < NCOMP; ++j) acc[k][j] = first ? v[j] : acc[k][j] + v[j];
                has |= 1u << k;
            }
        }
    }
    if (!FILL) {
        if (comp == 0) counts[node] = __popc(has);
        return;
    }
    // the CTA's rows are one contiguous range of blocks: stage them in shared memory (the kernel then
    // copies the range out with coalesced stores)
    const int base = offsets[(int64_t)blockIdx.x * (blockDim.x / LPR)];
    int pos = offsets[node] - base;
    const int64_t sy = DIM == 3 ? (g.nz + 1) : 1;
    const int64_t sx = DIM == 3 ? (int64_t)(g.ny + 1) * (g.nz + 1) : (g.ny + 1);
#pragma unroll
    for (int k = 0; k < NNB; ++k) {
        if (has & (1u << k)) {
            const int dx = DIM == 3 ? k / 9 - 1 : k / 3 - 1;
            const int dy = DIM == 3 ? (k / 3) % 3 - 1 : k % 3 - 1;
            const int dz = DIM == 3 ? k % 3 - 1 : 0;
            if (comp == 0) s_cols[pos] = (int)(node + dx * sx + dy * sy + dz);
            if (comp < NCOMP) {
#pragma unroll
                for (int j = 0; j < NCOMP; ++j) s_vals[(pos * NCOMP + ci) * NCOMP + j] = acc[k][j];
            }
            ++pos;
        }
    }
}

// Coalesced copy of a CTA's staged blocks (see k_q1_bsr): called after the CTA's barrier.
template <int NCOMP>
__device__ __forceinline__ void q1_bsr_flush(int nblocks, int base, const int* s_cols, const float* s_vals,
                                             int* __restrict__ columns, float* __restrict__ values)
{
    for (int t = threadIdx.x; t < nblocks; t += blockDim.x) columns[base + t] = s_cols[t];
    for (int t = threadIdx.x; t < nblocks * NCOMP * NCOMP; t += blockDim.x)
        values[(size_t)base * NCOMP * NCOMP + t] = s_vals[t];
}

template <int DIM, int NCOMP, bool FILL>
__global__ void __launch_bounds__(Q1_BSR_THREADS) k_q1_bsr(Grid g, const float* __restrict__ K0g,
                                                           const float* __restrict__ K1g,
                                                           const float* __restrict__ coef0, float coef0_const,
                                                           const float* __restrict__ coef1, float coef1_const,
                                                           int prune, int* __restrict__ counts,
                                                           const int* __restrict__ offsets, int* __restrict__ columns,
                                                           float* __restrict__ values)
{
    constexpr int NPE = DIM == 3 ? 8 : 4;
    constexpr int ND = NPE * NCOMP;
    constexpr int NNB = DIM == 3 ? 27 : 9;
    constexpr int LPR = NCOMP == 3 ? 4 : 1;
    constexpr int ROWS = Q1_BSR_THREADS / LPR;
    __shared__ float K0[ND * ND];
    __shared__ float K1[NCOMP == 3 ? ND * ND : 1];
    __shared__ int s_cols[FILL ? ROWS * NNB : 1];
    __shared__ float s_vals[FILL ? ROWS * NNB * NCOMP * NCOMP : 1];
    for (int t = threadIdx.x; t < ND * ND; t += blockDim.x) {
        K0[t] = K0g[t];
        if (NCOMP == 3) K1[t] = K1g[t];
    }
    __syncthreads();
    q1_bsr_row<DIM, NCOMP, FILL>(g, K0, K1, coef0, coef0_const, coef1, coef1_const, prune, counts, offsets, s_cols,
                                 s_vals);
    if (FILL) {
        const int64_t nnodes = (int64_t)(g.nx + 1) * (g.ny + 1) * (DIM == 3 ? g.nz + 1 : 1);
        const int64_t row0 = (int64_t)blockIdx.x * ROWS;
        const int64_t row1 = min(row0 + (int64_t)ROWS, nnodes);
        __syncthreads();
        const int base = offsets[row0];
        q1_bsr_flush<NCOMP>(offsets[row1] - base, base, s_cols, s_vals, columns, values);
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

// Q1 bilinear-form triplets.  ncomp = 1: K0 = unit-coefficient stiffness (NPE x NPE, fp32), coefficient
// per cell (coef0) or constant.  ncomp = 3: K0 = lambda part, K1 = mu part (3NPE x 3NPE, fp32).
GB_API int gb_q1_assemble_triplets(int dim, int nx, int ny, int nz, int ncomp, const float* K0, const float* K1,
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

// Upper bound (exact when nothing is pruned) of the blocks of the direct assembly: prod (3 m_d - 2).
GB_API int64_t gb_q1_bsr_nnz_max(int dim, int nx, int ny, int nz)
{
    int64_t n = (int64_t)(3 * (nx + 1) - 2) * (3 * (ny + 1) - 2);
    return dim == 3 ? n * (3 * (nz + 1) - 2) : n;
}

GB_API size_t gb_q1_assemble_bsr_workspace_bytes(int dim, int nx, int ny, int nz)
{
    return scan_workspace_bytes(grid_nodes(dim, nx, ny, nz) + 1);
}

// Direct compact-BSR assembly of the Q1 bilinear form (same tables and coefficients as
// gb_q1_assemble_triplets): the matrix bsr_set_from_triplets builds from those triplets, bit for bit,
// without writing or sorting them.  offsets: [nodes + 1]; columns / values: capacity
// gb_q1_bsr_nnz_max(); bsr_nnz_host (optional) receives offsets[nodes] asynchronously.
GB_API int gb_q1_assemble_bsr(int dim, int nx, int ny, int nz, int ncomp, const float* K0, const float* K1,
                              const float* coef0, float coef0_const, const float* coef1, float coef1_const, int prune,
                              int* offsets, int* columns, float* values, int* bsr_nnz_host, void* workspace,
                              size_t workspace_bytes, cudaStream_t stream)
{
    GB_REQUIRE(dim == 2 || dim == 3, "q1_assemble_bsr: dim must be 2 or 3");
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "q1_assemble_bsr: ncomp must be 1 or 3");
    GB_REQUIRE(nx > 0 && ny > 0 && (dim == 2 || nz > 0), "q1_assemble_bsr: empty grid");
    GB_REQUIRE(K0 && offsets && columns && values && (ncomp == 1 || K1), "q1_assemble_bsr: null argument");
    GB_REQUIRE(workspace_bytes >= gb_q1_assemble_bsr_workspace_bytes(dim, nx, ny, nz),
               "q1_assemble_bsr: workspace too small");
    Grid g{dim, nx, ny, dim == 3 ? nz : 0};
    const int64_t nn = grid_nodes(dim, nx, ny, nz);
    const int lpr = ncomp == 3 ? 4 : 1;
    const int grid = (int)ceil_div<int64_t>(nn * lpr, Q1_BSR_THREADS);
#define GB_Q1_BSR(D, C, F) \
    k_q1_bsr<D, C, F><<<grid, Q1_BSR_THREADS, 0, stream>>>(g, K0, K1, coef0, coef0_const, coef1, coef1_const, prune, offsets + 1, \
                                                offsets, columns, values)
    // pass 1: blocks per row (into offsets[1..]); exclusive scan; pass 2: write the rows
    GB_CHECK_CUDA(cudaMemsetAsync(offsets, 0, sizeof(int), stream));
    if (dim == 3 && ncomp == 1) GB_Q1_BSR(3, 1, false);
    else if (dim == 3) GB_Q1_BSR(3, 3, false);
    else if (ncomp == 1) GB_Q1_BSR(2, 1, false);
    else GB_Q1_BSR(2, 3, false);
    GB_CHECK_CUDA(cudaGetLastError());
    int rc = scan_i32(offsets + 1, offsets + 1, nn, true, workspace, stream);
    if (rc) return rc;
    if (dim == 3 && ncomp == 1) GB_Q1_BSR(3, 1, true);
    else if (dim == 3) GB_Q1_BSR(3, 3, true);
    else if (ncomp == 1) GB_Q1_BSR(2, 1, true);
    else GB_Q1_BSR(2, 3, true);
#undef GB_Q1_BSR
    GB_CHECK_CUDA(cudaGetLastError());
    if (bsr_nnz_host)
        GB_CHECK_CUDA(cudaMemcpyAsync(bsr_nnz_host, offsets + nn, sizeof(int), cudaMemcpyDeviceToHost, stream));
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
