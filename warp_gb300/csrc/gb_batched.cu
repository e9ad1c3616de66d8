// gb_batched.cu -- thousands of independent sparse SPD systems: batched Q1 assembly and a
// persistent batched Jacobi-CG launch.
//
// Reference semantics (warp/_src/optim/linear.py:33-133, 893-1032, 2047-2083, 2333-2373): a block-
// diagonal operator with batch_offsets[B+1] partitioning the scalar rows into B subproblems (rows at
// or beyond batch_offsets[B] are inactive and never touched); each subproblem has its own absolute
// tolerance atol_b = max(rtol * ||b_b||, atol) and its own alpha / beta, and stops updating once
// ||r_b||^2 <= atol_b^2; the loop ends when every subproblem has converged or after maxiter
// iterations.
//
// GB300 design: no grid-wide step at all.  One persistent launch; each CTA pulls subproblems from
// an atomic queue (ordered largest first, so the longest solves start first) and runs the whole
// Jacobi-CG of one subproblem to its own convergence with block-level reductions (fp32 partials,
// fp64 across warps, fixed order: deterministic for a given configuration).  Once the queue reaches
// subproblems of at most `small_rows` rows, the CTA's warps take one subproblem each and iterate with
// warp-level reductions only.  Per iteration a subproblem streams its rows once for A p (LPR lanes
// per row, shuffle-reduced) and twice for the vector updates; its vectors (a few hundred KB at most)
// stay in L1/L2 while it runs.  The configuration (threads per CTA, lanes per row, small-problem
// threshold) is chosen by the package's autotuner.
#include "gb_common.cuh"

namespace gb {

struct BatchArgs {
    int nbatch;
    const int* batch_offsets;  // [B+1]
    const int* order;          // [B] subproblem ids, largest first
    const int* offsets;        // CSR of the block-diagonal matrix (global row / column indices)
    const int* columns;
    const float* values;
    const float* dinv;         // Jacobi (inverse diagonal) or null
    const float* b;
    float* x;
    float* r;
    float* p;
    float* Ap;
    float *r0, *v, *t, *y, *z;  // BiCGSTAB only
    int left_precond;           // BiCGSTAB: left (1) or right (0) preconditioning
    float rtol, atol;
    int maxiter;
    int x_is_zero;
    int small_rows;
    int smem_rows;             // CTA-mode subproblems of at most this many rows keep p, r, Ap in shared memory
    int* queue;                // work counter, zero at launch
    int* iters;                // [B]
    float* rr_out;             // [B] final ||r||^2
    float* atol_sq_out;        // [B]
    int* status;
};

// Sum NV values over `nthreads` threads of a group (CTA mode: whole block; every thread gets the
// result).  red: >= 32 * NV doubles of shared memory.
template <int NV>
__device__ __forceinline__ void cta_allreduce(const float (&in)[NV], double (&out)[NV], double* red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const float s = warp_sum(in[k]);
        if (lane == 0) red[wid * NV + k] = (double)s;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += red[w * NV + k];
        out[k] = s;
    }
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void warp_allreduce(const float (&in)[NV], double (&out)[NV])
{
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = (double)warp_sum(in[k]);
}

// One CG of subproblem pid by a group of `nthr` threads (tid in [0, nthr)); WARP: the group is one
// warp (warp reductions, __syncwarp between phases), else the whole CTA.  SV: p, r and Ap live in
// `svec` (shared memory, 3 x smem_rows floats, indexed by row - r0): per iteration HBM then carries
// the matrix, x and D^-1 only; gathers of p stay on chip.  Column indices outside the subproblem's rows
// (none in a block-diagonal batch) read zero in that mode.
template <int LPR, bool WARP, bool SV>
__device__ void solve_one(const BatchArgs& a, int pid, int tid, int nthr, double* red, float* svec)
{
    const int r0 = a.batch_offsets[pid], r1 = a.batch_offsets[pid + 1];
    const int gid = tid / LPR, sub = tid % LPR;
    const int rows_per_pass = nthr / LPR;
    // vector p, r, Ap: element of global row i at vp[i - vb]
    const int vb = SV ? r0 : 0;
    float* vp = SV ? svec : a.p;
    float* vr = SV ? svec + a.smem_rows : a.r;
    float* vAp = SV ? svec + 2 * a.smem_rows : a.Ap;
    const unsigned nloc = (unsigned)(r1 - r0);
    auto sync = [&]() {
        if (WARP)
            __syncwarp();
        else
            __syncthreads();
    };
    // A v on this group's rows (v indexed from vbase); returns (per thread) the partial sum of
    // w[row] * (A v)[row] and stores (A v) into out (sub-lane 0 only; out and w indexed from vb);
    // residual: out = b - A v.  Two rows per group per pass, and each row's nonzeros of this lane are
    // loaded as one predicated batch of U, so a lane keeps 2 U column / value loads and then 2 U
    // gathers in flight instead of walking a chain.
    constexpr int U = LPR == 1 ? 9 : (LPR == 2 ? 5 : (LPR == 4 ? 3 : 2));
    auto matvec = [&](const float* v, int vbase, bool v_local, float* out, const float* w, bool residual) -> float {
        float part = 0.f;
        for (int base = r0; base < r1; base += 2 * rows_per_pass) {
            int row[2], k1[2], kb[2];
            float s[2] = {0.f, 0.f};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                row[h] = base + gid + h * rows_per_pass;
                const bool valid = row[h] < r1;
                kb[h] = valid ? a.offsets[row[h]] + sub : 0;
                k1[h] = valid ? a.offsets[row[h] + 1] : 0;
            }
            while (kb[0] < k1[0] || kb[1] < k1[1]) {
                int cc[2][U];
                float vv[2][U];
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int k = kb[h] + u * LPR;
                        const bool in = k < k1[h];
                        cc[h][u] = in ? a.columns[k] : -1;
                        vv[h][u] = in ? a.values[k] : 0.f;
                    }
                float xv[2][U];
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int c = cc[h][u];
                        if (v_local)
                            xv[h][u] = (unsigned)(c - r0) < nloc ? v[c - vbase] : 0.f;
                        else
                            xv[h][u] = c >= 0 ? v[c - vbase] : 0.f;
                    }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
#pragma unroll
                    for (int u = 0; u < U; ++u) s[h] += vv[h][u] * xv[h][u];
                    kb[h] += U * LPR;
                }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float sh = group_sum<LPR>(s[h]);
                if (row[h] < r1 && sub == 0) {
                    const float o = residual ? a.b[row[h]] - sh : sh;
                    out[row[h] - vb] = o;
                    if (w) part += w[row[h] - vb] * o;
                }
            }
        }
        return part;
    };

    // ---- init: r = b - A x (or b), z = D^-1 r, p = z, ||b||^2, ||r||^2, r.z --------------------
    if (a.x_is_zero) {
        for (int i = r0 + tid; i < r1; i += nthr) {
            a.x[i] = 0.f;
            vr[i - vb] = a.b[i];
        }
    } else {
        matvec(a.x, 0, false, vr, nullptr, true);
    }
    sync();
    float part3[3] = {0.f, 0.f, 0.f};
    for (int i = r0 + tid; i < r1; i += nthr) {
        const float ri = vr[i - vb], bi = a.b[i];
        const float zi = a.dinv ? a.dinv[i] * ri : ri;
        vp[i - vb] = zi;
        part3[0] += bi * bi;
        part3[1] += ri * ri;
        part3[2] += ri * zi;
    }
    double tot3[3];
    if (WARP)
        warp_allreduce<3>(part3, tot3);
    else
        cta_allreduce<3>(part3, tot3, red);
    sync();  // p is gathered by other lanes in the first A p
    const double an = fmax((double)a.rtol * sqrt(tot3[0]), (double)a.atol);
    const double atol_sq = an * an;
    double rr = tot3[1], rz = tot3[2];
    int it = 0;
    bool broke = false;
    while (it < a.maxiter && rr > atol_sq) {
        // ---- A p and p.Ap ----------------------------------------------------------------------
        float part1[1] = {matvec(vp, vb, SV, vAp, vp, false)};
        double pAp[1];
        if (WARP)
            warp_allreduce<1>(part1, pAp);
        else
            cta_allreduce<1>(part1, pAp, red);  // includes the block barriers between phases
        if (!(pAp[0] > 0.0) || !isfinite(pAp[0])) {
            broke = true;
            break;
        }
        const float alpha = (float)(rz / pAp[0]);
        if (WARP) __syncwarp();
        // ---- x += alpha p, r -= alpha Ap, z = D^-1 r, r.r, r.z --------------------------------
        float part2[2] = {0.f, 0.f};
#pragma unroll 4
        for (int i = r0 + tid; i < r1; i += nthr) {
            const float pi = vp[i - vb];
            a.x[i] += alpha * pi;
            const float ri = vr[i - vb] - alpha * vAp[i - vb];
            vr[i - vb] = ri;
            const float zi = a.dinv ? a.dinv[i] * ri : ri;
            part2[0] += ri * ri;
            part2[1] += ri * zi;
        }
        double tot2[2];
        if (WARP)
            warp_allreduce<2>(part2, tot2);
        else
            cta_allreduce<2>(part2, tot2, red);
        const float beta = (float)(tot2[1] / rz);
        if (!isfinite(beta)) {
            broke = true;
            break;
        }
        // ---- p = z + beta p --------------------------------------------------------------------
#pragma unroll 4
        for (int i = r0 + tid; i < r1; i += nthr) {
            const float ri = vr[i - vb];
            const float zi = a.dinv ? a.dinv[i] * ri : ri;
            vp[i - vb] = zi + beta * vp[i - vb];
        }
        sync();
        rr = tot2[0];
        rz = tot2[1];
        ++it;
    }
    if (tid == 0) {
        a.iters[pid] = it;
        a.rr_out[pid] = (float)rr;
        a.atol_sq_out[pid] = (float)atol_sq;
        if (broke) atomicOr(a.status, GB_DEV_BREAKDOWN);
    }
    sync();
}

// out[row] = (A v)[row] for the rows [r0, r1) of one subproblem by a CTA (LPR lanes per row).
template <int LPR>
__device__ void batch_spmv(const BatchArgs& a, int r0, int r1, const float* __restrict__ v, float* __restrict__ out)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int gid = tid / LPR, sub = tid % LPR;
    const int rows_per_pass = nthr / LPR;
    constexpr int U = LPR == 1 ? 9 : (LPR == 2 ? 5 : (LPR == 4 ? 3 : 2));
    for (int base = r0; base < r1; base += rows_per_pass) {
        const int row = base + gid;
        const bool valid = row < r1;
        int kb = valid ? a.offsets[row] + sub : 0;
        const int k1 = valid ? a.offsets[row + 1] : 0;
        float s = 0.f;
        while (kb < k1) {
            int cc[U];
            float vv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int k = kb + u * LPR;
                const bool in = k < k1;
                cc[u] = in ? a.columns[k] : -1;
                vv[u] = in ? a.values[k] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) s += vv[u] * (cc[u] >= 0 ? v[cc[u]] : 0.f);
            kb += U * LPR;
        }
        s = group_sum<LPR>(s);
        if (valid && sub == 0) out[row] = s;
    }
}

// BiCGSTAB of subproblem pid by the whole CTA, the same iteration as the fused single-system solver
// (right preconditioning by default: y = M p, z = M r, omega = (r.t)/(t.t); left: omega from M t),
// with M = D^-1 or the identity; stops on the subproblem's own tolerance.
template <int LPR>
__device__ void solve_one_bicgstab(const BatchArgs& a, int pid, double* red)
{
    const int r0 = a.batch_offsets[pid], r1 = a.batch_offsets[pid + 1];
    const int tid = threadIdx.x, nthr = blockDim.x;
    auto M = [&](int i, float u) { return a.dinv ? a.dinv[i] * u : u; };
    // ---- init: r = b - A x (or b), r0 = p = r, y = M p ----------------------------------------
    if (a.x_is_zero) {
        for (int i = r0 + tid; i < r1; i += nthr) a.x[i] = 0.f;
    } else {
        batch_spmv<LPR>(a, r0, r1, a.x, a.t);
        __syncthreads();
    }
    float part2[2] = {0.f, 0.f};
    for (int i = r0 + tid; i < r1; i += nthr) {
        const float bi = a.b[i];
        const float ri = a.x_is_zero ? bi : bi - a.t[i];
        a.r[i] = ri;
        a.r0[i] = ri;
        a.p[i] = ri;
        a.y[i] = M(i, ri);
        part2[0] += bi * bi;
        part2[1] += ri * ri;
    }
    double tot2[2];
    cta_allreduce<2>(part2, tot2, red);
    const double an = fmax((double)a.rtol * sqrt(tot2[0]), (double)a.atol);
    const double atol_sq = an * an;
    double rr = tot2[1], rho = tot2[1];
    int it = 0;
    bool broke = false;
    while (it < a.maxiter && rr > atol_sq) {
        // ---- v = A y, alpha = rho / (r0.v) ------------------------------------------------------
        batch_spmv<LPR>(a, r0, r1, a.y, a.v);
        __syncthreads();
        float p1[1] = {0.f};
        for (int i = r0 + tid; i < r1; i += nthr) p1[0] += a.r0[i] * a.v[i];
        double r0v[1];
        cta_allreduce<1>(p1, r0v, red);
        const double alpha_d = rho / r0v[0];
        if (!isfinite(alpha_d)) {
            broke = true;
            break;
        }
        const float alpha = (float)alpha_d;
        // ---- x += alpha y, r -= alpha v, z = M r, r.r (a converged half step ends the solve) -------
        float ph[1] = {0.f};
        for (int i = r0 + tid; i < r1; i += nthr) {
            a.x[i] += alpha * a.y[i];
            const float ri = a.r[i] - alpha * a.v[i];
            a.r[i] = ri;
            a.z[i] = M(i, ri);
            ph[0] += ri * ri;
        }
        double rh[1];
        cta_allreduce<1>(ph, rh, red);  // includes the barriers: z is complete for the product below
        if (!(rh[0] > atol_sq)) {
            rr = rh[0];
            ++it;
            break;
        }
        // ---- t = A z, omega = st / tt -------------------------------------------------------------
        batch_spmv<LPR>(a, r0, r1, a.z, a.t);
        __syncthreads();
        float p2[2] = {0.f, 0.f};
        for (int i = r0 + tid; i < r1; i += nthr) {
            const float ti = a.t[i];
            if (a.left_precond) {
                const float mt = M(i, ti);
                p2[0] += a.z[i] * mt;
                p2[1] += mt * mt;
            } else {
                p2[0] += a.r[i] * ti;
                p2[1] += ti * ti;
            }
        }
        double stt[2];
        cta_allreduce<2>(p2, stt, red);
        const double omega_d = stt[0] / stt[1];
        if (!isfinite(omega_d)) {
            broke = true;
            break;
        }
        const float omega = (float)omega_d;
        // ---- x += omega z, r -= omega t, rr, rho = r0.r -------------------------------------------
        float p3[2] = {0.f, 0.f};
        for (int i = r0 + tid; i < r1; i += nthr) {
            a.x[i] += omega * a.z[i];
            const float ri = a.r[i] - omega * a.t[i];
            a.r[i] = ri;
            p3[0] += ri * ri;
            p3[1] += a.r0[i] * ri;
        }
        double t3[2];
        cta_allreduce<2>(p3, t3, red);
        rr = t3[0];
        ++it;
        if (!(rr > atol_sq)) break;
        const double beta_d = t3[1] * stt[1] / (r0v[0] * stt[0]);
        const double bo_d = t3[1] / r0v[0];
        if (!isfinite(beta_d) || !isfinite(bo_d)) {
            broke = true;
            break;
        }
        rho = t3[1];
        const float beta = (float)beta_d, bo = (float)bo_d;
        // ---- p = r + beta p - beta_omega v, y = M p ---------------------------------------------
        for (int i = r0 + tid; i < r1; i += nthr) {
            const float pi = a.r[i] + beta * a.p[i] - bo * a.v[i];
            a.p[i] = pi;
            a.y[i] = M(i, pi);
        }
        __syncthreads();
    }
    if (tid == 0) {
        a.iters[pid] = it;
        a.rr_out[pid] = (float)rr;
        a.atol_sq_out[pid] = (float)atol_sq;
        if (broke) atomicOr(a.status, GB_DEV_BREAKDOWN);
    }
    __syncthreads();
}

template <int LPR>
__global__ void __launch_bounds__(512) k_batched_bicgstab(const BatchArgs a)
{
    __shared__ double red[32 * 3];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= a.nbatch) return;
        solve_one_bicgstab<LPR>(a, a.order[item], red);
    }
}

template <int LPR>
__global__ void __launch_bounds__(512) k_batched_pcg(const BatchArgs a)
{
    extern __shared__ __align__(16) float svec[];  // 3 * smem_rows floats (p, r, Ap) when enabled
    __shared__ double red[32 * 3];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= a.nbatch) return;
        const int pid = a.order[item];
        const int nrows = a.batch_offsets[pid + 1] - a.batch_offsets[pid];
        if (nrows > a.small_rows) {
            if (nrows <= a.smem_rows)
                solve_one<LPR, false, true>(a, pid, threadIdx.x, blockDim.x, red, svec);
            else
                solve_one<LPR, false, false>(a, pid, threadIdx.x, blockDim.x, red, nullptr);
            continue;
        }
        // from here on every subproblem is small (the queue is ordered by size): one warp each
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        int cur = (wid == 0) ? item : -1;
        for (;;) {
            if (cur < 0) {
                int got = 0;
                if (lane == 0) got = atomicAdd(a.queue, 1);
                cur = __shfl_sync(0xffffffffu, got, 0);
            }
            if (cur >= a.nbatch) break;
            solve_one<LPR, true, false>(a, a.order[cur], lane, 32, nullptr, nullptr);
            cur = -1;
        }
        return;
    }
}

// ---- batched Q1 assembly on square 2-D grids -----------------------------------------------------
// Subproblem i: unit square, n_i x n_i cells, (n_i+1)^2 nodes (node x*(n+1)+y), per-cell
// coefficient, nodal source f, zero Dirichlet on the whole boundary by projection (boundary rows
// -> identity, boundary columns of interior rows -> explicit zeros: the structure is kept).  The
// CSR structure of each block is the closed-form 9-point pattern, so no sort is needed.
__device__ __forceinline__ double q1_k(int a, int b) { return a == b ? 1.0 : -1.0; }          // 1-D stiffness * h
__device__ __forceinline__ double q1_m(int a, int b) { return a == b ? 1.0 / 3.0 : 1.0 / 6.0; }  // 1-D mass / h

__global__ void k_q1_batched_2d(int nbatch, const int* __restrict__ ncell, const int* __restrict__ row_off,
                                const int* __restrict__ nnz_off, const int* __restrict__ cell_off,
                                const float* __restrict__ coef, const float* __restrict__ f, int total_rows,
                                int* __restrict__ offsets, int* __restrict__ columns, float* __restrict__ values,
                                float* __restrict__ rhs)
{
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= total_rows) return;
    // subproblem of this row (binary search over row_off)
    int lo = 0, hi = nbatch;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (row_off[mid] <= row) lo = mid; else hi = mid;
    }
    const int pid = lo, n = ncell[pid], m = n + 1, r0 = row_off[pid];
    const int x = (row - r0) / m, y = (row - r0) % m;
    const int S = 3 * m - 2;
    auto cnt = [&](int c) { return 3 - (c == 0) - (c == m - 1); };
    auto before = [&](int c) { return 3 * c - (c > 0 ? 1 : 0); };
    int k = nnz_off[pid] + before(x) * S + before(y) * cnt(x);
    offsets[row] = k;
    if (row == total_rows - 1) offsets[total_rows] = k + cnt(x) * cnt(y);
    const bool bnd = x == 0 || y == 0 || x == m - 1 || y == m - 1;
    const float* a = coef + cell_off[pid];
    const double h = 1.0 / n;
    for (int xx = max(x - 1, 0); xx <= min(x + 1, m - 1); ++xx)
        for (int yy = max(y - 1, 0); yy <= min(y + 1, m - 1); ++yy, ++k) {
            const int col = r0 + xx * m + yy;
            columns[k] = col;
            double v = 0.0;
            const bool cbnd = xx == 0 || yy == 0 || xx == m - 1 || yy == m - 1;
            if (bnd) {
                v = (col == row) ? 1.0 : 0.0;
            } else if (!cbnd) {
                for (int ci = max(max(x, xx) - 1, 0); ci <= min(min(x, xx), n - 1); ++ci)
                    for (int cj = max(max(y, yy) - 1, 0); cj <= min(min(y, yy), n - 1); ++cj) {
                        const int ia = x - ci, ja = y - cj, ib = xx - ci, jb = yy - cj;
                        v += (double)a[ci * n + cj] * (q1_k(ia, ib) * q1_m(ja, jb) + q1_m(ia, ib) * q1_k(ja, jb));
                    }
            }
            values[k] = (float)v;
        }
    // rhs = M f (consistent mass), zero on the boundary
    double s = 0.0;
    if (!bnd) {
        const float* fp = f + r0;
        for (int ci = max(x - 1, 0); ci <= min(x, n - 1); ++ci)
            for (int cj = max(y - 1, 0); cj <= min(y, n - 1); ++cj)
                for (int lb = 0; lb < 4; ++lb) {
                    const int xb = ci + (lb >> 1), yb = cj + (lb & 1);
                    s += h * h * q1_m(x - ci, xb - ci) * q1_m(y - cj, yb - cj) * (double)fp[xb * m + yb];
                }
    }
    rhs[row] = (float)s;
}

}  // namespace gb

using namespace gb;

GB_API size_t gb_batched_pcg_workspace_bytes(int64_t n) { return 3 * sizeof(float) * (size_t)n + 256; }

// Persistent batched Jacobi-CG (see the file comment).  n: total rows (inactive tail included);
// dinv may be null (no preconditioner); x is read as the initial guess unless x_is_zero;
// threads in {128, 256, 512}; lanes_per_row in {1, 2, 4, 8}; small_rows: subproblems of at most
// this many rows are solved by one warp; smem_rows: larger subproblems of at most this many rows keep
// their CG vectors p, r, Ap in shared memory (3 * 4 * smem_rows bytes per CTA; 0 = off).
// iters / rr / atol_sq: per-subproblem results (device).

GB_API int gb_batched_pcg2(int nbatch, const int* batch_offsets, const int* order, int64_t n, const int* offsets,
                           const int* columns, const float* values, const float* dinv, const float* b, float* x,
                           double rtol, double atol, int maxiter, int x_is_zero, int threads, int lanes_per_row,
                           int small_rows, int smem_rows, int grid, int* iters, float* rr, float* atol_sq,
                           void* workspace, size_t workspace_bytes, int* status, cudaStream_t stream)
{
    GB_REQUIRE(smem_rows >= 0 && (size_t)smem_rows * 3 * sizeof(float) <= 200 * 1024,
               "batched_pcg: smem_rows must be in [0, %d]", (int)(200 * 1024 / (3 * sizeof(float))));
    GB_REQUIRE(nbatch >= 0 && n >= 0, "batched_pcg: negative sizes");
    GB_REQUIRE(threads == 128 || threads == 256 || threads == 512, "batched_pcg: threads must be 128, 256 or 512");
    GB_REQUIRE(workspace_bytes >= gb_batched_pcg_workspace_bytes(n), "batched_pcg: workspace too small");
    GB_REQUIRE(status != nullptr && iters != nullptr && rr != nullptr && atol_sq != nullptr,
               "batched_pcg: status and per-subproblem result arrays are required");
    if (nbatch == 0) return GB_OK;
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    BatchArgs a{};
    a.nbatch = nbatch;
    a.batch_offsets = batch_offsets;
    a.order = order;
    a.offsets = offsets;
    a.columns = columns;
    a.values = values;
    a.dinv = dinv;
    a.b = b;
    a.x = x;
    a.queue = reinterpret_cast<int*>(ws);
    a.r = reinterpret_cast<float*>(ws + 256);
    a.p = a.r + n;
    a.Ap = a.p + n;
    a.rtol = (float)rtol;
    a.atol = (float)atol;
    a.maxiter = maxiter;
    a.x_is_zero = x_is_zero;
    a.small_rows = small_rows;
    a.smem_rows = smem_rows;
    a.iters = iters;
    a.rr_out = rr;
    a.atol_sq_out = atol_sq;
    a.status = status;
    void (*kern)(const BatchArgs) = nullptr;
    switch (lanes_per_row) {
    case 1: kern = k_batched_pcg<1>; break;
    case 2: kern = k_batched_pcg<2>; break;
    case 4: kern = k_batched_pcg<4>; break;
    case 8: kern = k_batched_pcg<8>; break;
    default: gb::set_error("batched_pcg: lanes_per_row must be 1, 2, 4 or 8"); return GB_ERR_INVALID;
    }
    const size_t smem = (size_t)smem_rows * 3 * sizeof(float);
    GB_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (grid <= 0) {
        int dev = 0, sms = kSmCount, per_sm = 1;
        GB_CHECK_CUDA(cudaGetDevice(&dev));
        GB_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
        grid = sms * std::max(1, std::min(per_sm, 2048 / threads));
    }
    grid = std::min(grid, nbatch);
    GB_CHECK_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(int), stream));
    kern<<<grid, threads, smem, stream>>>(a);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// The same solve with global-memory work vectors only (smem_rows = 0).
GB_API int gb_batched_pcg(int nbatch, const int* batch_offsets, const int* order, int64_t n, const int* offsets,
                          const int* columns, const float* values, const float* dinv, const float* b, float* x,
                          double rtol, double atol, int maxiter, int x_is_zero, int threads, int lanes_per_row,
                          int small_rows, int grid, int* iters, float* rr, float* atol_sq, void* workspace,
                          size_t workspace_bytes, int* status, cudaStream_t stream)
{
    return gb_batched_pcg2(nbatch, batch_offsets, order, n, offsets, columns, values, dinv, b, x, rtol, atol, maxiter,
                           x_is_zero, threads, lanes_per_row, small_rows, 0, grid, iters, rr, atol_sq, workspace,
                           workspace_bytes, status, stream);
}

GB_API size_t gb_batched_bicgstab_workspace_bytes(int64_t n) { return 8 * sizeof(float) * (size_t)n + 256; }

// Persistent batched BiCGSTAB with the Jacobi (dinv) or no preconditioner: each CTA takes subproblems
// from the queue (order: largest first) and runs one subproblem's BiCGSTAB to its own tolerance
// (reference: BiCGSTAB with batch_offsets, warp/_src/optim/linear.py:1377-1574, per-subproblem
// tolerances :2063-2083).  left_precond selects left preconditioning; threads 128/256/512;
// lanes_per_row 1/2/4/8.
GB_API int gb_batched_bicgstab(int nbatch, const int* batch_offsets, const int* order, int64_t n, const int* offsets,
                               const int* columns, const float* values, const float* dinv, const float* b, float* x,
                               double rtol, double atol, int maxiter, int x_is_zero, int left_precond, int threads,
                               int lanes_per_row, int grid, int* iters, float* rr, float* atol_sq, void* workspace,
                               size_t workspace_bytes, int* status, cudaStream_t stream)
{
    GB_REQUIRE(nbatch >= 0 && n >= 0, "batched_bicgstab: negative sizes");
    GB_REQUIRE(threads == 128 || threads == 256 || threads == 512, "batched_bicgstab: threads must be 128, 256 or 512");
    GB_REQUIRE(workspace_bytes >= gb_batched_bicgstab_workspace_bytes(n), "batched_bicgstab: workspace too small");
    GB_REQUIRE(status != nullptr && iters != nullptr && rr != nullptr && atol_sq != nullptr,
               "batched_bicgstab: status and per-subproblem result arrays are required");
    if (nbatch == 0) return GB_OK;
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    BatchArgs a{};
    a.nbatch = nbatch;
    a.batch_offsets = batch_offsets;
    a.order = order;
    a.offsets = offsets;
    a.columns = columns;
    a.values = values;
    a.dinv = dinv;
    a.b = b;
    a.x = x;
    a.queue = reinterpret_cast<int*>(ws);
    a.r = reinterpret_cast<float*>(ws + 256);
    a.p = a.r + n;
    a.r0 = a.p + n;
    a.v = a.r0 + n;
    a.t = a.v + n;
    a.y = a.t + n;
    a.z = a.y + n;
    a.left_precond = left_precond;
    a.rtol = (float)rtol;
    a.atol = (float)atol;
    a.maxiter = maxiter;
    a.x_is_zero = x_is_zero;
    a.iters = iters;
    a.rr_out = rr;
    a.atol_sq_out = atol_sq;
    a.status = status;
    void (*kern)(const BatchArgs) = nullptr;
    switch (lanes_per_row) {
    case 1: kern = k_batched_bicgstab<1>; break;
    case 2: kern = k_batched_bicgstab<2>; break;
    case 4: kern = k_batched_bicgstab<4>; break;
    case 8: kern = k_batched_bicgstab<8>; break;
    default: gb::set_error("batched_bicgstab: lanes_per_row must be 1, 2, 4 or 8"); return GB_ERR_INVALID;
    }
    if (grid <= 0) {
        int dev = 0, sms = kSmCount, per_sm = 1;
        GB_CHECK_CUDA(cudaGetDevice(&dev));
        GB_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, 0));
        grid = sms * std::max(1, std::min(per_sm, 2048 / threads));
    }
    grid = std::min(grid, nbatch);
    GB_CHECK_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(int), stream));
    kern<<<grid, threads, 0, stream>>>(a);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// Batched 2-D Q1 assembly (see k_q1_batched_2d): ncell[B] cells per side, row_off / nnz_off / cell_off
// [B+1] (rows (n+1)^2, nonzeros (3n+1)^2, cells n^2 per subproblem), coef per cell, f per node.
GB_API int gb_q1_batched_assemble_2d(int nbatch, const int* ncell, const int* row_off, const int* nnz_off,
                                     const int* cell_off, const float* coef, const float* f, int total_rows,
                                     int* offsets, int* columns, float* values, float* rhs, cudaStream_t stream)
{
    GB_REQUIRE(nbatch >= 1 && total_rows >= 1, "q1_batched_assemble_2d: empty batch");
    k_q1_batched_2d<<<ceil_div(total_rows, 256), 256, 0, stream>>>(nbatch, ncell, row_off, nnz_off, cell_off, coef, f,
                                                                   total_rows, offsets, columns, values, rhs);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
