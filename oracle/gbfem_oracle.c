/*
 * gbfem_oracle.c -- CPU ORACLE for the FEM linear-solve path (test infrastructure only).
 *
 * This file is the checker, never the product: only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference leg load it.  Each function restates, in plain
 * C, the algorithm of the Warp reference at the file:line cited beside it (paths relative to
 * the Warp source tree).  Parity is pinned by:
 *   - the structure known-answer tests of warp/tests/test_sparse.py:156-161 and :199-222,
 *   - the compiled reference host function wp_bsr_matrix_from_triplets_host
 *     (warp/native/sparse.cpp:267-413, built into oracle/_ref by oracle/Makefile), compared
 *     against this restatement on seeded inputs and frozen into tests/golden/.
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp -shared).  OpenMP is only used by the timed CPU
 * baseline entry points (orc_*_omp); every parity entry point is single-threaded and
 * deterministic.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------ */
/* Triplets -> BSR topology.                                                                   */
/* Restates wp_bsr_matrix_from_triplets_device (warp/native/sparse.cu:1168-1325):              */
/*   key = (row << 32) | col, or ~0 when the triplet is pruned (sparse.cu:315-336, 234-238);   */
/*   a triplet is pruned when row/col are out of range, when masked and (row,col) is not an    */
/*   existing block (BsrBlockInMask, sparse.cu:271-311), or when every scalar of its block has */
/*   (bits & zero_mask) == 0 (BsrBlockIsNotZero, sparse.cu:245-269);                           */
/*   a STABLE sort of (key, triplet index) (cub::DeviceRadixSort::SortPairs, sparse.cu:1250);  */
/*   run-length encoding of the sorted keys (sparse.cu:1267-1282);                             */
/*   offsets[r] = lower bound of row r among the unique keys (sparse.cu:339-372);              */
/*   columns[b] = col of unique key b (sparse.cu:374-381);                                     */
/*   tpl_block_offsets = inclusive scan of the run lengths (sparse.cu:1305-1317).              */
/* Returns the number of BSR blocks (offsets[nrow]).                                           */
/* ------------------------------------------------------------------------------------------ */

static int orc_block_is_zero(const void* values, int scalar_size, int block_size, int64_t blk, uint64_t mask)
{
    for (int c = 0; c < block_size; ++c) {
        uint64_t bits = 0;
        const unsigned char* p = (const unsigned char*)values + ((size_t)blk * block_size + c) * (size_t)scalar_size;
        switch (scalar_size) {
        case 1: bits = *(const uint8_t*)p; break;
        case 2: { uint16_t v; memcpy(&v, p, 2); bits = v; } break;
        case 4: { uint32_t v; memcpy(&v, p, 4); bits = v; } break;
        case 8: { uint64_t v; memcpy(&v, p, 8); bits = v; } break;
        default: return 0;
        }
        if ((bits & mask) != 0) return 0;
    }
    return 1;
}

static int orc_in_mask(int row, int col, const int* m_offsets, const int* m_row_counts, const int* m_columns)
{
    int lower = m_offsets[row];
    int end = m_row_counts ? m_offsets[row] + m_row_counts[row] : m_offsets[row + 1];
    int upper = end - 1;
    if (upper < lower) return 0;
    while (lower < upper) {
        int mid = lower + (upper - lower) / 2;
        if (m_columns[mid] < col) lower = mid + 1; else upper = mid;
    }
    return m_columns[lower] == col;
}

/* Stable LSD radix sort (8-bit digits) of (key, idx) pairs.  Any stable sort gives the same
 * permutation; radix keeps the oracle linear-time for the large cases. */
static void orc_stable_sort(uint64_t* keys, int* idx, int64_t n)
{
    if (n <= 1) return;
    uint64_t* k2 = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
    int* i2 = (int*)malloc((size_t)n * sizeof(int));
    uint64_t all_or = 0, all_and = ~(uint64_t)0;
    for (int64_t i = 0; i < n; ++i) { all_or |= keys[i]; all_and &= keys[i]; }
    uint64_t varying = all_or ^ all_and;
    uint64_t *ks = keys, *kd = k2;
    int *is = idx, *id = i2;
    for (int shift = 0; shift < 64; shift += 8) {
        if (((varying >> shift) & 0xFF) == 0) continue; /* all keys share this digit */
        int64_t count[257];
        memset(count, 0, sizeof(count));
        for (int64_t i = 0; i < n; ++i) count[((ks[i] >> shift) & 0xFF) + 1]++;
        for (int d = 0; d < 256; ++d) count[d + 1] += count[d];
        for (int64_t i = 0; i < n; ++i) {
            int d = (int)((ks[i] >> shift) & 0xFF);
            int64_t pos = count[d]++;
            kd[pos] = ks[i];
            id[pos] = is[i];
        }
        uint64_t* tk = ks; ks = kd; kd = tk;
        int* ti = is; is = id; id = ti;
    }
    if (ks != keys) {
        memcpy(keys, ks, (size_t)n * sizeof(uint64_t));
        memcpy(idx, is, (size_t)n * sizeof(int));
    }
    free(k2);
    free(i2);
}

int64_t orc_bsr_from_triplets(int block_size, int scalar_size, int nrow, int ncol, int nnz, const int* rows,
                              const int* cols, const void* values, uint64_t zero_mask, int masked,
                              const int* m_offsets, const int* m_row_counts, const int* m_columns,
                              int* tpl_block_offsets, int* tpl_block_indices, int* bsr_offsets, int* bsr_columns)
{
    const uint64_t PRUNED = ~(uint64_t)0;
    uint64_t* keys = (uint64_t*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(uint64_t));
    int do_prune = (values != NULL && zero_mask != 0 && scalar_size > 0);
    for (int i = 0; i < nnz; ++i) {
        int r = rows[i], c = cols[i];
        int keep = !(r < 0 || r >= nrow || c < 0 || c >= ncol);
        if (keep && masked) keep = orc_in_mask(r, c, m_offsets, m_row_counts, m_columns);
        if (keep && do_prune) keep = !orc_block_is_zero(values, scalar_size, block_size, i, zero_mask);
        keys[i] = keep ? (((uint64_t)(uint32_t)r << 32) | (uint32_t)c) : PRUNED;
        tpl_block_indices[i] = i;
    }
    orc_stable_sort(keys, tpl_block_indices, nnz);

    /* unique valid runs */
    int64_t nb = 0;
    int* urow = (int*)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int));
    for (int i = 0; i < nnz; ++i) {
        if (keys[i] == PRUNED) break;
        if (i == 0 || keys[i] != keys[i - 1]) {
            bsr_columns[nb] = (int)(keys[i] & 0x7FFFFFFF);
            urow[nb] = (int)(keys[i] >> 32);
            ++nb;
        }
        tpl_block_offsets[nb - 1] = i + 1; /* inclusive end of the current run */
    }
    /* offsets[r] = lower bound of row r among the unique keys */
    int64_t u = 0;
    for (int r = 0; r <= nrow; ++r) {
        while (u < nb && urow[u] < r) ++u;
        bsr_offsets[r] = (int)u;
    }
    free(urow);
    free(keys);
    return nb;
}

/* Value accumulation: restates _bsr_accumulate_triplet_value (warp/_src/sparse.py:1122-1141):
 * val = v[idx[beg]]; for k in beg+1..end: val += v[idx[k]], in the matrix scalar type (fp32). */
void orc_bsr_accumulate_f32(int block_size, int64_t nnzb, const int* tpl_block_offsets,
                            const int* tpl_block_indices, const float* tpl_values, float* out_values)
{
    for (int64_t b = 0; b < nnzb; ++b) {
        int beg = (b == 0) ? 0 : tpl_block_offsets[b - 1];
        int end = tpl_block_offsets[b];
        for (int s = 0; s < block_size; ++s) {
            float v = tpl_values[(size_t)tpl_block_indices[beg] * block_size + s];
            for (int k = beg + 1; k < end; ++k) v += tpl_values[(size_t)tpl_block_indices[k] * block_size + s];
            out_values[(size_t)b * block_size + s] = v;
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* SpMV.  Restates bsr_mv_kernel (warp/_src/sparse.py:4627-4665): per scalar row,              */
/*   v = sum_blocks sum_c A[b,sub,c] * x[col*bc+c]; v *= alpha; v += beta * y; in fp32.       */
/* ------------------------------------------------------------------------------------------ */
void orc_bsr_mv_f32(int br, int bc, int nrow, const int* offsets, const int* row_counts, const int* columns,
                    const float* values, const float* x, float* y, float alpha, float beta)
{
    for (int row = 0; row < nrow; ++row) {
        int beg = offsets[row];
        int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
        for (int sub = 0; sub < br; ++sub) {
            float v = 0.0f;
            if (alpha != 0.0f) {
                for (int blk = beg; blk < end; ++blk) {
                    int xs = columns[blk] * bc;
                    for (int c = 0; c < bc; ++c) v += values[((size_t)blk * br + sub) * bc + c] * x[xs + c];
                }
                v *= alpha;
            }
            size_t yi = (size_t)row * br + sub;
            if (beta != 0.0f) v += beta * y[yi];
            y[yi] = v;
        }
    }
}

/* Same product evaluated in fp64 from fp32 matrix values (the exact reference the fp32 kernels are
 * bounded against, and the FP64 true residual r = b - A x of the refinement loop). */
void orc_bsr_mv_f64(int br, int bc, int nrow, const int* offsets, const int* row_counts, const int* columns,
                    const float* values, const double* x, double* y, double alpha, double beta)
{
    for (int row = 0; row < nrow; ++row) {
        int beg = offsets[row];
        int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
        for (int sub = 0; sub < br; ++sub) {
            double v = 0.0;
            for (int blk = beg; blk < end; ++blk) {
                int xs = columns[blk] * bc;
                for (int c = 0; c < bc; ++c) v += (double)values[((size_t)blk * br + sub) * bc + c] * x[xs + c];
            }
            size_t yi = (size_t)row * br + sub;
            y[yi] = alpha * v + (beta != 0.0 ? beta * y[yi] : 0.0);
        }
    }
}

/* Row-wise sum_j |A_ij x_j| in fp64: the scale that bounds fp32 rounding of a row product. */
void orc_bsr_abs_mv_f64(int br, int bc, int nrow, const int* offsets, const int* row_counts, const int* columns,
                        const float* values, const double* x, double* y)
{
    for (int row = 0; row < nrow; ++row) {
        int beg = offsets[row];
        int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
        for (int sub = 0; sub < br; ++sub) {
            double v = 0.0;
            for (int blk = beg; blk < end; ++blk) {
                int xs = columns[blk] * bc;
                for (int c = 0; c < bc; ++c) v += fabs((double)values[((size_t)blk * br + sub) * bc + c] * x[xs + c]);
            }
            y[(size_t)row * br + sub] = v;
        }
    }
}

/* Jacobi diagonal: restates bsr_get_diag (warp/_src/sparse.py:2871-2887) and
 * _inverse_diag_coefficient (warp/_src/optim/linear.py:2290-2329): for each block row the
 * diagonal entries of the diagonal block; inv = 1/d, or 1 when d == 0. */
void orc_inverse_diagonal_f32(int bs, int nrow, const int* offsets, const int* row_counts, const int* columns,
                              const float* values, float* inv_diag)
{
    for (int row = 0; row < nrow; ++row) {
        int beg = offsets[row];
        int end = row_counts ? beg + row_counts[row] : offsets[row + 1];
        for (int k = 0; k < bs; ++k) inv_diag[(size_t)row * bs + k] = 1.0f;
        for (int blk = beg; blk < end; ++blk) {
            if (columns[blk] == row) {
                for (int k = 0; k < bs; ++k) {
                    float d = values[((size_t)blk * bs + k) * bs + k];
                    inv_diag[(size_t)row * bs + k] = (d == 0.0f) ? 1.0f : 1.0f / d;
                }
                break;
            }
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Preconditioned CG, restating CG._run (warp/_src/optim/linear.py:934-1032) with the kernels  */
/* _cg_kernel_1/_cg_kernel_2 (:2332-2373), the tolerance rule of _get_tolerances (:2010-2032) */
/* and the loop/condition of _run_capturable_loop / _update_condition (:2086-2179):           */
/*   atol_sq = max(rtol*|b|, atol)^2; r = b - A x; z = M r; p = z;                             */
/*   iterate: Ap = A p; alpha = (rr > atol_sq) ? rz/pAp : 0; x += alpha p; r -= alpha Ap;      */
/*            z = M r; rr = r.r; rz_new = r.z; beta = (rr > atol_sq) ? rz_new/rz : 0;          */
/*            p = z + beta p; stop when rr <= atol_sq or iter >= maxiter.                      */
/* The arithmetic type is fp32 for vectors with dot products accumulated in fp64 (the         */
/* reference's tile reduction order is not reproducible on a CPU; fp64 accumulation bounds it).*/
/* inv_diag == NULL means no preconditioner.  Returns the iteration count; writes rr, atol_sq. */
/* nthreads > 1 uses OpenMP (CPU baseline timing only).                                        */
/* ------------------------------------------------------------------------------------------ */
static void orc_spmv_plain(int br, int bc, int nrow, const int* offsets, const int* columns, const float* values,
                           const float* x, float* y, int nthreads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
    for (int row = 0; row < nrow; ++row) {
        int beg = offsets[row], end = offsets[row + 1];
        for (int sub = 0; sub < br; ++sub) {
            float v = 0.0f;
            for (int blk = beg; blk < end; ++blk) {
                int xs = columns[blk] * bc;
                for (int c = 0; c < bc; ++c) v += values[((size_t)blk * br + sub) * bc + c] * x[xs + c];
            }
            y[(size_t)row * br + sub] = v;
        }
    }
    (void)nthreads;
}

static double orc_dot(const float* a, const float* b, int64_t n, int nthreads)
{
    double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(nthreads) if (nthreads > 1)
#endif
    for (int64_t i = 0; i < n; ++i) s += (double)a[i] * (double)b[i];
    (void)nthreads;
    return s;
}

int orc_pcg_f32(int br, int bc, int nrow, const int* offsets, const int* columns, const float* values,
                const float* inv_diag, const float* b, float* x, double tol, double atol, int maxiter, int nthreads,
                double* out_rr, double* out_atol_sq)
{
    int64_t n = (int64_t)nrow * br;
    float* r = (float*)malloc((size_t)n * sizeof(float));
    float* z = (float*)malloc((size_t)n * sizeof(float));
    float* p = (float*)malloc((size_t)n * sizeof(float));
    float* Ap = (float*)malloc((size_t)n * sizeof(float));

    double bb = orc_dot(b, b, n, nthreads);
    double a = fmax(tol * sqrt(bb), atol);
    double atol_sq = a * a;

    orc_spmv_plain(br, bc, nrow, offsets, columns, values, x, Ap, nthreads);
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - Ap[i];
    for (int64_t i = 0; i < n; ++i) z[i] = inv_diag ? inv_diag[i] * r[i] : r[i];
    double rr = orc_dot(r, r, n, nthreads);
    double rz = orc_dot(r, z, n, nthreads);
    memcpy(p, z, (size_t)n * sizeof(float));

    int iter = 0;
    while (!(rr <= atol_sq) && iter < maxiter) {
        orc_spmv_plain(br, bc, nrow, offsets, columns, values, p, Ap, nthreads);
        double pAp = orc_dot(p, Ap, n, nthreads);
        float alpha = (rr > atol_sq) ? (float)(rz / pAp) : 0.0f;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
        for (int64_t i = 0; i < n; ++i) {
            x[i] = x[i] + alpha * p[i];
            r[i] = r[i] - alpha * Ap[i];
            z[i] = inv_diag ? inv_diag[i] * r[i] : r[i];
        }
        double rz_new = orc_dot(r, z, n, nthreads);
        rr = orc_dot(r, r, n, nthreads);
        float beta = (rr > atol_sq) ? (float)(rz_new / rz) : 0.0f;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz = rz_new;
        ++iter;
    }
    if (out_rr) *out_rr = rr;
    if (out_atol_sq) *out_atol_sq = atol_sq;
    free(r); free(z); free(p); free(Ap);
    return iter;
}

/* Right-preconditioned BiCGSTAB, restating BiCGSTAB._run (warp/_src/optim/linear.py:1466-1574)
 * with _bicgstab_kernel_1/2/3 (:2426-2493):
 *   r = b - A x; rr = r.r; p = r; r0 = r; rho = rr;
 *   iterate: y = M p; v = A y; r0v = r0.v; alpha = rho/r0v; x += alpha y; r -= alpha v; rr = r.r;
 *            z = M r; t = A z; st = r.t; tt = t.t; omega = st/tt; x += omega z; r -= omega t;
 *            rr = r.r; rho = r0.r; beta = rho*tt/(r0v*st); beta_omega = rho/r0v;
 *            p = r + beta p - beta_omega v.   (all updates masked once rr <= atol_sq) */
int orc_bicgstab_f32(int br, int bc, int nrow, const int* offsets, const int* columns, const float* values,
                     const float* inv_diag, const float* b, float* x, double tol, double atol, int maxiter,
                     double* out_rr, double* out_atol_sq)
{
    int64_t n = (int64_t)nrow * br;
    float *r = malloc(n * sizeof(float)), *r0 = malloc(n * sizeof(float)), *p = malloc(n * sizeof(float));
    float *v = malloc(n * sizeof(float)), *t = malloc(n * sizeof(float)), *y = malloc(n * sizeof(float));
    float *z = malloc(n * sizeof(float));
    double bb = orc_dot(b, b, n, 1);
    double a = fmax(tol * sqrt(bb), atol);
    double atol_sq = a * a;
    orc_spmv_plain(br, bc, nrow, offsets, columns, values, x, v, 1);
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - v[i];
    double rr = orc_dot(r, r, n, 1);
    memcpy(p, r, n * sizeof(float));
    memcpy(r0, r, n * sizeof(float));
    double rho = rr;
    int iter = 0;
    while (!(rr <= atol_sq) && iter < maxiter) {
        int active = rr > atol_sq;
        for (int64_t i = 0; i < n; ++i) y[i] = inv_diag ? inv_diag[i] * p[i] : p[i];
        orc_spmv_plain(br, bc, nrow, offsets, columns, values, y, v, 1);
        double r0v = orc_dot(r0, v, n, 1);
        float alpha = active ? (float)(rho / r0v) : 0.0f;
        for (int64_t i = 0; i < n; ++i) { x[i] += alpha * y[i]; r[i] -= alpha * v[i]; }
        rr = orc_dot(r, r, n, 1);
        active = rr > atol_sq;
        for (int64_t i = 0; i < n; ++i) z[i] = inv_diag ? inv_diag[i] * r[i] : r[i];
        orc_spmv_plain(br, bc, nrow, offsets, columns, values, z, t, 1);
        double st = orc_dot(r, t, n, 1), tt = orc_dot(t, t, n, 1);
        float omega = active ? (float)(st / tt) : 0.0f;
        for (int64_t i = 0; i < n; ++i) { x[i] += omega * z[i]; r[i] -= omega * t[i]; }
        rr = orc_dot(r, r, n, 1);
        rho = orc_dot(r0, r, n, 1);
        active = rr > atol_sq;
        float beta = active ? (float)(rho * tt / (r0v * st)) : 0.0f;
        float beta_omega = active ? (float)(rho / r0v) : 0.0f;
        for (int64_t i = 0; i < n; ++i) p[i] = r[i] + beta * p[i] - beta_omega * v[i];
        ++iter;
    }
    if (out_rr) *out_rr = rr;
    if (out_atol_sq) *out_atol_sq = atol_sq;
    free(r); free(r0); free(p); free(v); free(t); free(y); free(z);
    return iter;
}

/* Same PCG with FP64 vectors and fp32 matrix values (the CPU baseline of the FP64-accurate solve:
 * convergence on the FP64 residual to tol * |b|).  nthreads > 1 uses OpenMP.  Returns iterations. */
static void orc_spmv_d(int br, int bc, int nrow, const int* offsets, const int* columns, const float* values,
                       const double* x, double* y, int nthreads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
    for (int row = 0; row < nrow; ++row) {
        int beg = offsets[row], end = offsets[row + 1];
        for (int sub = 0; sub < br; ++sub) {
            double v = 0.0;
            for (int blk = beg; blk < end; ++blk) {
                int xs = columns[blk] * bc;
                for (int c = 0; c < bc; ++c) v += (double)values[((size_t)blk * br + sub) * bc + c] * x[xs + c];
            }
            y[(size_t)row * br + sub] = v;
        }
    }
    (void)nthreads;
}

static double orc_dot_d(const double* a, const double* b, int64_t n, int nthreads)
{
    double s = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(+ : s) num_threads(nthreads) if (nthreads > 1)
#endif
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    (void)nthreads;
    return s;
}

int orc_pcg_f64(int br, int bc, int nrow, const int* offsets, const int* columns, const float* values,
                const float* inv_diag, const float* b32, double* x, double tol, int maxiter, int nthreads,
                double* out_rel)
{
    int64_t n = (int64_t)nrow * br;
    double *b = malloc(n * sizeof(double)), *r = malloc(n * sizeof(double)), *z = malloc(n * sizeof(double));
    double *p = malloc(n * sizeof(double)), *Ap = malloc(n * sizeof(double));
    for (int64_t i = 0; i < n; ++i) b[i] = b32[i];
    double bnorm = sqrt(orc_dot_d(b, b, n, nthreads));
    double atol_sq = tol * bnorm * tol * bnorm;
    orc_spmv_d(br, bc, nrow, offsets, columns, values, x, Ap, nthreads);
    for (int64_t i = 0; i < n; ++i) {
        r[i] = b[i] - Ap[i];
        z[i] = inv_diag ? inv_diag[i] * r[i] : r[i];
        p[i] = z[i];
    }
    double rr = orc_dot_d(r, r, n, nthreads), rz = orc_dot_d(r, z, n, nthreads);
    int iter = 0;
    while (rr > atol_sq && iter < maxiter) {
        orc_spmv_d(br, bc, nrow, offsets, columns, values, p, Ap, nthreads);
        double alpha = rz / orc_dot_d(p, Ap, n, nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * Ap[i];
            z[i] = inv_diag ? inv_diag[i] * r[i] : r[i];
        }
        double rz_new = orc_dot_d(r, z, n, nthreads);
        rr = orc_dot_d(r, r, n, nthreads);
        double beta = rz_new / rz;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rz = rz_new;
        ++iter;
    }
    if (out_rel) *out_rel = bnorm > 0 ? sqrt(rr) / bnorm : 0.0;
    free(b); free(r); free(z); free(p); free(Ap);
    return iter;
}

/* Timed CPU baseline: `iters` Jacobi-PCG iterations (SpMV + dots + updates) on all threads.
 * Returns wall seconds (CLOCK_MONOTONIC). */
static double orc_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

double orc_pcg_sample_seconds(int br, int bc, int nrow, const int* offsets, const int* columns, const float* values,
                              const float* inv_diag, const float* b, float* x, int iters, int nthreads)
{
    double rr, atol_sq;
    double t0 = orc_now();
    orc_pcg_f32(br, bc, nrow, offsets, columns, values, inv_diag, b, x, 0.0, 0.0, iters, nthreads, &rr, &atol_sq);
    return orc_now() - t0;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
