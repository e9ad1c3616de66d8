// gb_krylov.cu -- fused Jacobi-preconditioned CG and BiCGSTAB for BSR systems, captured as CUDA
// graphs with a device-side conditional while loop, plus the FP64 iterative-refinement helpers.
//
// Replaces, for BSR operators with the Jacobi ("diag") preconditioner or none:
//   CG._run          warp/_src/optim/linear.py:934-1032  (kernels _cg_kernel_1/2 :2332-2373)
//   BiCGSTAB._run    warp/_src/optim/linear.py:1466-1574 (kernels _bicgstab_kernel_1/2/3 :2426-2493)
//   TiledDot         warp/_src/optim/linear.py:309-576   (multi-level tree reductions)
//   _run_capturable_loop / _update_condition / capture_while  linear.py:2086-2179
// Per CG iteration the reference launches SpMV + ~5 vector kernels + 2 multi-level dot trees.
// Here one iteration is three kernels: (1) SpMV Ap = A p fused with p.Ap, (2) x/r update fused
// with z = D^-1 r and the r.r / r.z reductions, (3) p = z + beta p.  Each reduction is a single
// pass: CTAs publish partials and the last CTA to finish sums them in a fixed order (so results
// are deterministic) and computes the next scalar (alpha, beta, the loop condition).  Nothing
// spins: there is no inter-CTA waiting anywhere in the solve.
//
// Solver scalars live in device memory; the loop condition is evaluated on the device and drives
// a cudaGraphCondTypeWhile node, so a whole solve is one graph launch with no host round trip.
// Kernels read the operand pointers through a small device-side argument block so one captured
// graph serves every right-hand side / solution vector / matrix with the same shape.
#include "gb_common.cuh"
#include "gb_spmv.cuh"

#include <new>

namespace gb {

enum KrylovKind : int { KRYLOV_CG = 0, KRYLOV_BICGSTAB = 1, KRYLOV_FCG = 2 };

// Preconditioner callback of the flexible solver: enqueue z = M(r) on `stream` (called while a
// graph is being captured, or eagerly); returns 0 on success.
typedef int (*gb_precond_fn)(void* user, cudaStream_t stream, const float* r, float* z);

struct KrylovScalars {
    double bb, atol_sq, rr, rz, pAp, alpha, beta;
    double rho, r0v, st, tt, omega, beta_omega;
    double rr_ref;  // residual^2 at the start of the current stagnation window
    int iter, cond, maxiter, status;
    unsigned int counters[8];
};

struct SolveArgs {
    const int* offsets;
    const int* row_counts;
    const int* columns;
    const void* values;
    const float* dinv;  // inverse diagonal (scalar per dof) or null for no preconditioner
    const float* b;
    float* x;
    // work vectors
    float *r, *p, *Ap, *z, *r0, *v, *t, *y;
    double* partials;
    KrylovScalars* S;
    double tol, atol;
    int maxiter;
    int x_is_zero;
    int left_precond;
    int stag_window;     // > 0: every stag_window iterations require rr <= stag_factor^2 * rr_ref
    double stag_factor;  // (flexible solver; a failure sets GB_DEV_STAGNATION and stops the loop)
    int64_t n;  // scalar dofs
};

constexpr int VEC_THREADS = 256;

__device__ __forceinline__ void set_cond(KrylovScalars* S, int cond, cudaGraphConditionalHandle h, int has_cond)
{
    S->cond = cond;
    if (has_cond) cudaGraphSetConditional(h, cond ? 1u : 0u);
}

__device__ __forceinline__ bool finite(double v) { return isfinite(v); }

// ---------------------------------------------------------------------------------------------
// CG
// ---------------------------------------------------------------------------------------------
template <int BR, typename AT> struct EpiCgInit {
    const float *b, *dinv;
    float *r, *p;
    AT sign;  // r = b - A x  (sign = -1) or r = b when x is zero (sign = 0)
    float bb = 0.f, rr = 0.f, rz = 0.f;
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float bi = b[i];
            const float ri = bi + sign * pick<BR>(acc, lane_g);
            const float zi = dinv ? dinv[i] * ri : ri;
            r[i] = ri;
            p[i] = zi;
            bb += bi * bi;
            rr += ri * ri;
            rz += ri * zi;
        }
    }
};

__device__ __forceinline__ void cg_init_finish(const SolveArgs& a, const double (&t)[3],
                                               cudaGraphConditionalHandle h, int has_cond)
{
    KrylovScalars* S = a.S;
    const double bnorm = sqrt(t[0]);
    const double at = fmax(a.tol * bnorm, a.atol);
    S->bb = t[0];
    S->atol_sq = at * at;
    S->rr = t[1];
    S->rz = t[2];
    S->iter = 0;
    S->maxiter = a.maxiter;
    S->alpha = S->beta = 0.0;
    S->rr_ref = t[1];
    int cond = (t[1] > S->atol_sq) && (a.maxiter > 0);
    if (!finite(t[1])) {
        S->status |= GB_DEV_NONFINITE;
        cond = 0;
    }
    set_cond(S, cond, h, has_cond);
}

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_cg_init(const SolveArgs* __restrict__ args, int nrow, SpmvShape sh,
                                                          cudaGraphConditionalHandle h, int has_cond)
{
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[32 * 3];
    const SolveArgs a = *args;
    EpiCgInit<BR, float> epi{a.b, a.dinv, a.r, a.p, -1.0f};
    if (a.x_is_zero) {
        rows_run<BR, float>(nrow, sh, epi);  // r = b: no product needed
    } else {
        spmv_run<BR, BR, VT, float, float>(nrow, sh, a.offsets, a.row_counts, a.columns, (const VT*)a.values, a.x,
                                           smem, &a.S->status, epi);
    }
    float v[3] = {epi.bb, epi.rr, epi.rz};
    grid_reduce<3>(v, a.partials, &a.S->counters[0], s_red,
                   [&](const double (&t)[3]) { cg_init_finish(a, t, h, has_cond); });
}

template <int BR, typename AT> struct EpiCgAp {
    float* Ap;
    const float* p;
    float pAp = 0.f;
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float ap = pick<BR>(acc, lane_g);
            Ap[i] = ap;
            pAp += p[i] * ap;
        }
    }
};

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_cg_spmv(const SolveArgs* __restrict__ args, int nrow, SpmvShape sh)
{
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[32];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    EpiCgAp<BR, float> epi{a.Ap, a.p};
    spmv_run<BR, BR, VT, float, float>(nrow, sh, a.offsets, a.row_counts, a.columns, (const VT*)a.values, a.p, smem,
                                        &S->status, epi);
    float v[1] = {epi.pAp};
    grid_reduce<1>(v, a.partials, &S->counters[1], s_red, [&](const double (&t)[1]) {
        S->pAp = t[0];
        double alpha = 0.0;
        if (S->rr > S->atol_sq) {
            alpha = S->rz / t[0];
            if (!finite(alpha)) {
                S->status |= GB_DEV_BREAKDOWN;
                alpha = 0.0;
            }
        }
        S->alpha = alpha;
    });
}

// x += alpha p; r -= alpha Ap; z = D^-1 r; reductions r.r, r.z; then beta and the loop condition.
__global__ __launch_bounds__(VEC_THREADS) void k_cg_update(const SolveArgs* __restrict__ args,
                                                           cudaGraphConditionalHandle h, int has_cond)
{
    pdl_enter();
    __shared__ double s_red[32 * 2];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float alpha = (float)S->alpha;
    const int64_t n = a.n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float rr = 0.f, rz = 0.f;
    const bool vec4 = ((((uintptr_t)a.x | (uintptr_t)a.r | (uintptr_t)a.p | (uintptr_t)a.Ap |
                         (uintptr_t)(a.dinv ? a.dinv : a.r)) & 15) == 0);
    int64_t done = 0;
    if (vec4) {
        const int64_t n4 = n >> 2;
        float4* x4 = reinterpret_cast<float4*>(a.x);
        float4* r4 = reinterpret_cast<float4*>(a.r);
        const float4* p4 = reinterpret_cast<const float4*>(a.p);
        const float4* ap4 = reinterpret_cast<const float4*>(a.Ap);
        const float4* d4 = reinterpret_cast<const float4*>(a.dinv);
        for (int64_t i = tid; i < n4; i += stride) {
            float4 xv = x4[i], rv = r4[i];
            const float4 pv = p4[i], av = ap4[i];
            xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
            rv.x -= alpha * av.x; rv.y -= alpha * av.y; rv.z -= alpha * av.z; rv.w -= alpha * av.w;
            float4 zv = rv;
            if (d4) {
                const float4 dv = d4[i];
                zv.x *= dv.x; zv.y *= dv.y; zv.z *= dv.z; zv.w *= dv.w;
            }
            x4[i] = xv;
            r4[i] = rv;
            rr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
            rz += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
        }
        done = n4 << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) {
        const float xi = a.x[i] + alpha * a.p[i];
        const float ri = a.r[i] - alpha * a.Ap[i];
        const float zi = a.dinv ? a.dinv[i] * ri : ri;
        a.x[i] = xi;
        a.r[i] = ri;
        rr += ri * ri;
        rz += ri * zi;
    }
    float v[2] = {rr, rz};
    grid_reduce<2>(v, a.partials, &S->counters[2], s_red, [&](const double (&t)[2]) {
        const double rz_old = S->rz;
        S->rr = t[0];
        S->rz = t[1];
        double beta = 0.0;
        if (t[0] > S->atol_sq) {
            beta = t[1] / rz_old;
            if (!finite(beta)) {
                S->status |= GB_DEV_BREAKDOWN;
                beta = 0.0;
            }
        }
        S->beta = beta;
        S->iter += 1;
        int cond = (t[0] > S->atol_sq) && (S->iter < S->maxiter);
        if (!finite(t[0])) {
            S->status |= GB_DEV_NONFINITE;
            cond = 0;
        }
        if (a.stag_window > 0 && cond && (S->iter % a.stag_window) == 0) {
            if (S->iter > a.stag_window && t[0] > a.stag_factor * a.stag_factor * S->rr_ref) {
                S->status |= GB_DEV_STAGNATION;
                cond = 0;
            }
            S->rr_ref = t[0];
        }
        set_cond(S, cond, h, has_cond);
    });
}

// p = D^-1 r + beta p
__global__ __launch_bounds__(VEC_THREADS) void k_cg_pupdate(const SolveArgs* __restrict__ args)
{
    pdl_enter();
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float beta = (float)S->beta;
    const int64_t n = a.n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool vec4 = ((((uintptr_t)a.r | (uintptr_t)a.p | (uintptr_t)(a.dinv ? a.dinv : a.r)) & 15) == 0);
    int64_t done = 0;
    if (vec4) {
        const int64_t n4 = n >> 2;
        const float4* r4 = reinterpret_cast<const float4*>(a.r);
        float4* p4 = reinterpret_cast<float4*>(a.p);
        const float4* d4 = reinterpret_cast<const float4*>(a.dinv);
        for (int64_t i = tid; i < n4; i += stride) {
            float4 zv = r4[i];
            if (d4) {
                const float4 dv = d4[i];
                zv.x *= dv.x; zv.y *= dv.y; zv.z *= dv.z; zv.w *= dv.w;
            }
            float4 pv = p4[i];
            pv.x = zv.x + beta * pv.x; pv.y = zv.y + beta * pv.y; pv.z = zv.z + beta * pv.z; pv.w = zv.w + beta * pv.w;
            p4[i] = pv;
        }
        done = n4 << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) {
        const float zi = a.dinv ? a.dinv[i] * a.r[i] : a.r[i];
        a.p[i] = zi + beta * a.p[i];
    }
}

// ---------------------------------------------------------------------------------------------
// BiCGSTAB (right preconditioning by default, left with left_precond; M = D^-1 or identity)
// ---------------------------------------------------------------------------------------------
template <int BR, typename AT> struct EpiBiInit {
    const float *b, *dinv;
    float *r, *r0, *p, *y;
    AT sign;
    float bb = 0.f, rr = 0.f;
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float bi = b[i];
            const float ri = bi + sign * pick<BR>(acc, lane_g);
            r[i] = ri;
            r0[i] = ri;
            p[i] = ri;
            y[i] = dinv ? dinv[i] * ri : ri;
            bb += bi * bi;
            rr += ri * ri;
        }
    }
};

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_bi_init(const SolveArgs* __restrict__ args, int nrow, SpmvShape sh,
                                                          cudaGraphConditionalHandle h, int has_cond)
{
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[32 * 2];
    const SolveArgs a = *args;
    EpiBiInit<BR, float> epi{a.b, a.dinv, a.r, a.r0, a.p, a.y, -1.0f};
    if (a.x_is_zero) {
        rows_run<BR, float>(nrow, sh, epi);
    } else {
        spmv_run<BR, BR, VT, float, float>(nrow, sh, a.offsets, a.row_counts, a.columns, (const VT*)a.values, a.x,
                                           smem, &a.S->status, epi);
    }
    float v[2] = {epi.bb, epi.rr};
    grid_reduce<2>(v, a.partials, &a.S->counters[0], s_red, [&](const double (&t)[2]) {
        KrylovScalars* S = a.S;
        const double at = fmax(a.tol * sqrt(t[0]), a.atol);
        S->bb = t[0];
        S->atol_sq = at * at;
        S->rr = t[1];
        S->rho = t[1];
        S->iter = 0;
        S->maxiter = a.maxiter;
        int cond = (t[1] > S->atol_sq) && (a.maxiter > 0);
        if (!finite(t[1])) {
            S->status |= GB_DEV_NONFINITE;
            cond = 0;
        }
        set_cond(S, cond, h, has_cond);
    });
}

// v = A y ; r0.v -> alpha
template <int BR, typename AT> struct EpiBiV {
    float* v;
    const float* r0;
    float r0v = 0.f;
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float vi = pick<BR>(acc, lane_g);
            v[i] = vi;
            r0v += r0[i] * vi;
        }
    }
};

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_bi_spmv_v(const SolveArgs* __restrict__ args, int nrow,
                                                            SpmvShape sh)
{
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[32];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    EpiBiV<BR, float> epi{a.v, a.r0};
    spmv_run<BR, BR, VT, float, float>(nrow, sh, a.offsets, a.row_counts, a.columns, (const VT*)a.values, a.y, smem,
                                        &S->status, epi);
    float v[1] = {epi.r0v};
    grid_reduce<1>(v, a.partials, &S->counters[1], s_red, [&](const double (&t)[1]) {
        S->r0v = t[0];
        double alpha = 0.0;
        if (S->rr > S->atol_sq) {
            alpha = S->rho / t[0];
            if (!finite(alpha)) {
                S->status |= GB_DEV_BREAKDOWN;
                alpha = 0.0;
            }
        }
        S->alpha = alpha;
    });
}

// x += alpha y; r -= alpha v; z = M r; rr
__global__ __launch_bounds__(VEC_THREADS) void k_bi_update1(const SolveArgs* __restrict__ args)
{
    pdl_enter();
    __shared__ double s_red[32];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float alpha = (float)S->alpha;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    float rr = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        a.x[i] += alpha * a.y[i];
        const float ri = a.r[i] - alpha * a.v[i];
        a.r[i] = ri;
        a.z[i] = a.dinv ? a.dinv[i] * ri : ri;
        rr += ri * ri;
    }
    float v[1] = {rr};
    grid_reduce<1>(v, a.partials, &S->counters[2], s_red, [&](const double (&t)[1]) { S->rr = t[0]; });
}

// t = A z ; st, tt (right: r.t, t.t ; left: z.Mt, Mt.Mt) -> omega
template <int BR, typename AT> struct EpiBiT {
    float* t;
    const float *r, *z, *dinv;
    int left;
    float st = 0.f, tt = 0.f;
    __device__ __forceinline__ void operator()(int row, const AT (&acc)[BR], int lane_g)
    {
        if (lane_g < BR) {
            const size_t i = (size_t)row * BR + lane_g;
            const float ti = pick<BR>(acc, lane_g);
            t[i] = ti;
            if (left) {
                const float mt = dinv ? dinv[i] * ti : ti;
                st += z[i] * mt;
                tt += mt * mt;
            } else {
                st += r[i] * ti;
                tt += ti * ti;
            }
        }
    }
};

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS) void k_bi_spmv_t(const SolveArgs* __restrict__ args, int nrow,
                                                            SpmvShape sh)
{
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[32 * 2];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    EpiBiT<BR, float> epi{a.t, a.r, a.z, a.dinv, a.left_precond};
    spmv_run<BR, BR, VT, float, float>(nrow, sh, a.offsets, a.row_counts, a.columns, (const VT*)a.values, a.z, smem,
                                        &S->status, epi);
    float v[2] = {epi.st, epi.tt};
    grid_reduce<2>(v, a.partials, &S->counters[3], s_red, [&](const double (&t)[2]) {
        S->st = t[0];
        S->tt = t[1];
        double omega = 0.0;
        if (S->rr > S->atol_sq) {
            omega = t[0] / t[1];
            if (!finite(omega)) {
                S->status |= GB_DEV_BREAKDOWN;
                omega = 0.0;
            }
        }
        S->omega = omega;
    });
}

// x += omega z; r -= omega t; rr, rho = r0.r -> beta, beta*omega, condition
__global__ __launch_bounds__(VEC_THREADS) void k_bi_update2(const SolveArgs* __restrict__ args,
                                                            cudaGraphConditionalHandle h, int has_cond)
{
    pdl_enter();
    __shared__ double s_red[32 * 2];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float omega = (float)S->omega;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    float rr = 0.f, rho = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        a.x[i] += omega * a.z[i];
        const float ri = a.r[i] - omega * a.t[i];
        a.r[i] = ri;
        rr += ri * ri;
        rho += a.r0[i] * ri;
    }
    float v[2] = {rr, rho};
    grid_reduce<2>(v, a.partials, &S->counters[4], s_red, [&](const double (&t)[2]) {
        S->rr = t[0];
        const bool active = t[0] > S->atol_sq;
        double beta = 0.0, beta_omega = 0.0;
        if (active) {
            beta = t[1] * S->tt / (S->r0v * S->st);
            beta_omega = t[1] / S->r0v;
            if (!finite(beta) || !finite(beta_omega)) {
                S->status |= GB_DEV_BREAKDOWN;
                beta = beta_omega = 0.0;
            }
        }
        S->rho = t[1];
        S->beta = beta;
        S->beta_omega = beta_omega;
        S->iter += 1;
        int cond = active && (S->iter < S->maxiter);
        if (!finite(t[0])) {
            S->status |= GB_DEV_NONFINITE;
            cond = 0;
        }
        set_cond(S, cond, h, has_cond);
    });
}

// p = r + beta p - beta_omega v ; y = M p
__global__ __launch_bounds__(VEC_THREADS) void k_bi_pupdate(const SolveArgs* __restrict__ args)
{
    pdl_enter();
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float beta = (float)S->beta, bo = (float)S->beta_omega;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const float pi = a.r[i] + beta * a.p[i] - bo * a.v[i];
        a.p[i] = pi;
        a.y[i] = a.dinv ? a.dinv[i] * pi : pi;
    }
}

// ---------------------------------------------------------------------------------------------
// Flexible CG (FCG(1): each direction is A-orthogonalised against the previous one only)
//   z = M(r) (callback);  beta = -(z.Ap_prev)/(p_prev.Ap_prev);  p = z + beta p;
//   Ap = A p, alpha = (z.r)/(p.Ap) (k_cg_spmv);  x += alpha p, r -= alpha Ap (k_cg_update).
// ---------------------------------------------------------------------------------------------
__global__ __launch_bounds__(VEC_THREADS) void k_fcg_dir(const SolveArgs* __restrict__ args,
                                                         cudaGraphConditionalHandle h, int has_cond)
{
    pdl_enter();
    __shared__ double s_red[32 * 2];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    float zr = 0.f, zap = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const float zi = a.z[i];
        zr += zi * a.r[i];
        zap += zi * a.Ap[i];
    }
    float v[2] = {zr, zap};
    grid_reduce<2>(v, a.partials, &S->counters[5], s_red, [&](const double (&t)[2]) {
        S->rz = t[0];
        double beta = 0.0;
        if (S->iter > 0 && S->pAp != 0.0) beta = -t[1] / S->pAp;
        if (!finite(t[0]) || !finite(beta) || t[0] <= 0.0) {
            // the preconditioned residual is not a descent direction: hand over to the fallback
            S->status |= (t[0] <= 0.0 && finite(t[0])) ? GB_DEV_STAGNATION : GB_DEV_BREAKDOWN;
            set_cond(S, 0, h, has_cond);
            beta = 0.0;
        }
        S->beta = beta;
    });
}

__global__ __launch_bounds__(VEC_THREADS) void k_fcg_p(const SolveArgs* __restrict__ args)
{
    pdl_enter();
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float beta = (float)S->beta;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride)
        a.p[i] = a.z[i] + beta * a.p[i];
}

__global__ void k_store_args(SolveArgs* dst, SolveArgs src, int reset_status)
{
    *dst = src;
    if (reset_status) {
        src.S->status = 0;
        for (int k = 0; k < 8; ++k) src.S->counters[k] = 0u;
        src.S->cond = 1;
    }
}

// ---------------------------------------------------------------------------------------------
// Host-side solver handle
// ---------------------------------------------------------------------------------------------
struct Solver {
    int kind, br, nrow, val_dtype;
    int64_t n;
    SpmvShape sh;
    int spmv_grid, vec_grid;
    size_t spmv_smem;
    SolveArgs host;     // operand pointers currently set
    SolveArgs* d_args;  // device copy (inside the workspace)
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec_while = nullptr, exec_init = nullptr, exec_chunk = nullptr;
    int chunk_iters = 0;
    gb_precond_fn precond = nullptr;  // flexible solver only
    void* precond_user = nullptr;
};

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct WsLayout {
    size_t args, scalars, partials, vec;
    int nvec;
    size_t total;
};

static WsLayout ws_layout(int kind, int64_t n, int spmv_grid, int vec_grid)
{
    WsLayout L;
    L.args = align256(sizeof(SolveArgs));
    L.scalars = align256(sizeof(KrylovScalars));
    L.partials = align256(sizeof(double) * 3 * (size_t)std::max(spmv_grid, vec_grid));
    L.vec = align256(sizeof(float) * (size_t)n);
    L.nvec = (kind == KRYLOV_CG) ? 3 : (kind == KRYLOV_FCG ? 4 : 7);  // CG: r p Ap; FCG: + z; BiCGSTAB: 7
    L.total = L.args + L.scalars + L.partials + L.nvec * L.vec + 256;
    return L;
}

template <int BR, typename VT> static void set_smem_attr(Solver* s)
{
    if (s->spmv_smem > 48 * 1024) {
        cudaFuncSetAttribute(k_cg_init<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->spmv_smem);
        cudaFuncSetAttribute(k_cg_spmv<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->spmv_smem);
        cudaFuncSetAttribute(k_bi_init<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->spmv_smem);
        cudaFuncSetAttribute(k_bi_spmv_v<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->spmv_smem);
        cudaFuncSetAttribute(k_bi_spmv_t<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->spmv_smem);
    }
}

template <int BR, typename VT>
static int launch_init_t(Solver* s, cudaStream_t st, cudaGraphConditionalHandle h, int has_cond)
{
    if (s->kind == KRYLOV_CG || s->kind == KRYLOV_FCG)
        GB_CHECK_CUDA(launch_pdl(k_cg_init<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args, s->nrow, s->sh, h, has_cond));
    else
        GB_CHECK_CUDA(launch_pdl(k_bi_init<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args, s->nrow, s->sh, h, has_cond));
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

template <int BR, typename VT>
static int launch_iter_t(Solver* s, cudaStream_t st, cudaGraphConditionalHandle h, int has_cond)
{
    if (s->kind == KRYLOV_FCG) {
        if (!s->precond) {
            gb::set_error("flexible solver: no preconditioner set");
            return GB_ERR_INVALID;
        }
        if (s->precond(s->precond_user, st, s->host.r, s->host.z) != 0) {
            gb::set_error("flexible solver: preconditioner callback failed");
            return GB_ERR_INVALID;
        }
        GB_CHECK_CUDA(launch_pdl(k_fcg_dir, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
        GB_CHECK_CUDA(launch_pdl(k_fcg_p, s->vec_grid, VEC_THREADS, 0, st, s->d_args));
        GB_CHECK_CUDA(launch_pdl(k_cg_spmv<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args, s->nrow, s->sh));
        GB_CHECK_CUDA(launch_pdl(k_cg_update, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
    } else if (s->kind == KRYLOV_CG) {
        GB_CHECK_CUDA(launch_pdl(k_cg_spmv<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args, s->nrow, s->sh));
        GB_CHECK_CUDA(launch_pdl(k_cg_update, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
        GB_CHECK_CUDA(launch_pdl(k_cg_pupdate, s->vec_grid, VEC_THREADS, 0, st, s->d_args));
    } else {
        GB_CHECK_CUDA(launch_pdl(k_bi_spmv_v<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args, s->nrow, s->sh));
        GB_CHECK_CUDA(launch_pdl(k_bi_update1, s->vec_grid, VEC_THREADS, 0, st, s->d_args));
        GB_CHECK_CUDA(launch_pdl(k_bi_spmv_t<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args, s->nrow, s->sh));
        GB_CHECK_CUDA(launch_pdl(k_bi_update2, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
        GB_CHECK_CUDA(launch_pdl(k_bi_pupdate, s->vec_grid, VEC_THREADS, 0, st, s->d_args));
    }
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

static int launch_init(Solver* s, cudaStream_t st, cudaGraphConditionalHandle h, int has_cond)
{
    if (s->br == 1) return s->val_dtype == GB_BF16 ? launch_init_t<1, __nv_bfloat16>(s, st, h, has_cond)
                                                   : launch_init_t<1, float>(s, st, h, has_cond);
    return s->val_dtype == GB_BF16 ? launch_init_t<3, __nv_bfloat16>(s, st, h, has_cond)
                                   : launch_init_t<3, float>(s, st, h, has_cond);
}

static int launch_iter(Solver* s, cudaStream_t st, cudaGraphConditionalHandle h, int has_cond)
{
    if (s->br == 1) return s->val_dtype == GB_BF16 ? launch_iter_t<1, __nv_bfloat16>(s, st, h, has_cond)
                                                   : launch_iter_t<1, float>(s, st, h, has_cond);
    return s->val_dtype == GB_BF16 ? launch_iter_t<3, __nv_bfloat16>(s, st, h, has_cond)
                                   : launch_iter_t<3, float>(s, st, h, has_cond);
}

// Appends init + while(condition){iteration} to the capture active on `st`.  Works both for the
// solver's own cached graph and inside a caller's stream capture (the reference's
// check_every=0 contract: the whole solve is capturable).
static int capture_full_solve(Solver* s, cudaStream_t st)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t g;
    const cudaGraphNode_t* deps;
    const cudaGraphEdgeData* edata;
    size_t ndeps;
    GB_CHECK_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edata, &ndeps));
    if (cs != cudaStreamCaptureStatusActive) {
        gb::set_error("capture_full_solve: stream is not capturing");
        return GB_ERR_INVALID;
    }
    cudaGraphConditionalHandle h;
    GB_CHECK_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, 0));
    int rc = launch_init(s, st, h, 1);
    if (rc) return rc;
    GB_CHECK_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &edata, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    GB_CHECK_CUDA(cudaGraphAddNode(&cnode, g, deps, edata, ndeps, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    GB_CHECK_CUDA(cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies));
    GB_CHECK_CUDA(cudaStreamBeginCaptureToGraph(s->cap_stream, body, nullptr, nullptr, 0,
                                                cudaStreamCaptureModeRelaxed));
    rc = launch_iter(s, s->cap_stream, h, 1);
    cudaGraph_t body_out;
    cudaError_t e = cudaStreamEndCapture(s->cap_stream, &body_out);
    if (rc) return rc;
    GB_CHECK_CUDA(e);
    return GB_OK;
}

static int build_graphs(Solver* s, int chunk_iters)
{
    cudaGraph_t g;
    // full solve: init + conditional while loop
    if (!s->exec_while) {
        GB_CHECK_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeRelaxed));
        // capture_full_solve needs a second stream for the body capture
        cudaStream_t outer = s->cap_stream;
        cudaStream_t body_stream;
        GB_CHECK_CUDA(cudaStreamCreateWithFlags(&body_stream, cudaStreamNonBlocking));
        s->cap_stream = body_stream;
        int rc = capture_full_solve(s, outer);
        s->cap_stream = outer;
        cudaError_t e = cudaStreamEndCapture(outer, &g);
        cudaStreamDestroy(body_stream);
        if (rc) return rc;
        GB_CHECK_CUDA(e);
        GB_CHECK_CUDA(cudaGraphInstantiate(&s->exec_while, g, 0));
        cudaGraphDestroy(g);
    }
    if (!s->exec_init) {
        GB_CHECK_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeRelaxed));
        int rc = launch_init(s, s->cap_stream, 0, 0);
        cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
        if (rc) return rc;
        GB_CHECK_CUDA(e);
        GB_CHECK_CUDA(cudaGraphInstantiate(&s->exec_init, g, 0));
        cudaGraphDestroy(g);
    }
    if (chunk_iters > 0 && chunk_iters != s->chunk_iters) {
        if (s->exec_chunk) cudaGraphExecDestroy(s->exec_chunk);
        s->exec_chunk = nullptr;
        GB_CHECK_CUDA(cudaStreamBeginCapture(s->cap_stream, cudaStreamCaptureModeRelaxed));
        int rc = GB_OK;
        for (int k = 0; k < chunk_iters && rc == GB_OK; ++k) rc = launch_iter(s, s->cap_stream, 0, 0);
        cudaError_t e = cudaStreamEndCapture(s->cap_stream, &g);
        if (rc) return rc;
        GB_CHECK_CUDA(e);
        GB_CHECK_CUDA(cudaGraphInstantiate(&s->exec_chunk, g, 0));
        cudaGraphDestroy(g);
        s->chunk_iters = chunk_iters;
    }
    return GB_OK;
}

}  // namespace gb

using namespace gb;

GB_API size_t gb_krylov_workspace_bytes(int kind, int block_dim, int nrow, int64_t nnz, int val_dtype)
{
    const int64_t n = (int64_t)nrow * block_dim;
    const int grid = std::max(sm_count(), kSmCount) * 4;  // upper bound of both persistent grids
    return ws_layout(kind, n, grid, grid).total;
}

// Creates a solver handle for a BSR system with block_dim x block_dim blocks (1 or 3) and values
// of val_dtype (GB_F32 or GB_BF16).  The workspace (from gb_krylov_workspace_bytes) holds the
// work vectors, scalars and reduction partials; the handle owns only its CUDA graphs.
GB_API int gb_krylov_create(int kind, int block_dim, int nrow, int64_t nnz, int64_t ncap, int val_dtype,
                            int rows_per_cta, int lanes_per_row, int cap_blocks, void* workspace,
                            size_t workspace_bytes, void** handle_out)
{
    GB_REQUIRE(kind == KRYLOV_CG || kind == KRYLOV_BICGSTAB || kind == KRYLOV_FCG, "krylov: unknown solver kind %d",
               kind);
    GB_REQUIRE(block_dim == 1 || block_dim == 3, "krylov: block_dim must be 1 or 3");
    GB_REQUIRE(val_dtype == GB_F32 || val_dtype == GB_BF16, "krylov: values must be float32 or bfloat16");
    GB_REQUIRE(nrow > 0 && handle_out && workspace, "krylov: bad arguments");
    Solver* s = new (std::nothrow) Solver();
    if (!s) {
        gb::set_error("krylov: out of host memory");
        return GB_ERR_INVALID;
    }
    s->kind = kind;
    s->br = block_dim;
    s->nrow = nrow;
    s->val_dtype = val_dtype;
    s->n = (int64_t)nrow * block_dim;
    s->sh = default_shape(block_dim, block_dim, val_dtype, nrow, nnz, ncap, true);
    if (rows_per_cta > 0) s->sh.rows = rows_per_cta;
    if (lanes_per_row > 0) s->sh.G = lanes_per_row;
    if (cap_blocks > 0) s->sh.cap = cap_blocks & ~(SPMV_ALIGN - 1);
    s->sh.ncap = ncap;
    s->sh.rows = std::max(4, (s->sh.rows + 3) & ~3);
    s->spmv_smem = (block_dim == 1)
                       ? (val_dtype == GB_BF16 ? spmv_smem_bytes<1, 1, __nv_bfloat16>(s->sh.rows, s->sh.cap, s->sh.stages)
                                               : spmv_smem_bytes<1, 1, float>(s->sh.rows, s->sh.cap, s->sh.stages))
                       : (val_dtype == GB_BF16 ? spmv_smem_bytes<3, 3, __nv_bfloat16>(s->sh.rows, s->sh.cap, s->sh.stages)
                                               : spmv_smem_bytes<3, 3, float>(s->sh.rows, s->sh.cap, s->sh.stages));
    if (s->spmv_smem > 227 * 1024) {
        gb::set_error("krylov: tile shape needs %zu bytes of shared memory", s->spmv_smem);
        delete s;
        return GB_ERR_INVALID;
    }
    finalize_shape(s->sh, nrow, s->spmv_smem, nullptr);  // offsets alignment is set per operand
    s->spmv_grid = s->sh.grid;
    s->vec_grid = sm_count() * 4;
    WsLayout L = ws_layout(kind, s->n, std::max(sm_count(), kSmCount) * 4, std::max(sm_count(), kSmCount) * 4);
    if (workspace_bytes < L.total) {
        gb::set_error("krylov: workspace too small (%zu < %zu)", workspace_bytes, L.total);
        delete s;
        return GB_ERR_CAPACITY;
    }
    unsigned char* ws = reinterpret_cast<unsigned char*>(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
    s->d_args = reinterpret_cast<SolveArgs*>(ws);
    ws += L.args;
    s->host = SolveArgs{};
    s->host.S = reinterpret_cast<KrylovScalars*>(ws);
    ws += L.scalars;
    s->host.partials = reinterpret_cast<double*>(ws);
    ws += L.partials;
    float* vecs[7] = {nullptr};
    for (int k = 0; k < L.nvec; ++k) {
        vecs[k] = reinterpret_cast<float*>(ws);
        ws += L.vec;
    }
    if (kind == KRYLOV_CG || kind == KRYLOV_FCG) {
        s->host.r = vecs[0];
        s->host.p = vecs[1];
        s->host.Ap = vecs[2];
        if (kind == KRYLOV_FCG) s->host.z = vecs[3];
    } else {
        s->host.r = vecs[0];
        s->host.r0 = vecs[1];
        s->host.p = vecs[2];
        s->host.v = vecs[3];
        s->host.t = vecs[4];
        s->host.y = vecs[5];
        s->host.z = vecs[6];
    }
    s->host.n = s->n;
    if (block_dim == 1) {
        if (val_dtype == GB_BF16) set_smem_attr<1, __nv_bfloat16>(s); else set_smem_attr<1, float>(s);
    } else {
        if (val_dtype == GB_BF16) set_smem_attr<3, __nv_bfloat16>(s); else set_smem_attr<3, float>(s);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&s->cap_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return gb::cuda_fail(e, "cudaStreamCreateWithFlags");
    }
    // scalars/counters start zeroed
    e = cudaMemset(s->host.S, 0, sizeof(KrylovScalars));
    if (e != cudaSuccess) {
        cudaStreamDestroy(s->cap_stream);
        delete s;
        return gb::cuda_fail(e, "cudaMemset");
    }
    *handle_out = s;
    return GB_OK;
}

GB_API int gb_krylov_destroy(void* handle)
{
    Solver* s = static_cast<Solver*>(handle);
    if (!s) return GB_OK;
    if (s->exec_while) cudaGraphExecDestroy(s->exec_while);
    if (s->exec_init) cudaGraphExecDestroy(s->exec_init);
    if (s->exec_chunk) cudaGraphExecDestroy(s->exec_chunk);
    if (s->cap_stream) cudaStreamDestroy(s->cap_stream);
    delete s;
    return GB_OK;
}

// Sets the operands of the next solve (stream-ordered: a one-thread kernel writes the device
// argument block, so this is capturable too).  dinv may be null (no preconditioner).
GB_API int gb_krylov_set_operands(void* handle, const int* offsets, const int* row_counts, const int* columns,
                                  const void* values, const float* dinv, const float* b, float* x, int x_is_zero,
                                  double tol, double atol, int maxiter, int left_precond, cudaStream_t stream)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s && offsets && columns && values && b && x, "krylov_set_operands: null argument");
    s->host.offsets = offsets;
    s->host.row_counts = row_counts;
    s->host.columns = columns;
    s->host.values = values;
    s->host.dinv = (s->kind == KRYLOV_FCG) ? nullptr : dinv;
    s->host.b = b;
    s->host.x = x;
    s->host.x_is_zero = x_is_zero;
    s->host.tol = tol;
    s->host.atol = atol;
    s->host.maxiter = maxiter;
    s->host.left_precond = left_precond;
    const bool aligned = ((uintptr_t)columns % 16 == 0) && ((uintptr_t)values % 16 == 0);
    if (!aligned && s->sh.cap != 0) {
        gb::set_error("krylov_set_operands: columns/values must be 16-byte aligned");
        return GB_ERR_INVALID;
    }
    const int off_bulk = ((uintptr_t)offsets % 16 == 0) ? 1 : 0;
    if (off_bulk != s->sh.off_bulk) {
        // the shape is baked into the cached graphs: rebuild them for the new alignment
        s->sh.off_bulk = off_bulk;
        if (s->exec_while) cudaGraphExecDestroy(s->exec_while);
        if (s->exec_init) cudaGraphExecDestroy(s->exec_init);
        if (s->exec_chunk) cudaGraphExecDestroy(s->exec_chunk);
        s->exec_while = s->exec_init = s->exec_chunk = nullptr;
        s->chunk_iters = 0;
    }
    k_store_args<<<1, 1, 0, stream>>>(s->d_args, s->host, 1);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}

// what: 0 = whole solve (init + device-side while loop), 1 = init only, 2 = `chunk_iters`
// iterations (each iteration is a no-op once converged), 3 = one eager (non-graph) iteration,
// 4 = eager init.  Modes 0-2 replay cached graphs; if `stream` is capturing, mode 0 is appended
// to the caller's capture instead.
GB_API int gb_krylov_launch(void* handle, int what, int chunk_iters, cudaStream_t stream)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s, "krylov_launch: null handle");
    cudaStreamCaptureStatus cs;
    GB_CHECK_CUDA(cudaStreamIsCapturing(stream, &cs));
    const bool capturing = (cs == cudaStreamCaptureStatusActive);
    if (what == 3) return launch_iter(s, stream, 0, 0);
    if (what == 4) return launch_init(s, stream, 0, 0);
    if (capturing) {
        if (what == 0) return capture_full_solve(s, stream);
        if (what == 1) return launch_init(s, stream, 0, 0);
        int rc = GB_OK;
        for (int k = 0; k < chunk_iters && rc == GB_OK; ++k) rc = launch_iter(s, stream, 0, 0);
        return rc;
    }
    int rc = build_graphs(s, what == 2 ? chunk_iters : 0);
    if (rc) return rc;
    if (what == 0) GB_CHECK_CUDA(cudaGraphLaunch(s->exec_while, stream));
    else if (what == 1) GB_CHECK_CUDA(cudaGraphLaunch(s->exec_init, stream));
    else if (what == 2) GB_CHECK_CUDA(cudaGraphLaunch(s->exec_chunk, stream));
    else {
        gb::set_error("krylov_launch: bad mode %d", what);
        return GB_ERR_INVALID;
    }
    return GB_OK;
}

// Device addresses of the solver scalars (iteration count, residual^2, atol^2, status), so the
// host can return them as device arrays (the check_every == 0 contract) or copy them back.
GB_API int gb_krylov_scalars(void* handle, int** iter, double** rr, double** atol_sq, int** status)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s, "krylov_scalars: null handle");
    if (iter) *iter = &s->host.S->iter;
    if (rr) *rr = &s->host.S->rr;
    if (atol_sq) *atol_sq = &s->host.S->atol_sq;
    if (status) *status = &s->host.S->status;
    return GB_OK;
}

// Copies {iter, cond, status} and {rr, atol_sq, bb} to host buffers (stream-ordered).
GB_API int gb_krylov_read(void* handle, int* host_ints3, double* host_doubles3, cudaStream_t stream)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s && host_ints3 && host_doubles3, "krylov_read: null argument");
    KrylovScalars* S = s->host.S;
    GB_CHECK_CUDA(cudaMemcpyAsync(host_ints3, &S->iter, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(host_ints3 + 2, &S->status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(host_doubles3, &S->rr, sizeof(double), cudaMemcpyDeviceToHost, stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(host_doubles3 + 1, &S->atol_sq, sizeof(double), cudaMemcpyDeviceToHost, stream));
    GB_CHECK_CUDA(cudaMemcpyAsync(host_doubles3 + 2, &S->bb, sizeof(double), cudaMemcpyDeviceToHost, stream));
    return GB_OK;
}

// Device pointers of the work vectors (r, p/r0, Ap/p, ...) for tests and the FCG driver.
GB_API int gb_krylov_vectors(void* handle, float** r, float** p, float** Ap)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s, "krylov_vectors: null handle");
    if (r) *r = s->host.r;
    if (p) *p = s->host.p;
    if (Ap) *Ap = (s->kind == KRYLOV_BICGSTAB) ? s->host.v : s->host.Ap;
    return GB_OK;
}

// Flexible solver: set the preconditioner callback (called with the solver's r and z vectors
// whenever an iteration is enqueued -- at graph capture time for the cached graphs) and the
// stagnation rule (window > 0: every `window` iterations the residual norm must have dropped by
// at least `factor`, else GB_DEV_STAGNATION stops the loop).  Drops any cached graphs.
GB_API int gb_krylov_set_precond(void* handle, gb_precond_fn fn, void* user, int stag_window, double stag_factor)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s && s->kind == KRYLOV_FCG, "krylov_set_precond: flexible solver handle required");
    s->precond = fn;
    s->precond_user = user;
    s->host.stag_window = stag_window;
    s->host.stag_factor = stag_factor;
    if (s->exec_while) cudaGraphExecDestroy(s->exec_while);
    if (s->exec_init) cudaGraphExecDestroy(s->exec_init);
    if (s->exec_chunk) cudaGraphExecDestroy(s->exec_chunk);
    s->exec_while = s->exec_init = s->exec_chunk = nullptr;
    s->chunk_iters = 0;
    return GB_OK;
}
