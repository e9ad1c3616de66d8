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
// are deterministic; double-float across warps and CTAs, grid_reduce_df) and computes the next
// scalar (alpha, beta, the loop condition).  Nothing in these kernels waits on another CTA; the
// persistent CG below does, at grid barriers of a cooperative launch.
//
// Solver scalars live in device memory; the loop condition is evaluated on the device and drives
// a cudaGraphCondTypeWhile node, so a whole solve is one graph launch with no host round trip.
// Kernels read the operand pointers through a small device-side argument block so one captured
// graph serves every right-hand side / solution vector / matrix with the same shape.
#include "gb_common.cuh"
#include "gb_df32.cuh"
#include "gb_spmv.cuh"
#include "gb_st27.cuh"

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
    // grid barrier of the persistent CG: arrival count and generation on cache lines of their own
    // (the generation is polled by every CTA; the count takes one atomic per CTA)
    alignas(128) unsigned int bar_count;
    alignas(128) unsigned int bar_gen;
    // tile queues of the persistent CG's SpMV phase, one per iteration parity (zero between launches)
    alignas(128) unsigned int tile_ctr[2];
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
    grid_reduce_df<3>(v, a.partials, &a.S->counters[0], s_red,
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
    grid_reduce_df<1>(v, a.partials, &S->counters[1], s_red, [&](const double (&t)[1]) {
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
    grid_reduce_df<2>(v, a.partials, &S->counters[2], s_red, [&](const double (&t)[2]) {
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
        if (S->status & GB_DEV_BREAKDOWN) cond = 0;  // a non-finite alpha or beta ends the loop
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
// CG as one persistent cooperative launch
// ---------------------------------------------------------------------------------------------
// The three phases of an iteration -- (1) Ap = A p with p.Ap, (2) x += alpha p, r -= alpha Ap with
// r.r and r.z, (3) p = D^-1 r + beta p -- run inside one kernel whose CTAs are all resident
// (cooperative launch) and meet at a grid barrier after each phase.  Phase 1 is the SpMV pipeline over
// tiles of block rows that each CTA's producer takes from the iteration's queue (an atomic counter),
// so SMs that stream faster take more tiles; phases 2 and 3 walk the vectors grid-stride (after a
// barrier every CTA may read any row).  Every CTA sums all CTAs' partials in the same fixed order
// (double-float), so all derive bit-identical alpha, beta and loop condition without a broadcast.
// The producer warp streams the matrix tiles continuously across iterations (the matrix does not
// change), so the copy ring does not drain at the barriers; those copies carry an L2 evict-first
// policy so that the vectors of phases 2 and 3 stay in L2.  p is gathered with coherent (non-.nc)
// loads since it changes between phases of the same launch.  Per iteration the arithmetic is that of
// k_cg_spmv / k_cg_update / k_cg_pupdate except for the sums: double-float instead of FP64, and
// alpha, beta formed in fp32 (the three-kernel path rounds its FP64 quotients to fp32 before use).
// Every wait is bounded: a barrier that does not complete within kWaitLimitNs sets
// GB_DEV_WAIT_TIMEOUT and ends the CTA's loop.

__device__ __forceinline__ void consumer_sync()
{
    asm volatile("bar.sync 1, %0;" ::"r"(SPMV_CONSUMERS) : "memory");
}

__device__ __forceinline__ unsigned int ld_acquire_u32(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u32(unsigned int* p, unsigned int v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier among the consumer threads of every CTA (thread 32 arrives for its CTA): the last
// arrival resets the count and advances the generation; the others poll the generation.  Returns
// the same value in every consumer thread of the CTA: false if the wait ran out or a warp of the CTA
// flagged a failed wait beforehand (*s_fail).  The last arrival also zeroes *reset_on_last, if given,
// before it releases the others.
__device__ __forceinline__ bool cg_grid_barrier(KrylovScalars* S, volatile int* s_ok, volatile int* s_fail,
                                                unsigned int* reset_on_last = nullptr)
{
    consumer_sync();
    if (threadIdx.x == 32) {
        const unsigned int g = ld_acquire_u32(&S->bar_gen);
        unsigned int prev;
        // release: the CTA's writes (ordered before this thread by the barrier above) become visible
        // to every CTA that acquires the new generation
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(prev) : "l"(&S->bar_count) : "memory");
        int ok = 1;
        if (prev == gridDim.x - 1) {
            atomicExch(&S->bar_count, 0u);
            if (reset_on_last) atomicExch(reset_on_last, 0u);
            st_release_u32(&S->bar_gen, g + 1u);
        } else {
            const uint64_t t0 = globaltimer_ns();
            while (ld_acquire_u32(&S->bar_gen) == g) {
                if (globaltimer_ns() - t0 > kWaitLimitNs) {
                    ok = 0;
                    break;
                }
            }
        }
        *s_ok = ok && !*s_fail;
    }
    consumer_sync();
    return *s_ok != 0;
}

// Sums inside the persistent CG run in double-float (gb_df32.cuh): GB300's FP64 pipe is a small
// fraction of its FP32 rate and its latency sat on the critical path between the grid barriers.

// Sum of NV per-thread fp32 values over the 512 consumer threads (fp32 within a warp, double-float
// across warps); the result is valid in thread 32.
template <int NV> __device__ __forceinline__ void consumer_sum(const float (&v)[NV], float* s_red, df32 (&out)[NV])
{
    const int cw = (threadIdx.x >> 5) - 1, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const float w = warp_sum(v[k]);
        if (lane == 0) s_red[cw * NV + k] = w;
    }
    consumer_sync();
    if (cw == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            out[k] = warp_sum_df(df32(lane < SPMV_CONSUMER_WARPS ? s_red[lane * NV + k] : 0.f, 0.f));
    }
}

// The same sum of per-thread double-float values (2 floats per warp per value in s_red).
template <int NV> __device__ __forceinline__ void consumer_sum_df(const df32 (&v)[NV], float* s_red, df32 (&out)[NV])
{
    const int cw = (threadIdx.x >> 5) - 1, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const df32 w = warp_sum_df(v[k]);
        if (lane == 0) {
            s_red[(cw * NV + k) * 2] = w.hi;
            s_red[(cw * NV + k) * 2 + 1] = w.lo;
        }
    }
    consumer_sync();
    if (cw == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const bool in = lane < SPMV_CONSUMER_WARPS;
            out[k] = warp_sum_df(df32(in ? s_red[(lane * NV + k) * 2] : 0.f, in ? s_red[(lane * NV + k) * 2 + 1] : 0.f));
        }
    }
}

// Sum of every CTA's double-float partials part[k * gridDim.x + c] over the consumer threads (one or
// two loads each, warp sums, then a sum of the 16 warp totals), in the same fixed order in every CTA;
// thread 32 passes the totals to `update` (which changes the shared solver state), and the consumers
// resynchronise so that all of them see the new state.
template <int NV, typename Update>
__device__ __forceinline__ void all_partials(const float2* part, float* s_red, Update update)
{
    const int ct = threadIdx.x - 32, cw = ct >> 5, lane = threadIdx.x & 31;
    df32 acc[NV];
    for (int c = ct; c < (int)gridDim.x; c += SPMV_CONSUMERS) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const float2 v = __ldcg(part + (size_t)k * gridDim.x + c);
            acc[k] += df32(v.x, v.y);
        }
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const df32 w = warp_sum_df(acc[k]);
        if (lane == 0) {
            s_red[(cw * NV + k) * 2] = w.hi;
            s_red[(cw * NV + k) * 2 + 1] = w.lo;
        }
    }
    consumer_sync();
    if (cw == 0) {
        df32 t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const bool in = lane < SPMV_CONSUMER_WARPS;
            t[k] = warp_sum_df(df32(in ? s_red[(lane * NV + k) * 2] : 0.f, in ? s_red[(lane * NV + k) * 2 + 1] : 0.f));
        }
        if (lane == 0) update(t);
    }
    consumer_sync();
}

struct LoopState {
    df32 rz, rr, rr_ref, atol_sq, pAp;
    float alpha, beta;
    int iter, cond, maxiter, breakdown;
};

template <int BR, typename VT>
__global__ __launch_bounds__(SPMV_THREADS, 2) void k_cg_loop(const SolveArgs* __restrict__ args, int nrow, SpmvShape sh,
                                                          int max_iters)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ float s_red[SPMV_CONSUMER_WARPS * 2 * 2];
    __shared__ __align__(16) unsigned char st_raw[sizeof(LoopState)];  // no constructor: thread 32 fills it
    LoopState& st = *reinterpret_cast<LoopState*>(st_raw);
    __shared__ int s_ok, s_fail, s_stop, s_citer, s_pdone;
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    const SpmvRing R = spmv_ring<BR, BR, VT>(smem, sh);
    const int NS = sh.stages;
    const int ntiles = (nrow + sh.rows - 1) / sh.rows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const VT* values = (const VT*)a.values;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&R.full[s], 1);
            mbar_init(&R.empty[s], SPMV_CONSUMER_WARPS);
        }
        fence_mbar_init();
        s_stop = 0;
        s_fail = 0;
        s_citer = 0;
        s_pdone = 0;
    }
    __syncthreads();

    if (warp == 0) {
        // ------------------ producer: tiles of successive iterations, until told to stop -----------
        // Tiles are taken from the iteration's queue (an atomic counter), so CTAs that stream faster
        // take more of them; each CTA's run of tiles for an iteration ends with a sentinel slot (no
        // copy, header nr = -1).  The producer starts on iteration j once the consumers are in
        // iteration j - 1: the queue of iteration j (parity j & 1) was zeroed at the phase-1 barrier
        // of iteration j - 2, after every CTA's last take from it.
        if (lane == 0) {
            const uint64_t policy = l2_policy_evict_first();
            int t = 0, b0 = 0, b1 = 0;
            auto take = [&](int j) {
                t = (int)atomicAdd(&S->tile_ctr[j & 1], 1u);
                if (t < ntiles) {
                    const int r0 = t * sh.rows;
                    b0 = a.offsets[r0];
                    b1 = a.offsets[min(r0 + sh.rows, nrow)];
                }
            };
            int i = 0;
            bool timed_out = false, stop = false;
            for (int j = 0; !stop; ++j) {
                if (j >= 2) {  // gate: the consumers have entered iteration j - 1
                    const uint64_t t0 = globaltimer_ns();
                    while (*(volatile int*)&s_citer < j - 1) {
                        if (*(volatile int*)&s_stop) {
                            stop = true;
                            break;
                        }
                        if (globaltimer_ns() - t0 > kWaitLimitNs) {
                            timed_out = stop = true;
                            break;
                        }
                        __nanosleep(128);
                    }
                    if (stop) break;
                }
                take(j);
                for (;;) {
                    const int s = i % NS;
                    const uint32_t ph = (uint32_t)(i / NS) & 1u;
                    if (i >= NS) {
                        const uint64_t t0 = globaltimer_ns();
                        for (;;) {
                            if (mbar_try_wait(&R.empty[s], ph ^ 1u)) break;
                            if (*(volatile int*)&s_stop) {
                                stop = true;
                                break;
                            }
                            if (globaltimer_ns() - t0 > kWaitLimitNs) {
                                timed_out = stop = true;
                                break;
                            }
                        }
                    } else if (*(volatile int*)&s_stop) {
                        stop = true;
                    }
                    if (stop) break;
                    if (t >= ntiles) {  // sentinel: this CTA's tiles of iteration j are all issued
                        R.hdr[s].nr = -1;
                        mbar_arrive(&R.full[s]);
                        ++i;
                        break;
                    }
                    spmv_issue<BR, BR, VT>(R, sh, nrow, s, t, b0, b1, a.offsets, a.columns, values, true, policy);
                    ++i;
                    take(j);  // the next tile's take and offsets overlap the copies just issued
                }
            }
            if (timed_out) atomicOr(&S->status, GB_DEV_WAIT_TIMEOUT);
            // drain: no bulk copy of this CTA may still be in flight when it exits
            for (int q = max(0, i - NS); q < i; ++q) mbar_wait_bounded(&R.full[q % NS], (uint32_t)(q / NS) & 1u);
            __threadfence_block();
            *(volatile int*)&s_pdone = 1;
        }
    } else {
        // ------------------ consumers: the three phases of every iteration ------------------------
        // The solver scalars live in shared memory, updated by thread 32 from the grid-wide sums
        // (identical in every CTA); CTA 0 writes them back to the device scalars at the end.
        const int ct = threadIdx.x - 32;
        if (threadIdx.x == 32) {
            st.rz = df_from_double(S->rz);
            st.rr = df_from_double(S->rr);
            st.rr_ref = df_from_double(S->rr_ref);
            st.atol_sq = df_from_double(S->atol_sq);
            st.pAp = df_from_double(S->pAp);
            st.alpha = (float)S->alpha;
            st.beta = (float)S->beta;
            st.iter = S->iter;
            st.cond = S->cond;
            st.maxiter = S->maxiter;
            st.breakdown = 0;
        }
        consumer_sync();
        const bool lead = (blockIdx.x == 0 && threadIdx.x == 32);
        constexpr int BB = BR * BR;
        const int G = sh.G;
        const int lane_g = ct & (G - 1);
        const int grp = ct / G;
        const int ngroups = SPMV_CONSUMERS / G;
        float2* partA = reinterpret_cast<float2*>(a.partials);  // [gridDim.x]: p.Ap (double-float)
        float2* partB = partA + gridDim.x;                        // [2][gridDim.x]: r.r, r.z
        const bool vec4 = ((((uintptr_t)a.x | (uintptr_t)a.r | (uintptr_t)a.p | (uintptr_t)a.Ap |
                             (uintptr_t)(a.dinv ? a.dinv : a.r)) & 15) == 0);
        int i = 0, done = 0;
        bool ok = true;
        while (st.cond && (max_iters <= 0 || done < max_iters)) {
            if (threadIdx.x == 32) *(volatile int*)&s_citer = done;
            // (1) Ap = A p, p.Ap over the tiles this CTA's producer took, up to its sentinel.  Each thread's
            // fp32 sum covers the rows one tile gives it (the same in every run, whichever CTA takes the
            // tile); the tile sums then go into a double-float total, so the schedule changes p.Ap only at
            // the double-float rounding level
            EpiCgAp<BR, float> epi{a.Ap, a.p};
            df32 pap_df;
            for (;; ++i) {
                const int s = i % NS;
                const uint32_t ph = (uint32_t)(i / NS) & 1u;
                const bool full_ok = __all_sync(0xffffffffu, mbar_wait_bounded(&R.full[s], ph));
                const bool tile = full_ok && R.hdr[s].nr >= 0;
                if (tile) {
                    // the rows of the staged tile (the loop of spmv_run, with coherent gathers of p)
                    epi.pAp = 0.f;
                    const StageHeader h = R.hdr[s];
                    const unsigned char* stg = R.ring + (size_t)s * R.stage_bytes;
                    const int* s_off = reinterpret_cast<const int*>(stg);
                    const int* cbase = h.staged ? reinterpret_cast<const int*>(stg + R.off_bytes) - h.a0 : a.columns;
                    const VT* vbase = h.staged ? reinterpret_cast<const VT*>(stg + R.off_bytes + R.col_bytes) -
                                                     (size_t)h.a0 * BB
                                               : values;
                    for (int kb = 0; kb < h.nr; kb += ngroups) {
                        const int k = kb + grp;
                        const bool active = k < h.nr;
                        int beg = 0, end = 0;
                        if (active) {
                            beg = s_off[k];
                            end = a.row_counts ? beg + a.row_counts[h.r0 + k] : s_off[k + 1];
                        }
                        float acc[BR];
#pragma unroll
                        for (int q = 0; q < BR; ++q) acc[q] = 0.f;
                        constexpr int U = (BB == 1) ? 8 : 4;
                        for (int base = beg + lane_g; base < end; base += U * G) {
                            int cc[U];
#pragma unroll
                            for (int u = 0; u < U; ++u) {
                                const int bi = base + u * G;
                                cc[u] = (bi < end) ? cbase[bi] : -1;
                            }
                            float xv[U][BR];
#pragma unroll
                            for (int u = 0; u < U; ++u) {
#pragma unroll
                                for (int jj = 0; jj < BR; ++jj)
                                    xv[u][jj] = (cc[u] >= 0) ? __ldca(a.p + (size_t)cc[u] * BR + jj) : 0.f;
                            }
#pragma unroll
                            for (int u = 0; u < U; ++u) {
                                const int bi = base + u * G;
                                if (cc[u] >= 0) {
                                    const VT* vv = vbase + (size_t)bi * BB;
#pragma unroll
                                    for (int q = 0; q < BR; ++q) {
#pragma unroll
                                        for (int jj = 0; jj < BR; ++jj) acc[q] += cvt<float>(vv[q * BR + jj]) * xv[u][jj];
                                    }
                                }
                            }
                        }
#pragma unroll
                        for (int q = 0; q < BR; ++q) acc[q] = group_reduce(acc[q], G);
                        if (active) epi(h.r0 + k, acc, lane_g);
                    }
                    pap_df += df32(epi.pAp, 0.f);
                } else if (!full_ok && lane == 0) {
                    *(volatile int*)&s_fail = 1;
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&R.empty[s]);
                if (!tile) {
                    ++i;
                    break;
                }
            }
            {
                const df32 v[1] = {pap_df};
                df32 t[1];
                consumer_sum_df<1>(v, s_red, t);
                if (threadIdx.x == 32) partA[blockIdx.x] = make_float2(t[0].hi, t[0].lo);
            }
            // every CTA's producer has made its last take for this iteration: its queue is zeroed for
            // iteration done + 2
            if (!cg_grid_barrier(S, &s_ok, &s_fail, &S->tile_ctr[done & 1])) {
                ok = false;
                break;
            }
            all_partials<1>(partA, s_red, [&](const df32 (&t)[1]) {
                st.pAp = t[0];
                float alpha = 0.f;
                if (df_gt(st.rr, st.atol_sq)) {
                    alpha = (st.rz.hi + st.rz.lo) / (t[0].hi + t[0].lo);
                    if (!isfinite(alpha)) {
                        if (blockIdx.x == 0) atomicOr(&S->status, GB_DEV_BREAKDOWN);
                        st.breakdown = 1;
                        alpha = 0.f;
                    }
                }
                st.alpha = alpha;
            });
            // (2) x += alpha p, r -= alpha Ap; r.r and r.z (grid-stride: after the barrier every CTA
            // may read any row of Ap)
            float prr = 0.f, prz = 0.f;
            {
                const float al = st.alpha;
                int64_t e = 0;
                if (vec4) {
                    const int64_t n4 = a.n >> 2;
                    for (int64_t q = (int64_t)blockIdx.x * SPMV_CONSUMERS + ct; q < n4;
                         q += (int64_t)gridDim.x * SPMV_CONSUMERS) {
                        float4 xv = reinterpret_cast<float4*>(a.x)[q], rv = reinterpret_cast<float4*>(a.r)[q];
                        const float4 pv = reinterpret_cast<const float4*>(a.p)[q];
                        const float4 av = reinterpret_cast<const float4*>(a.Ap)[q];
                        xv.x += al * pv.x; xv.y += al * pv.y; xv.z += al * pv.z; xv.w += al * pv.w;
                        rv.x -= al * av.x; rv.y -= al * av.y; rv.z -= al * av.z; rv.w -= al * av.w;
                        float4 zv = rv;
                        if (a.dinv) {
                            const float4 dv = reinterpret_cast<const float4*>(a.dinv)[q];
                            zv.x *= dv.x; zv.y *= dv.y; zv.z *= dv.z; zv.w *= dv.w;
                        }
                        reinterpret_cast<float4*>(a.x)[q] = xv;
                        reinterpret_cast<float4*>(a.r)[q] = rv;
                        prr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
                        prz += rv.x * zv.x + rv.y * zv.y + rv.z * zv.z + rv.w * zv.w;
                    }
                    e = n4 << 2;
                }
                for (int64_t k = e + (int64_t)blockIdx.x * SPMV_CONSUMERS + ct; k < a.n;
                     k += (int64_t)gridDim.x * SPMV_CONSUMERS) {
                    const float ri = a.r[k] - al * a.Ap[k];
                    const float zi = a.dinv ? a.dinv[k] * ri : ri;
                    a.x[k] += al * a.p[k];
                    a.r[k] = ri;
                    prr += ri * ri;
                    prz += ri * zi;
                }
            }
            {
                const float v[2] = {prr, prz};
                df32 t[2];
                consumer_sum<2>(v, s_red, t);
                if (threadIdx.x == 32) {
                    partB[blockIdx.x] = make_float2(t[0].hi, t[0].lo);
                    partB[gridDim.x + blockIdx.x] = make_float2(t[1].hi, t[1].lo);
                }
            }
            if (!cg_grid_barrier(S, &s_ok, &s_fail)) {
                ok = false;
                break;
            }
            all_partials<2>(partB, s_red, [&](const df32 (&t)[2]) {
                const float rz_old = st.rz.hi + st.rz.lo;
                st.rr = t[0];
                st.rz = t[1];
                float beta = 0.f;
                const bool above = df_gt(t[0], st.atol_sq);
                if (above) {
                    beta = (t[1].hi + t[1].lo) / rz_old;
                    if (!isfinite(beta)) {
                        if (blockIdx.x == 0) atomicOr(&S->status, GB_DEV_BREAKDOWN);
                        st.breakdown = 1;
                        beta = 0.f;
                    }
                }
                st.beta = beta;
                st.iter += 1;
                int cond = above && (st.iter < st.maxiter) && !st.breakdown;
                if (!isfinite(t[0].hi)) {
                    if (blockIdx.x == 0) atomicOr(&S->status, GB_DEV_NONFINITE);
                    cond = 0;
                }
                if (a.stag_window > 0 && cond && (st.iter % a.stag_window) == 0) {
                    const float f2 = (float)(a.stag_factor * a.stag_factor);
                    if (st.iter > a.stag_window && t[0].hi > f2 * st.rr_ref.hi) {
                        if (blockIdx.x == 0) atomicOr(&S->status, GB_DEV_STAGNATION);
                        cond = 0;
                    }
                    st.rr_ref = t[0];
                }
                st.cond = cond;
            });
            ++done;
            if (!st.cond) break;
            // (3) p = D^-1 r + beta p (grid-stride)
            {
                const float be = st.beta;
                int64_t e = 0;
                if (vec4) {
                    const int64_t n4 = a.n >> 2;
                    for (int64_t q = (int64_t)blockIdx.x * SPMV_CONSUMERS + ct; q < n4;
                         q += (int64_t)gridDim.x * SPMV_CONSUMERS) {
                        float4 zv = reinterpret_cast<const float4*>(a.r)[q];
                        if (a.dinv) {
                            const float4 dv = reinterpret_cast<const float4*>(a.dinv)[q];
                            zv.x *= dv.x; zv.y *= dv.y; zv.z *= dv.z; zv.w *= dv.w;
                        }
                        float4 pv = reinterpret_cast<float4*>(a.p)[q];
                        pv.x = zv.x + be * pv.x; pv.y = zv.y + be * pv.y; pv.z = zv.z + be * pv.z;
                        pv.w = zv.w + be * pv.w;
                        reinterpret_cast<float4*>(a.p)[q] = pv;
                    }
                    e = n4 << 2;
                }
                for (int64_t k = e + (int64_t)blockIdx.x * SPMV_CONSUMERS + ct; k < a.n;
                     k += (int64_t)gridDim.x * SPMV_CONSUMERS) {
                    const float zi = a.dinv ? a.dinv[k] * a.r[k] : a.r[k];
                    a.p[k] = zi + be * a.p[k];
                }
            }
            if (!cg_grid_barrier(S, &s_ok, &s_fail)) {
                ok = false;
                break;
            }
        }
        consumer_sync();
        if (threadIdx.x == 32 && !ok) {
            atomicOr(&S->status, GB_DEV_WAIT_TIMEOUT);
            st.cond = 0;
        }
        if (lead) {
            S->rr = df_to_double(st.rr);
            S->rz = df_to_double(st.rz);
            S->rr_ref = df_to_double(st.rr_ref);
            S->pAp = df_to_double(st.pAp);
            S->alpha = st.alpha;
            S->beta = st.beta;
            S->iter = st.iter;
            S->cond = ok ? st.cond : 0;
        }
        consumer_sync();
        // stop the producer; once every CTA's producer has stopped taking tiles, CTA 0 zeroes both
        // queues for the next launch
        if (threadIdx.x == 32) {
            *(volatile int*)&s_stop = 1;
            const uint64_t t0 = globaltimer_ns();
            while (!*(volatile int*)&s_pdone) {
                if (globaltimer_ns() - t0 > kWaitLimitNs) {
                    atomicOr(&S->status, GB_DEV_WAIT_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        if (cg_grid_barrier(S, &s_ok, &s_fail) && lead) {
            S->tile_ctr[0] = 0u;
            S->tile_ctr[1] = 0u;
        }
    }
    __syncthreads();
}

// Flexible-CG step on the 27-point stencil form of A (the fine level of the multigrid carrier holds
// it), in two kernels instead of four.  With p = z + beta p_old, A p = A z + beta A p_old, so the product
// runs on z as soon as the preconditioner has written it (Az into v) and forms z.r, z.Ap_old and z.Az in
// the same pass; from those beta = -(z.Ap_old)/(p_old.Ap_old), p.Ap = z.Az + beta z.Ap_old (A symmetric:
// p_old.Az = z.Ap_old) and alpha = (z.r)/(p.Ap).  k_fcg_update then forms p, Ap, x and r in one pass.  The
// product reads 108 B of coefficients and 16 B of vectors per node (the CSR's 8 B per nonzero otherwise);
// its staging is k_st27_apply's (gb_stencil.cu): per 256-node tile one bulk copy into a 2-stage ring,
// four CTAs per SM.
__global__ void __launch_bounds__(ST_TILE) k_fcg_st27_az(const SolveArgs* __restrict__ args, St27Grid g,
                                                         const float* __restrict__ Sc, cudaGraphConditionalHandle h,
                                                         int has_cond)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[32 * 3];
    pdl_enter();
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
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
        bulk_g2s(ring + (size_t)s * ST_TILE * 27, Sc + i0 * 27, bytes, &full[s]);
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < ST_STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        for (int s = 0; s < ST_STAGES; ++s)
            if (blockIdx.x + (int64_t)s * gridDim.x < ntiles) issue(blockIdx.x + (int64_t)s * gridDim.x, s);
    }
    __syncthreads();
    // before the first step Ap_old holds nothing of this solve: z.Ap_old is neither formed nor used
    const bool first = S->iter == 0;
    const int64_t yz = (int64_t)g.ny * g.nz;
    float zr = 0.f, zap = 0.f, zaz = 0.f;
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
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
                if (okx[dx + 1] && oky[dy + 1] && okz[dz + 1])
                    acc = fmaf(c[k], __ldg(a.z + i + dx * yz + (int64_t)dy * g.nz + dz), acc);
            }
            a.v[i] = acc;
            const float zi = a.z[i];
            zaz += zi * acc;
            zr += zi * a.r[i];
            if (!first) zap += zi * a.Ap[i];
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
            atomicOr(&S->status, GB_DEV_WAIT_TIMEOUT);
        }
        __syncthreads();
    }
    float v[3] = {zr, zap, zaz};
    grid_reduce_df<3>(v, a.partials, &S->counters[1], s_red, [&](const double (&t)[3]) {
        S->rz = t[0];
        double beta = 0.0, alpha = 0.0, pap = t[2];
        if (!first && S->pAp != 0.0) {
            beta = -t[1] / S->pAp;
            pap = t[2] + beta * t[1];
        }
        if (!finite(t[0]) || !finite(beta) || t[0] <= 0.0) {
            // the preconditioned residual is not a descent direction: hand over to the fallback
            S->status |= (t[0] <= 0.0 && finite(t[0])) ? GB_DEV_STAGNATION : GB_DEV_BREAKDOWN;
            set_cond(S, 0, h, has_cond);
            beta = 0.0;
        } else {
            alpha = t[0] / pap;
            if (!finite(alpha) || !(pap > 0.0)) {
                S->status |= GB_DEV_BREAKDOWN;
                set_cond(S, 0, h, has_cond);
                alpha = 0.0;
            }
        }
        S->beta = beta;
        S->pAp = pap;
        S->alpha = alpha;
    });
}

// p = z + beta p_old, Ap = Az + beta Ap_old (kept for the next step), x += alpha p, r -= alpha Ap; r.r and
// the loop condition (with the stagnation window of k_cg_update).
__global__ __launch_bounds__(VEC_THREADS) void k_fcg_update(const SolveArgs* __restrict__ args,
                                                            cudaGraphConditionalHandle h, int has_cond)
{
    pdl_enter();
    __shared__ double s_red[32];
    const SolveArgs a = *args;
    KrylovScalars* S = a.S;
    if (!S->cond) return;
    const float alpha = (float)S->alpha, beta = (float)S->beta;
    const bool first = S->iter == 0;  // p_old and Ap_old are not read before the first step
    const int64_t n = a.n;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float rr = 0.f;
    const bool vec4 = ((((uintptr_t)a.x | (uintptr_t)a.r | (uintptr_t)a.p | (uintptr_t)a.Ap | (uintptr_t)a.z |
                         (uintptr_t)a.v) & 15) == 0);
    int64_t done = 0;
    if (vec4) {
        const int64_t n4 = n >> 2;
        for (int64_t i = tid; i < n4; i += stride) {
            const float4 zv = reinterpret_cast<const float4*>(a.z)[i];
            const float4 av = reinterpret_cast<const float4*>(a.v)[i];
            float4 pv = zv, qv = av;
            if (!first) {
                const float4 po = reinterpret_cast<const float4*>(a.p)[i];
                const float4 qo = reinterpret_cast<const float4*>(a.Ap)[i];
                pv.x = fmaf(beta, po.x, zv.x); pv.y = fmaf(beta, po.y, zv.y);
                pv.z = fmaf(beta, po.z, zv.z); pv.w = fmaf(beta, po.w, zv.w);
                qv.x = fmaf(beta, qo.x, av.x); qv.y = fmaf(beta, qo.y, av.y);
                qv.z = fmaf(beta, qo.z, av.z); qv.w = fmaf(beta, qo.w, av.w);
            }
            reinterpret_cast<float4*>(a.p)[i] = pv;
            reinterpret_cast<float4*>(a.Ap)[i] = qv;
            float4 xv = reinterpret_cast<float4*>(a.x)[i], rv = reinterpret_cast<float4*>(a.r)[i];
            xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
            rv.x -= alpha * qv.x; rv.y -= alpha * qv.y; rv.z -= alpha * qv.z; rv.w -= alpha * qv.w;
            reinterpret_cast<float4*>(a.x)[i] = xv;
            reinterpret_cast<float4*>(a.r)[i] = rv;
            rr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
        }
        done = n4 << 2;
    }
    for (int64_t i = done + tid; i < n; i += stride) {
        const float pi = first ? a.z[i] : fmaf(beta, a.p[i], a.z[i]);
        const float qi = first ? a.v[i] : fmaf(beta, a.Ap[i], a.v[i]);
        a.p[i] = pi;
        a.Ap[i] = qi;
        a.x[i] += alpha * pi;
        const float ri = a.r[i] - alpha * qi;
        a.r[i] = ri;
        rr += ri * ri;
    }
    float v[1] = {rr};
    grid_reduce_df<1>(v, a.partials, &S->counters[2], s_red, [&](const double (&t)[1]) {
        S->rr = t[0];
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
    grid_reduce_df<2>(v, a.partials, &a.S->counters[0], s_red, [&](const double (&t)[2]) {
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
    grid_reduce_df<1>(v, a.partials, &S->counters[1], s_red, [&](const double (&t)[1]) {
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
    grid_reduce_df<1>(v, a.partials, &S->counters[2], s_red, [&](const double (&t)[1]) { S->rr = t[0]; });
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
    grid_reduce_df<2>(v, a.partials, &S->counters[3], s_red, [&](const double (&t)[2]) {
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
    grid_reduce_df<2>(v, a.partials, &S->counters[4], s_red, [&](const double (&t)[2]) {
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
// These four kernels serve the CSR product; on a stencil-form operator the same step takes the two
// kernels k_fcg_st27_az and k_fcg_update above.
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
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float zr = 0.f, zap = 0.f;
    int64_t done = 0;
    if ((((uintptr_t)a.z | (uintptr_t)a.r | (uintptr_t)a.Ap) & 15) == 0) {
        const int64_t n4 = a.n >> 2;
        for (int64_t i = tid; i < n4; i += stride) {
            const float4 zv = reinterpret_cast<const float4*>(a.z)[i];
            const float4 rv = reinterpret_cast<const float4*>(a.r)[i];
            const float4 av = reinterpret_cast<const float4*>(a.Ap)[i];
            zr += zv.x * rv.x + zv.y * rv.y + zv.z * rv.z + zv.w * rv.w;
            zap += zv.x * av.x + zv.y * av.y + zv.z * av.z + zv.w * av.w;
        }
        done = n4 << 2;
    }
    for (int64_t i = done + tid; i < a.n; i += stride) {
        const float zi = a.z[i];
        zr += zi * a.r[i];
        zap += zi * a.Ap[i];
    }
    float v[2] = {zr, zap};
    grid_reduce_df<2>(v, a.partials, &S->counters[5], s_red, [&](const double (&t)[2]) {
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
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if ((((uintptr_t)a.z | (uintptr_t)a.p) & 15) == 0) {
        const int64_t n4 = a.n >> 2;
        for (int64_t i = tid; i < n4; i += stride) {
            const float4 zv = reinterpret_cast<const float4*>(a.z)[i];
            float4 pv = reinterpret_cast<float4*>(a.p)[i];
            pv.x = zv.x + beta * pv.x; pv.y = zv.y + beta * pv.y; pv.z = zv.z + beta * pv.z; pv.w = zv.w + beta * pv.w;
            reinterpret_cast<float4*>(a.p)[i] = pv;
        }
        done = n4 << 2;
    }
    for (int64_t i = done + tid; i < a.n; i += stride) a.p[i] = a.z[i] + beta * a.p[i];
}

__global__ void k_store_args(SolveArgs* dst, SolveArgs src, int reset_status)
{
    *dst = src;
    if (reset_status) {
        src.S->status = 0;
        for (int k = 0; k < 8; ++k) src.S->counters[k] = 0u;
        src.S->bar_count = 0u;
        src.S->tile_ctr[0] = src.S->tile_ctr[1] = 0u;
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
    int loop_grid = 0;   // CTAs of the persistent CG launch (0: the device cannot hold the SpMV grid at once)
    int persistent = 1;  // CG: run iterations as one cooperative launch when loop_grid > 0
    const float* st_S = nullptr;  // flexible solver: 27-point stencil form of A for its product (or null)
    St27Grid st_g = {};
    int st_grid = 0;
};

static bool use_loop(const Solver* s) { return s->kind == KRYLOV_CG && s->persistent && s->loop_grid > 0; }

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
    L.nvec = (kind == KRYLOV_CG) ? 3 : (kind == KRYLOV_FCG ? 5 : 7);  // CG: r p Ap; FCG: + z Az; BiCGSTAB: 7
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
        cudaFuncSetAttribute(k_cg_loop<BR, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->spmv_smem);
    }
    // the persistent CG needs every CTA resident at once: as many as the device holds, at most the
    // SpMV's own grid
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cg_loop<BR, VT>, SPMV_THREADS, s->spmv_smem) !=
        cudaSuccess) {
        (void)cudaGetLastError();
        per_sm = 0;
    }
    int coop = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        coop = 0;
    }
    s->loop_grid = coop ? std::min(s->spmv_grid, per_sm * sm_count()) : 0;
}

// One cooperative launch of the persistent CG: at most max_iters iterations (0: until the loop
// condition clears).
template <int BR, typename VT> static int launch_loop_t(Solver* s, cudaStream_t st, int max_iters)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)s->loop_grid);
    cfg.blockDim = dim3(SPMV_THREADS);
    cfg.dynamicSmemBytes = s->spmv_smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_CHECK_CUDA(cudaLaunchKernelEx(&cfg, k_cg_loop<BR, VT>, (const SolveArgs*)s->d_args, s->nrow, s->sh, max_iters));
    return GB_OK;
}

static int launch_loop(Solver* s, cudaStream_t st, int max_iters)
{
    if (s->br == 1) return s->val_dtype == GB_BF16 ? launch_loop_t<1, __nv_bfloat16>(s, st, max_iters)
                                                   : launch_loop_t<1, float>(s, st, max_iters);
    return s->val_dtype == GB_BF16 ? launch_loop_t<3, __nv_bfloat16>(s, st, max_iters)
                                   : launch_loop_t<3, float>(s, st, max_iters);
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
        if (s->st_S) {
            GB_CHECK_CUDA(launch_pdl(k_fcg_st27_az, s->st_grid, ST_TILE, st27_smem<float>(), st, s->d_args, s->st_g,
                                     s->st_S, h, has_cond));
            GB_CHECK_CUDA(launch_pdl(k_fcg_update, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
        } else {
            GB_CHECK_CUDA(launch_pdl(k_fcg_dir, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
            GB_CHECK_CUDA(launch_pdl(k_fcg_p, s->vec_grid, VEC_THREADS, 0, st, s->d_args));
            GB_CHECK_CUDA(launch_pdl(k_cg_spmv<BR, VT>, s->spmv_grid, SPMV_THREADS, s->spmv_smem, st, s->d_args,
                                     s->nrow, s->sh));
            GB_CHECK_CUDA(launch_pdl(k_cg_update, s->vec_grid, VEC_THREADS, 0, st, s->d_args, h, has_cond));
        }
    } else if (s->kind == KRYLOV_CG && use_loop(s)) {
        return launch_loop(s, st, 1);
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
    if (use_loop(s)) {  // init, then the whole loop in one launch: no conditional node needed
        int rc = launch_init(s, st, 0, 0);
        if (rc) return rc;
        return launch_loop(s, st, 0);
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
        if (use_loop(s)) rc = launch_loop(s, s->cap_stream, chunk_iters);
        else
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
        if (kind == KRYLOV_FCG) {
            s->host.z = vecs[3];
            s->host.v = vecs[4];  // A z (the stencil-form step)
        }
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
        if (use_loop(s)) return chunk_iters > 0 ? launch_loop(s, stream, chunk_iters) : GB_OK;
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

// CG only: enable (1, the default) or disable (0) running the iterations as one persistent
// cooperative launch (used when the device holds the whole SpMV grid at once); 0 keeps the three
// kernels per iteration under a conditional graph node.  Drops any cached graphs.  Returns, through
// active_out (may be null), whether the persistent launch will be used.
GB_API int gb_krylov_set_persistent(void* handle, int enable, int* active_out)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s, "krylov_set_persistent: null handle");
    s->persistent = enable ? 1 : 0;
    if (s->exec_while) cudaGraphExecDestroy(s->exec_while);
    if (s->exec_init) cudaGraphExecDestroy(s->exec_init);
    if (s->exec_chunk) cudaGraphExecDestroy(s->exec_chunk);
    s->exec_while = s->exec_init = s->exec_chunk = nullptr;
    s->chunk_iters = 0;
    if (active_out) *active_out = use_loop(s) ? 1 : 0;
    return GB_OK;
}

// Flexible solver with 1x1 blocks on an nx x ny x nz node grid: use the 27-point stencil form S of A
// (node-major fp32 coefficients, gb_st27_build / gb_st27_bytes, 16-byte aligned; the caller keeps it
// alive and equal to A) for the product of every iteration; S = null returns to the CSR product.
// Drops any cached graphs.
GB_API int gb_krylov_set_stencil(void* handle, int nx, int ny, int nz, const float* S)
{
    Solver* s = static_cast<Solver*>(handle);
    GB_REQUIRE(s && s->kind == KRYLOV_FCG, "krylov_set_stencil: flexible solver handle required");
    if (S) {
        GB_REQUIRE(s->br == 1, "krylov_set_stencil: 1x1 blocks required");
        GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1 && (int64_t)nx * ny * nz == (int64_t)s->nrow,
                   "krylov_set_stencil: grid %dx%dx%d does not match %d rows", nx, ny, nz, s->nrow);
        GB_REQUIRE((uintptr_t)S % 16 == 0, "krylov_set_stencil: S must be 16-byte aligned");
        static bool attr_set = false;
        if (!attr_set) {
            GB_CHECK_CUDA(cudaFuncSetAttribute(k_fcg_st27_az, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)st27_smem<float>()));
            attr_set = true;
        }
        s->st_g = St27Grid{nx, ny, nz, (int64_t)nx * ny * nz};
        s->st_grid = (int)std::max<int64_t>(
            1, std::min<int64_t>(ceil_div<int64_t>(s->st_g.n, ST_TILE), (int64_t)sm_count() * St27Coef<float>::ctas_per_sm));
    }
    s->st_S = S;
    if (s->exec_while) cudaGraphExecDestroy(s->exec_while);
    if (s->exec_init) cudaGraphExecDestroy(s->exec_init);
    if (s->exec_chunk) cudaGraphExecDestroy(s->exec_chunk);
    s->exec_while = s->exec_init = s->exec_chunk = nullptr;
    s->chunk_iters = 0;
    return GB_OK;
}
