// gb_conv_tc.cu -- the learned smoother's 3x3x3 convolution layers as a tcgen05 implicit GEMM.
//
// No reference counterpart (Warp's preconditioners are Jacobi only).
//
// Planar padded activation layout: the node grid is padded by one zero voxel on every side,
// (nx+2) x (ny+2) x (nz+2), padded row p = ((x+1)(ny+2) + (y+1))(nz+2) + (z+1); channels 0-7 of
// every row live in plane 0 and channels 8-15 in plane 1, 16 bytes (8 bf16) per row:
//     byte address of (plane h, row p) = base + (h * plane_rows + p) * 16.
// Border rows are zero and stay zero (no kernel writes them); plane_rows = P + 640 leaves room for
// the reads past the last tile.  The tap (dx, dy, dz) of output row p is input row
// p + dx sx + dy sy + dz (sx = (ny+2)(nz+2), sy = nz+2).
//
// The dz taps are folded into the GEMM's N dimension: for 128 consecutive rows q,
//     Z[q][dz][co] = sum_{dx,dy} sum_ci in[q + dx sx + dy sy][ci] W[dx,dy,dz][ci][co]
// is 9 MMAs (one per (dx, dy); M = 128 rows, N = 48 = 3 dz x 16 co, K = 16 channels), each A
// operand being 128 consecutive staged rows -- a K-major, non-swizzled UMMA operand (8-row core
// matrices 128 B apart, the two 8-channel halves one plane apart) -- and then
//     out[p] = Z[p-1][-1] + Z[p][0] + Z[p+1][+1]
// for the 126 rows whose neighbours lie in the same 128-row window (lane shuffles, plus one value
// exchanged between neighbouring epilogue warps).
//
// A stage covers TC_SUB = 4 such windows (504 output rows): for each dx, rows
// [q0 + dx sx - sy, q0 + dx sx + sy + 126*3 + 128) of both planes are staged with 1-D bulk copies
// (6 copies) into a 2-3 stage ring; one MMA thread issues the 36 MMAs (dx, dy)-major so the four
// windows' accumulators (4 x 48 TMEM columns, two slots) form independent chains; four epilogue
// warps read them with tcgen05.ld (each warp its 32-lane quarter), sum the dz taps, apply ReLU and
// store bf16 rows of interior voxels -- or, for the last layer, write
// w[v] = omega dinv[v] r[v] + (mask[v] ? 0 : out[v][0]) in fp32 (the Jacobi step fused).
// Every wait is bounded (globaltimer); a timeout sets GB_DEV_WAIT_TIMEOUT, the CTA drains its own
// copies and MMAs (bounded) and frees its TMEM before returning.
#include "gb_bulk.cuh"
#include "gb_common.cuh"
#include "gb_spmv.cuh"  // sm_count()

namespace gb {

constexpr int TC_M = 128;                  // rows of one window (UMMA M)
constexpr int TC_OUT = TC_M - 2;           // output rows per window
constexpr int TC_SUB = 4;                  // windows per work item (504 output rows of one x-slab)
constexpr int TC_N = 48;                   // 3 dz taps x 16 output channels (UMMA N)
constexpr int TC_ISSUERS = TC_SUB;         // one MMA-issuing warp per window
constexpr int TC_EPI_GROUPS = 2;           // epilogue groups of 4 warps (one per TMEM lane quarter)
constexpr int TC_EPI_WARP0 = 1 + TC_ISSUERS;  // warp 0 copies, warps 1..4 issue MMAs, then the epilogue
constexpr int TC_THREADS = 32 * TC_EPI_WARP0 + TC_EPI_GROUPS * 128;
constexpr uint32_t TC_TMEM_COLS = 512;     // 2 slots x 4 windows x 48 columns = 384, rounded up
constexpr int TC_W_BYTES = 9 * 1536;       // per (dx, dy): [k-half][dz 3 x co 16][8 ci] bf16
constexpr int TC_WPG = TC_SUB / TC_EPI_GROUPS;  // windows per epilogue group per item (drained together)
constexpr int TC_XCHG_BYTES = TC_EPI_GROUPS * 2 * TC_WPG * 4 * 2 * 16 * 4;  // [group][parity][window][quarter][lo/hi][16]
constexpr int TC_MAX_SLOTS = 8;            // x-plane blocks in the shared-memory ring
constexpr int TC_MIN_SLOTS = 4;            // three in use (x-1, x, x+1) plus one in flight
constexpr size_t TC_SMEM_LIMIT = 220 * 1024;
constexpr int TC_BAR_PROLOGUE = 2 + TC_EPI_GROUPS;  // named barriers: 0 CTA, 1..groups epilogue groups,
                                                    // 1 + groups all epilogue warps, then the prologue

// Division by a loop-invariant divisor with a multiply and shifts (Granlund and Montgomery, "Division
// by invariant integers using multiplication", PLDI 1994, figure 4.1): exact for every 32-bit n.
struct FastDivU32 {
    uint32_t m, s1, s2;
};

static inline FastDivU32 make_fastdiv(uint32_t d)
{
    uint32_t l = 0;
    while (l < 32 && (uint64_t(1) << l) < d) ++l;  // l = ceil(log2 d)
    const uint64_t m = ((((uint64_t)1 << l) - d) << 32) / d + 1;
    return FastDivU32{(uint32_t)m, l ? 1u : 0u, l ? l - 1 : 0u};
}

__device__ __forceinline__ uint32_t fastdiv(uint32_t n, FastDivU32 f)
{
    const uint32_t t = __umulhi(f.m, n);
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

struct TcConv {
    int nx, ny, nz;
    FastDivU32 div_sx, div_sy;  // row -> (x, y, z) of the padded grid
    int sy;              // nz + 2
    int slots;           // x-plane blocks in the ring
    int ncols;           // work items per x-slab (columns of TC_SUB * TC_OUT rows)
    int64_t sx;          // (ny + 2) * (nz + 2)
    int64_t nitems;      // ncols * nx; item k = (column k / nx, x = 1 + k % nx)
    int64_t plane_rows;  // rows per plane (plane stride)
    uint32_t rows_bytes; // R * 16, R = 2 sy + TC_OUT (TC_SUB - 1) + TC_M
    uint32_t block_bytes;  // 2 * rows_bytes: one x-plane block, both channel planes
    const unsigned char* in;
    const __nv_bfloat16* Wt;  // [27][16 co][16 ci] bf16
    unsigned char* out;       // hidden layers: planar padded bf16
    float* w;                 // last layer: fp32 [n]
    const float* r;
    const float* dinv;
    const float* mask;
    float omega;
    int* status;
};

__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    // start address, leading (K) byte offset, stride (M/N) byte offset, all >> 4; version 1 (bit 46);
    // base offset 0, no swizzle.
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D fp32, A and B bf16, both K-major, N >> 3, M >> 4.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive1(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ float tc_ld1(uint32_t taddr)
{
    uint32_t r;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr));
    return __uint_as_float(r);
}

// bounded wait that also gives up when another role has aborted
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

// named barriers (non-aligned form: lanes may arrive after divergent code): id 1 + group for the four
// warps of one epilogue group, id 1 + TC_EPI_GROUPS for all epilogue warps
__device__ __forceinline__ void epi_group_barrier(int group)
{
    asm volatile("barrier.sync %0, 128;" ::"r"(1 + group) : "memory");
}
__device__ __forceinline__ void epi_all_barrier()
{
    asm volatile("barrier.sync %0, %1;" ::"r"(1 + TC_EPI_GROUPS), "r"(TC_EPI_GROUPS * 128) : "memory");
}

template <bool LAST>
__global__ void __launch_bounds__(TC_THREADS, 1) k_conv3_tc(const TcConv c)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    pdl_enter();
    unsigned char* ring = smem;
    unsigned char* wsm = smem + (size_t)c.slots * c.block_bytes;
    float* xchg = reinterpret_cast<float*>(wsm + TC_W_BYTES);  // [group][parity][window][quarter][lo/hi][16]
    uint64_t* full = reinterpret_cast<uint64_t*>(wsm + TC_W_BYTES + TC_XCHG_BYTES);
    uint64_t* empty = full + TC_MAX_SLOTS;
    uint64_t* accfull = empty + TC_MAX_SLOTS;
    uint64_t* accempty = accfull + 2;
    uint64_t* done = accempty + 2;  // every issuer's last commit: all MMAs of the CTA completed
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
    volatile int* s_issued = s_abort + 1;      // x-plane blocks whose copies were issued
    volatile int* s_epi_abort = s_issued + 1;  // written by epilogue warps only, read after their barrier
    const int NS = c.slots;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // contiguous range of work items; consecutive items of one column differ by one x-slab, so the
    // blocks x and x+1 of an item are the blocks x-1 and x of the next one
    const int64_t k_begin = (int64_t)blockIdx.x * c.nitems / gridDim.x;
    const int64_t k_end = (int64_t)(blockIdx.x + 1) * c.nitems / gridDim.x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], TC_ISSUERS);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&accfull[a], TC_ISSUERS);
            mbar_init(&accempty[a], 4 * TC_EPI_GROUPS);
        }
        mbar_init(done, TC_ISSUERS);
        *s_abort = 0;
        *s_issued = 0;
        *s_epi_abort = 0;
        fence_mbar_init();
    }
    uint32_t tmem = 0;
    if (warp == 0) {
        // the copy warp needs only the barriers: it starts filling the ring while the other warps
        // stage the weights and allocate TMEM
        __syncwarp();
        __threadfence_block();  // the barrier words and flags written by thread 0 before the arrival
        asm volatile("bar.arrive %0, %1;" ::"r"(TC_BAR_PROLOGUE), "r"(TC_THREADS) : "memory");
    } else {
        // weights -> B operands: (dx, dy) pair g, k-half kc, row n = 16 dz_idx + co at g*1536 + kc*768 + n*16
        for (int i = threadIdx.x - 32; i < 27 * 16 * 2; i += blockDim.x - 32) {
            const int t = i >> 5, co = (i >> 1) & 15, kc = i & 1;
            const int g = t / 3, dzi = t % 3;
            const uint4 v = reinterpret_cast<const uint4*>(c.Wt)[(t * 16 + co) * 2 + kc];
            *reinterpret_cast<uint4*>(wsm + g * 1536 + kc * 768 + (dzi * 16 + co) * 16) = v;
        }
        fence_proxy_async_shared();  // make the generic-proxy stores visible to the tensor cores
        if (warp == 1) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                         "r"(TC_TMEM_COLS)
                         : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
        tc_fence_before();
        asm volatile("bar.sync %0, %1;" ::"r"(TC_BAR_PROLOGUE), "r"(TC_THREADS) : "memory");
        tc_fence_after();
        tmem = *s_tmem;
    }

    if (warp == 0) {
        // ------------------------- copy warp: x-plane blocks into the ring ----------------------------
        if (lane == 0) {
            int q = 0;  // sequence number of the next block; its slot is q % NS
            bool ok = true;
            for (int64_t k = k_begin; k < k_end && ok;) {
                const int o = (int)(k / c.nx);
                const int x0 = (int)(k % c.nx) + 1;
                const int64_t run_end = min(k_end, (int64_t)(o + 1) * c.nx);
                const int x1 = (int)((run_end - 1) % c.nx) + 1;
                for (int xb = x0 - 1; xb <= x1 + 1; ++xb, ++q) {
                    const int s = q % NS;
                    if (q >= NS && !tc_wait(&empty[s], ((q / NS) - 1) & 1, s_abort)) {
                        *s_abort = 1;
                        ok = false;
                        break;
                    }
                    if (*s_abort) {
                        ok = false;
                        break;
                    }
                    const int64_t row = (int64_t)xb * c.sx + (int64_t)o * (TC_SUB * TC_OUT);
                    unsigned char* dst = ring + (size_t)s * c.block_bytes;
                    mbar_arrive_expect_tx(&full[s], c.block_bytes);
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        bulk_g2s(dst + h * c.rows_bytes, c.in + ((int64_t)h * c.plane_rows + row) * 16, c.rows_bytes,
                                 &full[s]);
                    *s_issued = q + 1;
                }
                k = run_end;
            }
        }
    } else if (warp <= TC_ISSUERS) {
        // ------------- MMA warps: warp 1 + j issues the 9 (dx, dy) MMAs of window j --------------------
        if (lane == 0) {
            const int j = warp - 1;
            const uint32_t wbase = smem_u32(wsm);
            const uint32_t rbase = smem_u32(ring);
            int it = 0;  // items of this CTA so far (TMEM slot it & 1)
            int q0 = 0;  // sequence number of the current run's first block (x0 - 1)
            bool ok = true;
            for (int64_t k = k_begin; k < k_end && ok;) {
                const int o = (int)(k / c.nx);
                const int64_t run_end = min(k_end, (int64_t)(o + 1) * c.nx);
                const int run = (int)(run_end - k);
                for (int t = 0; t < run; ++t, ++it) {
                    const int a = it & 1;
                    // blocks q0+t (x-1), q0+t+1 (x), q0+t+2 (x+1); the earlier item of the run waited for the first two
                    for (int d = (t == 0 ? 0 : 2); d < 3 && ok; ++d) {
                        const int q = q0 + t + d;
                        ok = tc_wait(&full[q % NS], (q / NS) & 1, s_abort);
                    }
                    if (ok && it >= 2) ok = tc_wait(&accempty[a], ((it >> 1) & 1) ^ 1, s_abort);
                    if (!ok) {
                        *s_abort = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dcol = tmem + (uint32_t)((a * TC_SUB + j) * TC_N);
#pragma unroll
                    for (int g = 0; g < 9; ++g) {
                        const int b = g / 3, dyi = g % 3;
                        const uint32_t arow = rbase + (uint32_t)((q0 + t + b) % NS) * c.block_bytes +
                                              (uint32_t)(dyi * c.sy + j * TC_OUT) * 16u;
                        tc_mma(dcol, umma_desc(arow, c.rows_bytes, 128), umma_desc(wbase + g * 1536, 768, 128),
                               kTcIdesc, g > 0 ? 1u : 0u);
                    }
                    // x-1 is not read again in this run; after the run's last item neither are x and x+1
                    tc_commit(&empty[(q0 + t) % NS]);
                    if (t == run - 1) {
                        tc_commit(&empty[(q0 + t + 1) % NS]);
                        tc_commit(&empty[(q0 + t + 2) % NS]);
                    }
                    tc_commit(&accfull[a]);
                }
                q0 += run + 2;
                k = run_end;
            }
            tc_commit(done);  // arrives once every MMA this thread issued has completed
        }
    } else {
        // --------------------------------- epilogue warps --------------------------------------------
        const int quarter = warp & 3;                   // TMEM lanes 32*quarter .. +31 belong to this warp
        const int group = (warp - TC_EPI_WARP0) >> 2;   // windows group, group + TC_EPI_GROUPS, ...
        const int i = quarter * 32 + lane;              // row of the 128-row window
        const uint32_t usx = (uint32_t)c.sx, usy = (uint32_t)c.sy;
        float* xg = xchg + group * (2 * TC_WPG * 4 * 2 * 16);
        int it = 0;
        int xp = 0;  // exchange buffer parity
        for (int64_t k = k_begin; k < k_end; ++k, ++it) {
            const int a = it & 1;
            const uint32_t xk = (uint32_t)(k % c.nx) + 1u;
            // row of lane 0 of window 0: one row before the item's first output row
            const uint32_t q0 = xk * usx + usy + (uint32_t)(k / c.nx) * (uint32_t)(TC_SUB * TC_OUT);
            int ok = 1;
            if (lane == 0) ok = tc_wait(&accfull[a], (it >> 1) & 1, s_abort) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok && lane == 0) *s_epi_abort = 1;
            // all epilogue warps decide together: the flag only changes before this barrier
            epi_all_barrier();
            if (*s_epi_abort) {
                if (lane == 0) *s_abort = 1;
                break;
            }
            tc_fence_after();
            __syncwarp();
            // this group's windows j = group + w * TC_EPI_GROUPS are drained together: all TMEM loads,
            // one exchange of the quarter-boundary rows, one barrier, then the outputs
            float* xb = xg + xp * (TC_WPG * 4 * 2 * 16);
            uint32_t taddr[TC_WPG];
            bool valid[TC_WPG];
            uint32_t prow[TC_WPG];
            int64_t vox[TC_WPG];
#pragma unroll
            for (int w = 0; w < TC_WPG; ++w) {
                const int j = group + w * TC_EPI_GROUPS;
                taddr[w] = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((a * TC_SUB + j) * TC_N);
                // voxel of row p (rows < 2^31: checked on the host); rows of the next x-slab belong to
                // the next item of the column
                const uint32_t up = q0 + (uint32_t)(j * TC_OUT + i);
                const uint32_t xq = fastdiv(up, c.div_sx);
                const uint32_t rem = up - xq * usx;
                const uint32_t yq = fastdiv(rem, c.div_sy);
                const uint32_t zq = rem - yq * usy;
                prow[w] = up;
                valid[w] = i >= 1 && i <= TC_OUT && xq == xk && yq - 1u < (uint32_t)c.ny && zq - 1u < (uint32_t)c.nz;
                vox[w] = ((int64_t)(xq - 1) * c.ny + (yq - 1)) * (int64_t)c.nz + (zq - 1);
            }
            if (LAST) {
                float zm[TC_WPG], z0[TC_WPG], zp[TC_WPG];
#pragma unroll
                for (int w = 0; w < TC_WPG; ++w) {
                    zm[w] = tc_ld1(taddr[w]);
                    z0[w] = tc_ld1(taddr[w] + 16);
                    zp[w] = tc_ld1(taddr[w] + 32);
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int w = 0; w < TC_WPG; ++w) {
                    if (lane == 31) xb[((w * 4 + quarter) * 2 + 0) * 16] = zm[w];
                    if (lane == 0) xb[((w * 4 + quarter) * 2 + 1) * 16] = zp[w];
                }
                epi_group_barrier(group);
#pragma unroll
                for (int w = 0; w < TC_WPG; ++w) {
                    float lo = __shfl_up_sync(0xffffffffu, zm[w], 1);
                    float hi = __shfl_down_sync(0xffffffffu, zp[w], 1);
                    if (lane == 0 && quarter > 0) lo = xb[((w * 4 + quarter - 1) * 2 + 0) * 16];
                    if (lane == 31 && quarter < 3) hi = xb[((w * 4 + quarter + 1) * 2 + 1) * 16];
                    if (valid[w]) {
                        const int64_t v = vox[w];
                        float o = lo + z0[w] + hi;
                        if (c.mask && c.mask[v] != 0.f) o = 0.f;
                        if (c.dinv) o += c.omega * c.dinv[v] * c.r[v];
                        c.w[v] = o;
                    }
                }
            } else {
                float zm[TC_WPG][16], z0[TC_WPG][16], zp[TC_WPG][16];
#pragma unroll
                for (int w = 0; w < TC_WPG; ++w) {
                    tc_ld16(taddr[w], zm[w]);
                    tc_ld16(taddr[w] + 16, z0[w]);
                    tc_ld16(taddr[w] + 32, zp[w]);
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int w = 0; w < TC_WPG; ++w) {
                    float4* lo_dst = reinterpret_cast<float4*>(xb + ((w * 4 + quarter) * 2 + 0) * 16);
                    float4* hi_dst = reinterpret_cast<float4*>(xb + ((w * 4 + quarter) * 2 + 1) * 16);
                    if (lane == 31) {
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            lo_dst[q] = make_float4(zm[w][4 * q], zm[w][4 * q + 1], zm[w][4 * q + 2], zm[w][4 * q + 3]);
                    }
                    if (lane == 0) {
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            hi_dst[q] = make_float4(zp[w][4 * q], zp[w][4 * q + 1], zp[w][4 * q + 2], zp[w][4 * q + 3]);
                    }
                }
                epi_group_barrier(group);
#pragma unroll
                for (int w = 0; w < TC_WPG; ++w) {
                    float lo[16], hi[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        lo[q] = __shfl_up_sync(0xffffffffu, zm[w][q], 1);
                        hi[q] = __shfl_down_sync(0xffffffffu, zp[w][q], 1);
                    }
                    if (lane == 0 && quarter > 0) {
                        const float4* src = reinterpret_cast<const float4*>(xb + ((w * 4 + quarter - 1) * 2 + 0) * 16);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float4 v = src[q];
                            lo[4 * q] = v.x; lo[4 * q + 1] = v.y; lo[4 * q + 2] = v.z; lo[4 * q + 3] = v.w;
                        }
                    }
                    if (lane == 31 && quarter < 3) {
                        const float4* src = reinterpret_cast<const float4*>(xb + ((w * 4 + quarter + 1) * 2 + 1) * 16);
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const float4 v = src[q];
                            hi[4 * q] = v.x; hi[4 * q + 1] = v.y; hi[4 * q + 2] = v.z; hi[4 * q + 3] = v.w;
                        }
                    }
                    if (valid[w]) {
                        uint32_t pk[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const __nv_bfloat162 h2 =
                                __floats2bfloat162_rn(fmaxf(lo[2 * q] + z0[w][2 * q] + hi[2 * q], 0.f),
                                                      fmaxf(lo[2 * q + 1] + z0[w][2 * q + 1] + hi[2 * q + 1], 0.f));
                            pk[q] = *reinterpret_cast<const uint32_t*>(&h2);
                        }
                        const int64_t p = prow[w];
                        *reinterpret_cast<uint4*>(c.out + p * 16) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                        *reinterpret_cast<uint4*>(c.out + (c.plane_rows + p) * 16) =
                            make_uint4(pk[4], pk[5], pk[6], pk[7]);
                    }
                }
            }
            xp ^= 1;
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive1(&accempty[a]);
        }
    }

    // teardown: every MMA finished and every copy landed before shared memory and TMEM go away
    __syncthreads();
    if (threadIdx.x == 32) {
        bool ok = mbar_wait_bounded(done, 0);
        const int issued = *s_issued;
        // the last NS blocks occupy distinct slots; earlier fills of a slot were consumed before reuse
        for (int q = issued > NS ? issued - NS : 0; q < issued; ++q)
            ok = mbar_wait_bounded(&full[q % NS], (q / NS) & 1) && ok;
        if (!ok || *s_abort) atomicOr(c.status, GB_DEV_WAIT_TIMEOUT);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// features in the planar padded bf16 layout (interior rows only)
__global__ void k_features_planar(int nx, int ny, int nz, int64_t plane_rows, const float* __restrict__ r,
                                  const float* __restrict__ dinv, const float* __restrict__ chat,
                                  const float* __restrict__ mask, unsigned char* __restrict__ out)
{
    pdl_enter();
    const int64_t n = (int64_t)nx * ny * nz;
    const int64_t sy = nz + 2, sx = (int64_t)(ny + 2) * sy;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(v / ((int64_t)ny * nz));
        const int y = (int)((v / nz) % ny);
        const int z = (int)(v % nz);
        const int64_t p = (x + 1) * sx + (y + 1) * sy + (z + 1);
        const float xm = (mask && mask[v] != 0.f) ? 0.f : dinv[v] * r[v];
        float f[16];
        f[0] = xm;
#pragma unroll
        for (int k = 0; k < 8; ++k) f[1 + k] = xm * chat[v * 8 + k];
#pragma unroll
        for (int k = 9; k < 16; ++k) f[k] = 0.f;
        uint32_t pk[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const __nv_bfloat162 h2 = __floats2bfloat162_rn(f[2 * k], f[2 * k + 1]);
            pk[k] = *reinterpret_cast<const uint32_t*>(&h2);
        }
        *reinterpret_cast<uint4*>(out + p * 16) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        *reinterpret_cast<uint4*>(out + (plane_rows + p) * 16) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
    }
}

static int64_t planar_rows(int nx, int ny, int nz)
{
    const int64_t P = (int64_t)(nx + 2) * (ny + 2) * (nz + 2);
    return (P + 640 + 7) / 8 * 8;
}

}  // namespace gb

using namespace gb;

GB_API int64_t gb_conv3_planar_rows(int nx, int ny, int nz) { return planar_rows(nx, ny, nz); }

GB_API int gb_net_features_planar(int nx, int ny, int nz, const float* r, const float* dinv, const float* chat,
                                  const float* mask, void* out, cudaStream_t stream)
{
    const int64_t n = (int64_t)nx * ny * nz;
    if (n <= 0) return GB_OK;
    GB_REQUIRE((uintptr_t)out % 16 == 0, "net_features_planar: output must be 16-byte aligned");
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(n, 256), kSmCount * 16));
    GB_CHECK_CUDA(launch_pdl(k_features_planar, grid, 256, 0, stream, nx, ny, nz, planar_rows(nx, ny, nz), r, dinv,
                             chat, mask, static_cast<unsigned char*>(out)));
    return GB_OK;
}

// One 16 -> 16 layer (last = 0: ReLU, planar bf16 output) or the last layer (last = 1: output channel 0
// only, w = omega dinv r + (mask ? 0 : out) in fp32).  in/out: planar padded bf16 buffers of
// 2 * gb_conv3_planar_rows() rows of 16 bytes whose border rows are zero; Wt: [27][16][16] bf16.
GB_API int gb_conv3_fwd_tc(int nx, int ny, int nz, int last, const void* in, const void* Wt, void* out, float* w,
                           const float* r, const float* dinv, const float* mask, float omega, int* status,
                           cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1, "conv3_fwd_tc: empty grid");
    GB_REQUIRE((uintptr_t)in % 16 == 0 && (uintptr_t)Wt % 16 == 0, "conv3_fwd_tc: in/Wt must be 16-byte aligned");
    GB_REQUIRE(last ? (w != nullptr && (dinv == nullptr || r != nullptr)) : (out != nullptr && (uintptr_t)out % 16 == 0),
               "conv3_fwd_tc: missing output");
    GB_REQUIRE(status != nullptr, "conv3_fwd_tc: status word required");
    TcConv c{};
    c.nx = nx;
    c.ny = ny;
    c.nz = nz;
    c.sy = nz + 2;
    c.sx = (int64_t)(ny + 2) * (nz + 2);
    c.div_sx = make_fastdiv((uint32_t)c.sx);
    c.div_sy = make_fastdiv((uint32_t)c.sy);
    // work items: columns of TC_SUB * TC_OUT rows covering an x-slab's interior rows (y = 1, z = 1 up
    // to y = ny, z = nz), times the nx slabs
    const int64_t span = (int64_t)(ny - 1) * c.sy + nz;
    c.ncols = (int)ceil_div<int64_t>(span, TC_SUB * TC_OUT);
    c.nitems = (int64_t)c.ncols * nx;
    c.plane_rows = planar_rows(nx, ny, nz);
    GB_REQUIRE(c.plane_rows < (int64_t(1) << 31), "conv3_fwd_tc: grid too large (padded rows must fit in 31 bits)");
    const int64_t rows = 2 * (int64_t)c.sy + TC_OUT * (TC_SUB - 1) + TC_M;
    // the last block read (x = nx + 1, last column) must end inside the padded planes
    GB_REQUIRE((int64_t)(nx + 1) * c.sx + (int64_t)(c.ncols - 1) * (TC_SUB * TC_OUT) + rows <= c.plane_rows,
               "conv3_fwd_tc: planar padding too small");
    c.rows_bytes = (uint32_t)(rows * 16);
    c.block_bytes = 2 * c.rows_bytes;
    const size_t fixed = TC_W_BYTES + TC_XCHG_BYTES + 256;
    c.slots = (int)std::min<size_t>(TC_MAX_SLOTS, (TC_SMEM_LIMIT - fixed) / c.block_bytes);
    if (c.slots < TC_MIN_SLOTS) {
        gb::set_error("conv3_fwd_tc: grid too long in z (nz = %d) for the staged x-plane blocks", nz);
        return GB_ERR_UNSUPPORTED;
    }
    const size_t smem = (size_t)c.slots * c.block_bytes + fixed;
    c.in = static_cast<const unsigned char*>(in);
    c.Wt = static_cast<const __nv_bfloat16*>(Wt);
    c.out = static_cast<unsigned char*>(out);
    c.w = w;
    c.r = r;
    c.dinv = dinv;
    c.mask = mask;
    c.omega = omega;
    c.status = status;
    // one-time per process: the largest dynamic shared memory either variant may use
    static bool attr_set = false;
    if (!attr_set) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_conv3_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)TC_SMEM_LIMIT));
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_conv3_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)TC_SMEM_LIMIT));
        attr_set = true;
    }
    // one CTA per SM: it holds all 512 TMEM columns
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(c.nitems, (int64_t)sm_count()));
    if (last)
        GB_CHECK_CUDA(launch_pdl(k_conv3_tc<true>, grid, TC_THREADS, smem, stream, c));
    else
        GB_CHECK_CUDA(launch_pdl(k_conv3_tc<false>, grid, TC_THREADS, smem, stream, c));
    return GB_OK;
}
