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

namespace gb {

constexpr int TC_M = 128;                  // rows of one window (UMMA M)
constexpr int TC_OUT = TC_M - 2;           // output rows per window
constexpr int TC_SUB = 4;                  // windows per stage
constexpr int TC_N = 48;                   // 3 dz taps x 16 output channels (UMMA N)
constexpr int TC_EPI_GROUPS = 2;           // epilogue groups of 4 warps (one per TMEM lane quarter)
constexpr int TC_THREADS = 64 + TC_EPI_GROUPS * 128;  // warp 0 copies, warp 1 MMA, warps 2.. epilogue
constexpr uint32_t TC_TMEM_COLS = 512;     // 2 slots x 4 windows x 48 columns = 384, rounded up
constexpr int TC_W_BYTES = 9 * 1536;       // per (dx, dy): [k-half][dz 3 x co 16][8 ci] bf16
constexpr int TC_XCHG_BYTES = TC_EPI_GROUPS * 2 * 4 * 2 * 16 * 4;
constexpr int TC_MAX_STAGES = 3;

struct TcConv {
    int nx, ny, nz;
    int sy;              // nz + 2
    int stages;
    int64_t sx;          // (ny + 2) * (nz + 2)
    int64_t p_begin;     // first interior row
    int64_t ntiles;      // stage tiles of TC_SUB * TC_OUT output rows
    int64_t plane_rows;  // rows per plane (plane stride)
    uint32_t rows_bytes; // R * 16, R = 2 sy + TC_OUT (TC_SUB - 1) + TC_M
    uint32_t stage_bytes;  // 6 * rows_bytes
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
    if (mbar_test_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        if (mbar_test_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
        __nanosleep(32);
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
    unsigned char* stages = smem;
    unsigned char* wsm = smem + (size_t)c.stages * c.stage_bytes;
    float* xchg = reinterpret_cast<float*>(wsm + TC_W_BYTES);  // [parity][quarter][lo/hi][16]
    uint64_t* full = reinterpret_cast<uint64_t*>(wsm + TC_W_BYTES + TC_XCHG_BYTES);
    uint64_t* empty = full + TC_MAX_STAGES;
    uint64_t* accfull = empty + TC_MAX_STAGES;
    uint64_t* accempty = accfull + 2;
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(accempty + 2);
    volatile int* s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
    volatile int* s_counts = s_abort + 1;  // [0] copies issued, [1] tiles taken by MMA, [2] tiles committed
    volatile int* s_epi_abort = s_counts + 3;  // written by epilogue warps only, read after their barrier
    const int S = c.stages;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&accfull[a], 1);
            mbar_init(&accempty[a], 4 * TC_EPI_GROUPS);
        }
        *s_abort = 0;
        *s_epi_abort = 0;
        s_counts[0] = s_counts[1] = s_counts[2] = 0;
        fence_mbar_init();
    }
    // weights -> B operands: (dx, dy) pair g, k-half kc, row n = 16 dz_idx + co at g*1536 + kc*768 + n*16
    for (int i = threadIdx.x; i < 27 * 16 * 2; i += blockDim.x) {
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
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            for (int64_t tile = blockIdx.x; tile < c.ntiles; tile += gridDim.x, ++it) {
                const int s = it % S;
                if (it >= S && !tc_wait(&empty[s], ((it / S) & 1) ^ 1, s_abort)) {
                    *s_abort = 1;
                    break;
                }
                if (*s_abort) break;
                const int64_t q0 = c.p_begin + tile * (TC_SUB * TC_OUT) - 1;
                unsigned char* dst = stages + (size_t)s * c.stage_bytes;
                mbar_arrive_expect_tx(&full[s], c.stage_bytes);
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    const int64_t row = q0 + (int64_t)(b - 1) * c.sx - c.sy;
#pragma unroll
                    for (int h = 0; h < 2; ++h)
                        bulk_g2s(dst + (b * 2 + h) * c.rows_bytes, c.in + ((int64_t)h * c.plane_rows + row) * 16,
                                 c.rows_bytes, &full[s]);
                }
                s_counts[0] = it + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t wbase = smem_u32(wsm);
            int it = 0;
            for (int64_t tile = blockIdx.x; tile < c.ntiles; tile += gridDim.x, ++it) {
                const int s = it % S;
                const int a = it & 1;
                if (!tc_wait(&full[s], (it / S) & 1, s_abort)) {
                    *s_abort = 1;
                    break;
                }
                s_counts[1] = it + 1;
                if (it >= 2 && !tc_wait(&accempty[a], ((it >> 1) & 1) ^ 1, s_abort)) {
                    *s_abort = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t base = smem_u32(stages + (size_t)s * c.stage_bytes);
#pragma unroll 1
                for (int g = 0; g < 9; ++g) {
                    const int b = g / 3, dyi = g % 3;
                    const uint64_t bdesc = umma_desc(wbase + g * 1536, 768, 128);
                    const uint32_t arow = base + (uint32_t)(b * 2) * c.rows_bytes + (uint32_t)(dyi * c.sy) * 16u;
#pragma unroll
                    for (int j = 0; j < TC_SUB; ++j)
                        tc_mma(tmem + (uint32_t)((a * TC_SUB + j) * TC_N),
                               umma_desc(arow + (uint32_t)(j * TC_OUT) * 16u, c.rows_bytes, 128), bdesc, kTcIdesc,
                               g > 0 ? 1u : 0u);
                }
                tc_commit(&empty[s]);
                tc_commit(&accfull[a]);
                s_counts[2] = it + 1;
            }
        }
    } else {
        const int quarter = warp & 3;        // TMEM lanes 32*quarter .. +31 belong to this warp
        const int group = (warp - 2) >> 2;   // windows group, group + TC_EPI_GROUPS, ...
        const int i = quarter * 32 + lane;   // row of the 128-row window
        const uint32_t usx = (uint32_t)c.sx, usy = (uint32_t)c.sy;
        float* xg = xchg + group * (2 * 4 * 2 * 16);
        int it = 0;
        int xp = 0;  // exchange buffer parity
        for (int64_t tile = blockIdx.x; tile < c.ntiles; tile += gridDim.x, ++it) {
            const int a = it & 1;
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
#pragma unroll 1
            for (int j = group; j < TC_SUB; j += TC_EPI_GROUPS) {
                __syncwarp();
                const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((a * TC_SUB + j) * TC_N);
                float* xb = xg + xp * (4 * 2 * 16);
                const int64_t p = c.p_begin + (tile * TC_SUB + j) * TC_OUT - 1 + i;
                // voxel of row p (rows < 2^31: checked on the host)
                const uint32_t up = (uint32_t)p;
                const uint32_t xq = up / usx;
                const uint32_t rem = up - xq * usx;
                const uint32_t yq = rem / usy;
                const uint32_t zq = rem - yq * usy;
                const bool valid = i >= 1 && i <= TC_OUT && xq >= 1 && xq <= (uint32_t)c.nx && yq >= 1 &&
                                   yq <= (uint32_t)c.ny && zq >= 1 && zq <= (uint32_t)c.nz;
                if (LAST) {
                    const float zm = tc_ld1(taddr), z0 = tc_ld1(taddr + 16), zp = tc_ld1(taddr + 32);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (lane == 31) xb[(quarter * 2 + 0) * 16] = zm;
                    if (lane == 0) xb[(quarter * 2 + 1) * 16] = zp;
                    epi_group_barrier(group);
                    float lo = __shfl_up_sync(0xffffffffu, zm, 1);
                    float hi = __shfl_down_sync(0xffffffffu, zp, 1);
                    if (lane == 0 && quarter > 0) lo = xb[((quarter - 1) * 2 + 0) * 16];
                    if (lane == 31 && quarter < 3) hi = xb[((quarter + 1) * 2 + 1) * 16];
                    xp ^= 1;
                    if (valid) {
                        const int64_t vox = ((int64_t)(xq - 1) * c.ny + (yq - 1)) * (int64_t)c.nz + (zq - 1);
                        float o = lo + z0 + hi;
                        if (c.mask && c.mask[vox] != 0.f) o = 0.f;
                        if (c.dinv) o += c.omega * c.dinv[vox] * c.r[vox];
                        c.w[vox] = o;
                    }
                } else {
                    float zm[16], z0[16], zp[16];
                    tc_ld16(taddr, zm);
                    tc_ld16(taddr + 16, z0);
                    tc_ld16(taddr + 32, zp);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    if (lane == 31) {
#pragma unroll
                        for (int k = 0; k < 16; ++k) xb[(quarter * 2 + 0) * 16 + k] = zm[k];
                    }
                    if (lane == 0) {
#pragma unroll
                        for (int k = 0; k < 16; ++k) xb[(quarter * 2 + 1) * 16 + k] = zp[k];
                    }
                    epi_group_barrier(group);
                    float o[16];
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        float lo = __shfl_up_sync(0xffffffffu, zm[k], 1);
                        float hi = __shfl_down_sync(0xffffffffu, zp[k], 1);
                        if (lane == 0 && quarter > 0) lo = xb[((quarter - 1) * 2 + 0) * 16 + k];
                        if (lane == 31 && quarter < 3) hi = xb[((quarter + 1) * 2 + 1) * 16 + k];
                        o[k] = fmaxf(lo + z0[k] + hi, 0.f);
                    }
                    xp ^= 1;
                    if (valid) {
                        uint32_t pk[8];
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const __nv_bfloat162 h2 = __floats2bfloat162_rn(o[2 * k], o[2 * k + 1]);
                            pk[k] = *reinterpret_cast<const uint32_t*>(&h2);
                        }
                        *reinterpret_cast<uint4*>(c.out + p * 16) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                        *reinterpret_cast<uint4*>(c.out + (c.plane_rows + p) * 16) =
                            make_uint4(pk[4], pk[5], pk[6], pk[7]);
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive1(&accempty[a]);
        }
    }

    // teardown: every copy landed and every MMA finished before shared memory and TMEM go away
    __syncthreads();
    if (threadIdx.x == 32) {
        const int issued = s_counts[0], taken = s_counts[1], committed = s_counts[2];
        bool ok = true;
        for (int j = taken; j < issued; ++j)  // copies nobody consumed (abort path only)
            ok = mbar_wait_bounded(&full[j % S], (j / S) & 1) && ok;
        for (int j = committed > S ? committed - S : 0; j < committed; ++j)
            ok = mbar_wait_bounded(&empty[j % S], (j / S) & 1) && ok;
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
    k_features_planar<<<grid, 256, 0, stream>>>(nx, ny, nz, planar_rows(nx, ny, nz), r, dinv, chat, mask,
                                                 static_cast<unsigned char*>(out));
    GB_CHECK_CUDA(cudaGetLastError());
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
    c.p_begin = c.sx + c.sy + 1;
    const int64_t p_last = (int64_t)nx * c.sx + (int64_t)ny * c.sy + nz;
    c.ntiles = ceil_div<int64_t>(p_last - c.p_begin + 1, TC_SUB * TC_OUT);
    c.plane_rows = planar_rows(nx, ny, nz);
    GB_REQUIRE(c.plane_rows < (int64_t(1) << 31), "conv3_fwd_tc: grid too large (padded rows must fit in 31 bits)");
    const int64_t rows = 2 * (int64_t)c.sy + TC_OUT * (TC_SUB - 1) + TC_M;
    c.rows_bytes = (uint32_t)(rows * 16);
    c.stage_bytes = 6 * c.rows_bytes;
    const size_t fixed = TC_W_BYTES + TC_XCHG_BYTES + 256;
    c.stages = TC_MAX_STAGES;
    while (c.stages > 2 && (size_t)c.stages * c.stage_bytes + fixed > 220 * 1024) --c.stages;
    const size_t smem = (size_t)c.stages * c.stage_bytes + fixed;
    if (smem > 220 * 1024) {
        gb::set_error("conv3_fwd_tc: grid too long in z (nz = %d) for the staged tile", nz);
        return GB_ERR_UNSUPPORTED;
    }
    c.in = static_cast<const unsigned char*>(in);
    c.Wt = static_cast<const __nv_bfloat16*>(Wt);
    c.out = static_cast<unsigned char*>(out);
    c.w = w;
    c.r = r;
    c.dinv = dinv;
    c.mask = mask;
    c.omega = omega;
    c.status = status;
    int dev = 0, sms = kSmCount, per_sm = 1;
    GB_CHECK_CUDA(cudaGetDevice(&dev));
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (last) {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_conv3_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3_tc<true>, TC_THREADS, smem));
    } else {
        GB_CHECK_CUDA(cudaFuncSetAttribute(k_conv3_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_conv3_tc<false>, TC_THREADS, smem));
    }
    per_sm = 1;  // one CTA per SM: it holds all 512 TMEM columns
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(c.ntiles, (int64_t)sms * per_sm));
    if (last)
        k_conv3_tc<true><<<grid, TC_THREADS, smem, stream>>>(c);
    else
        k_conv3_tc<false><<<grid, TC_THREADS, smem, stream>>>(c);
    GB_CHECK_CUDA(cudaGetLastError());
    return GB_OK;
}
