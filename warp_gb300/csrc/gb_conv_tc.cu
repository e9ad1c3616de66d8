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
// The dx and dz taps are folded into the GEMM's N dimension.  For a window of 128 consecutive rows
// q of input x-plane x_in and one dy,
//     Z[q][dx][dz][co] = sum_ci in[x_in][q + dy sy][ci] W[dx,dy,dz][ci][co]
// is one MMA (M = 128 rows, N = 144 = 3 dx x 3 dz x 16 co, K = 16 channels) whose A operand is 128
// consecutive staged rows -- a K-major, non-swizzled UMMA operand (8-row core matrices 128 B apart,
// the two 8-channel halves one plane apart).  Input plane x_in feeds output planes x_in + 1, x_in,
// x_in - 1 (dx = -1, 0, +1), so the B operand orders its rows [dx = +1 | 0 | -1] and the MMA's 144
// accumulator columns are three 48-column chunks of a per-window ring of output planes in TMEM:
// the chunks of consecutive output planes are adjacent, and one MMA adds this input plane's
// contribution to all three.  Over its three input planes an output plane's chunk receives its 27
// taps: 3 dy MMAs per (window, input plane) instead of 9 when only dz was folded (the MMA issue
// rate, not its N, bounds these K = 16 MMAs).  A chunk whose three planes wrap around the ring end
// is split into two MMAs; at the ends of a CTA's run of x-planes only the chunks of planes in the
// run are written (N = 48 or 96).  The epilogue then forms
//     out[p] = Z[p-1][dz=-1] + Z[p][0] + Z[p+1][+1]
// for the 126 rows whose neighbours lie in the same 128-row window (lane shuffles, plus one value
// exchanged between neighbouring epilogue warps), and zeroes the chunk for its next plane.
//
// A work item is one output x-plane of a column of TC_SUB = 2 windows (252 output rows); a CTA walks
// x through a contiguous range of items, so each input x-plane block (both planes, rows
// [q0 - sy, q0 + sy + 126 + 128)) is copied once with 1-D bulk copies into a ring of slots.  Warp
// roles: a copy warp, two MMA-issuing warps per window (alternate input planes; 3 dy MMAs per input
// plane on the window's chunk ring), and two groups of four epilogue warps per window (one warp per TMEM lane quarter;
// the groups take alternate output planes) that read a finished chunk with tcgen05.ld, sum the dz
// taps, apply ReLU and store bf16 rows of interior voxels -- or, for the last layer, write
// w[v] = omega dinv[v] r[v] + (mask[v] ? 0 : out[v][0]) in fp32 (the Jacobi step fused; for vec3
// fields the node's three dofs from output channels 0..2).  A chunk is zeroed with tcgen05.st and
// handed back to the issuers as soon as its values are in registers, before the exchange and stores.
// The two issuers of a window take turns in block order (a shared-memory sequence word), so a plane's
// three contributions are summed in the same order in every launch: results are bitwise reproducible.
//
// Whole-network launch (gb_convnet_fwd_tc, NET = true): one cooperative launch runs (optionally) the features and
// all four layers; each CTA walks its items layer after layer, and layer l reads activations that
// other CTAs wrote in layer l - 1.  Per-item counters in global memory carry the dependency: a counter
// warp raises an item's counter by 8 once the item's 8 epilogue warps have stored a hidden layer
// (several items per fence, so the epilogue never waits on its stores), and the copy warp's 32 lanes
// read the counters of the next planes' neighbouring columns in one round trip before staging them.
// Every wait is bounded (globaltimer); a timeout sets GB_DEV_WAIT_TIMEOUT, the CTA drains its own
// copies and MMAs (bounded) and frees its TMEM before returning.
#include "gb_bulk.cuh"
#include "gb_common.cuh"
#include "gb_net_features.cuh"
#include "gb_spmv.cuh"  // sm_count()

namespace gb {

constexpr int TC_M = 128;                  // rows of one window (UMMA M)
constexpr int TC_OUT = TC_M - 2;           // output rows per window
constexpr int TC_SUB = 2;                  // windows per work item (252 output rows of one x-plane)
constexpr int TC_CHUNK = 48;               // TMEM columns of one (window, output plane): 3 dz x 16 co
constexpr int TC_RING = 5;                 // output planes in flight per window (chunk ring)
constexpr int TC_N = 3 * TC_CHUNK;         // 144 = 3 dx x 3 dz x 16 co (UMMA N of a full MMA)
constexpr int TC_ISSUE_PAR = 2;            // MMA-issuing threads per window: alternate input planes
constexpr int TC_ISSUERS = TC_SUB * TC_ISSUE_PAR;
constexpr int TC_EPI_PAR = 2;              // epilogue groups per window: items drained alternately
constexpr int TC_EPI_GROUPS = TC_SUB * TC_EPI_PAR;  // groups of 4 warps (one per TMEM lane quarter)
constexpr int TC_EPI_WARP0 = 1 + TC_ISSUERS;  // warp 0 copies, warps 1..TC_ISSUERS issue MMAs, then the epilogue
constexpr int TC_THREADS = 32 * TC_EPI_WARP0 + TC_EPI_GROUPS * 128;
constexpr int TC_NET_THREADS = TC_THREADS + 32;  // whole-network launch: one more warp raises the counters
constexpr int TC_FLAG_RING = 8;                   // item steps between the epilogue and the counter warp
constexpr uint32_t TC_TMEM_COLS = 512;     // TC_SUB x TC_RING x TC_CHUNK = 480, rounded up
constexpr uint32_t TC_WIN_COLS = TC_RING * TC_CHUNK;  // 240 columns per window
constexpr int TC_WB_KHALF = TC_N * 16;     // B operand of one dy: [k-half][n 144][8 ci] bf16
constexpr int TC_WB_DY = 2 * TC_WB_KHALF;  // 4608 bytes
constexpr int TC_W_BYTES = 3 * TC_WB_DY;   // 13824 bytes for the 3 dy
constexpr int TC_XCHG_BYTES = TC_EPI_GROUPS * 2 * 4 * 2 * 16 * 4;  // [group][parity][quarter][lo/hi][16]
constexpr int TC_MAX_SLOTS = 8;            // x-plane blocks in the shared-memory ring
constexpr int TC_MAX_LAYERS = 4;           // layers of the learned smoother's network
constexpr int TC_POLL = 32;                // completion counters read per poll of the copy warp (one per lane)
constexpr int TC_MIN_SLOTS = 3;            // one being read, one landing, one in flight
constexpr size_t TC_SMEM_LIMIT = 200 * 1024;
constexpr int TC_BAR_PROLOGUE = 1 + TC_EPI_GROUPS;  // named barriers: 0 CTA, 1..groups epilogue groups,
                                                    // then the prologue
constexpr int TC_BAR_EPI_ALL = TC_BAR_PROLOGUE + 1;  // all epilogue warps (the features phase)
static_assert(TC_SUB * TC_WIN_COLS <= TC_TMEM_COLS, "chunk rings exceed the TMEM allocation");

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
    int nlayers;                      // layers run by one launch (1, or TC_MAX_LAYERS for the whole network)
    const unsigned char* in[TC_MAX_LAYERS];   // layer l reads in[l] (planar padded bf16)
    const __nv_bfloat16* Wt[TC_MAX_LAYERS];   // [27][16 co][16 ci] bf16 per layer
    unsigned char* out[TC_MAX_LAYERS];        // hidden layer l writes out[l] (planar padded bf16)
    float* w;                 // last layer: fp32 [n]
    const float* r;
    const float* dinv;
    const float* mask;
    float omega;
    int* status;
    // whole-network launch (flags != null): per-item completion counters and the launch epoch
    unsigned int* flags;      // [nitems]: +8 per completed stage of the item (features, each hidden layer)
    unsigned int* epoch;      // [2]: launches completed, CTAs done in the current launch
    const float* chat;        // features phase (in[0] written by this launch) when not null
    int ncomp;
};

__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    // start address, leading (K) byte offset, stride (M/N) byte offset, all >> 4; version 1 (bit 46);
    // base offset 0, no swizzle.
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D fp32, A and B bf16, both K-major, N >> 3, M >> 4.
__host__ __device__ constexpr uint32_t tc_idesc(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);
}

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

// zero 16 consecutive accumulator columns of this warp's lane quarter
__device__ __forceinline__ void tc_st16_zero(uint32_t taddr)
{
    const uint32_t z = 0u;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1, %1};" ::"r"(taddr),
        "r"(z)
        : "memory");
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

__device__ __forceinline__ unsigned int ld_acquire_u32_gpu(const unsigned int* p)
{
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_cta(volatile int* p, int v)
{
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_u32((const void*)p)), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_acquire_cta(volatile int* p)
{
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32((const void*)p)) : "memory");
    return v;
}

// bounded wait until *seq == want (another issuer's release), or an abort; the clock and the abort flag
// are read once per 32 polls, so that the hand-off is seen within a poll or two
__device__ __forceinline__ bool tc_wait_seq(volatile int* seq, int want, volatile int* abort_flag)
{
    if (ld_acquire_cta(seq) == want) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        for (int k = 0; k < 32; ++k)
            if (ld_acquire_cta(seq) == want) return true;
        if (*abort_flag) return false;
        if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

// bounded wait until *seq > bound (another role's release), or an abort
__device__ __forceinline__ bool tc_wait_seq_gt(volatile int* seq, int bound, volatile int* abort_flag)
{
    if (ld_acquire_cta(seq) > bound) return true;
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        if (ld_acquire_cta(seq) > bound) return true;
        if (*abort_flag) return false;
        if (globaltimer_ns() - t0 > kWaitLimitNs) return false;
    }
}

// named barriers (non-aligned form: lanes may arrive after divergent code): id 1 + group for the four
// warps of one epilogue group
__device__ __forceinline__ void epi_group_barrier(int group)
{
    asm volatile("barrier.sync %0, 128;" ::"r"(1 + group) : "memory");
}

template <int NOUT, bool NET>
__global__ void __launch_bounds__(NET ? TC_NET_THREADS : TC_THREADS, 1) k_conv3_tc(const TcConv c)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    pdl_enter();
    unsigned char* ring = smem;
    unsigned char* wsm = smem + (size_t)c.slots * c.block_bytes;  // B operands of every layer
    const int NL = NET ? c.nlayers : 1;
    float* xchg = reinterpret_cast<float*>(wsm + NL * TC_W_BYTES);  // [group][parity][quarter][lo/hi][16]
    uint64_t* full = reinterpret_cast<uint64_t*>(wsm + NL * TC_W_BYTES + TC_XCHG_BYTES);
    uint64_t* empty = full + TC_MAX_SLOTS;
    uint64_t* accfull = empty + TC_MAX_SLOTS;  // [TC_RING]: an output plane's chunks are complete
    uint64_t* accempty = accfull + TC_RING;    // [TC_RING]: a chunk was drained and zeroed
    uint64_t* done = accempty + TC_RING;       // every issuer's last commit: all MMAs of the CTA completed
    uint64_t* stored = done + 1;  // [TC_FLAG_RING] (whole network) the 8 epilogue warps of a step stored its rows
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(stored + TC_FLAG_RING);
    volatile int* s_abort = reinterpret_cast<volatile int*>(s_tmem + 1);
    volatile int* s_issued = s_abort + 1;      // x-plane blocks whose copies were issued
    const int NS = c.slots;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int* s_gabort = s_issued + 1;  // [TC_EPI_GROUPS] per epilogue group, read after its barrier
    volatile int* s_seq = s_gabort + TC_EPI_GROUPS;  // [TC_SUB] blocks whose MMAs a window has issued
    volatile int* s_flagged = s_seq + TC_SUB;        // hidden-layer steps whose counters were raised
    // contiguous range of work items (output planes); consecutive items of one column are consecutive
    // x-planes, so every input plane of a run is staged once
    const int64_t k_begin = (int64_t)blockIdx.x * c.nitems / gridDim.x;
    const int64_t k_end = (int64_t)(blockIdx.x + 1) * c.nitems / gridDim.x;
    const int nit = (int)(k_end - k_begin);  // items per layer; step G = l * nit + (k - k_begin)
    // whole-network launch: an item's counter grows by 8 per completed stage; this launch's stages
    // start at epoch * 8 * stages (the previous launches' total)
    constexpr bool fused = NET;
    const int feat = (NET && c.chat) ? 1 : 0;
    const unsigned int stages = (unsigned int)(feat + NL - 1);
    const unsigned int flag_base = fused ? __ldcg(c.epoch) * 8u * stages : 0u;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], TC_SUB);  // an input plane is read by one issuer per window
        }
        for (int a = 0; a < TC_RING; ++a) {
            mbar_init(&accfull[a], TC_ISSUERS);  // per window: the last contribution of each issuer
            mbar_init(&accempty[a], 4 * TC_SUB);  // the 4 warps of each window's group draining the plane
        }
        mbar_init(done, TC_ISSUERS);
        for (int a = 0; a < TC_FLAG_RING; ++a) mbar_init(&stored[a], 4 * TC_SUB);
        *s_flagged = 0;
        *s_abort = 0;
        *s_issued = 0;
        for (int gq = 0; gq < TC_EPI_GROUPS; ++gq) s_gabort[gq] = 0;
        for (int j = 0; j < TC_SUB; ++j) s_seq[j] = 0;
        fence_mbar_init();
    }
    uint32_t tmem = 0;
    if (warp == 0) {
        // the copy warp needs only the barriers: it starts filling the ring while the other warps
        // stage the weights and allocate TMEM
        __syncwarp();
        __threadfence_block();  // the barrier words and flags written by thread 0 before the arrival
        asm volatile("bar.arrive %0, %1;" ::"r"(TC_BAR_PROLOGUE), "r"(blockDim.x) : "memory");
    } else {
        // weights -> B operands: dy index g, k-half kc, row n = 48 (1 - dx) + 16 (dz + 1) + co at
        // g * TC_WB_DY + kc * TC_WB_KHALF + n * 16 (rows ordered by the output plane they feed)
        for (int i = threadIdx.x - 32; i < NL * 27 * 16 * 2; i += (int)blockDim.x - 32) {
            const int l = i / (27 * 16 * 2), il = i - l * (27 * 16 * 2);
            const int t = il >> 5, co = (il >> 1) & 15, kc = il & 1;
            const int dx = t / 9 - 1, g = (t / 3) % 3, dz = t % 3 - 1;
            const uint4 v = reinterpret_cast<const uint4*>(c.Wt[l])[(t * 16 + co) * 2 + kc];
            const int n = TC_CHUNK * (1 - dx) + 16 * (dz + 1) + co;
            *reinterpret_cast<uint4*>(wsm + l * TC_W_BYTES + g * TC_WB_DY + kc * TC_WB_KHALF + n * 16) = v;
        }
        fence_proxy_async_shared();  // make the generic-proxy stores visible to the tensor cores
        if (warp == 1) {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                         "r"(TC_TMEM_COLS)
                         : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
        tc_fence_before();
        asm volatile("bar.sync %0, %1;" ::"r"(TC_BAR_PROLOGUE), "r"(blockDim.x) : "memory");
        tc_fence_after();
        tmem = *s_tmem;
    }

    if (warp == 0) {
        // ------------------------- copy warp: x-plane blocks into the ring ----------------------------
        // Lane 0 waits for free slots and issues the bulk copies; all lanes walk the same loops.  In a
        // whole-network launch, before staging input plane x of layer l the warp waits until every
        // column whose rows the block spans has finished stage l - 1 + feat at that plane (other CTAs'
        // items): its lanes read up to 32 (plane, column) counters from plane x on at once (one round
        // trip), the planes before the first unfinished one are then ready, and a proxy fence orders the
        // acquired stores before the bulk copies.
        // a single-layer launch needs lane 0 only (no counters to read)
        if (NET || lane == 0) {
            constexpr unsigned kLanes = NET ? 0xffffffffu : 1u;
            int q = 0;  // sequence number of the next block; its slot is q % NS
            bool ok = true;
            const int span = (int)(((int64_t)c.sy + 2 + TC_SUB * TC_OUT - 1) / (TC_SUB * TC_OUT));  // columns
            for (int l = 0; l < NL && ok; ++l) {
                const unsigned int need = flag_base + 8u * (unsigned int)(l + feat);
                const bool wait_flags = fused && (l + feat) > 0;
                for (int64_t k = k_begin; k < k_end && ok;) {
                    const int o = (int)(k / c.nx);
                    const int x0 = (int)(k % c.nx) + 1;
                    const int64_t run_end = min(k_end, (int64_t)(o + 1) * c.nx);
                    const int x1 = (int)((run_end - 1) % c.nx) + 1;
                    int ready = 0;  // planes up to this one are finished (this layer's input, this run)
                    for (int xb = x0 - 1; xb <= x1 + 1; ++xb, ++q) {
                        const int s = q % NS;
                        int wok = 1;
                        if (lane == 0 && ((q >= NS && !tc_wait(&empty[s], ((q / NS) - 1) & 1, s_abort)) || *s_abort))
                            wok = 0;
                        if (!__shfl_sync(kLanes, wok, 0)) {
                            if (lane == 0) *s_abort = 1;
                            ok = false;
                            break;
                        }
                        if (wait_flags && xb >= 1 && xb <= c.nx && xb > ready) {
                            const int cmin = max(0, o - span), cmax = min(c.ncols - 1, o + span);
                            const int ncl = cmax - cmin + 1;  // <= TC_POLL (checked on the host)
                            const int npl = max(1, min(min(c.nx, x1 + 1) - xb + 1, TC_POLL / ncl));
                            const int pe = lane / ncl, ce = lane - pe * ncl;  // this lane's (plane, column)
                            const bool mine = pe < npl;
                            const unsigned int* fp = c.flags + (int64_t)(cmin + ce) * c.nx + (xb - 1 + pe);
                            const uint64_t t0 = globaltimer_ns();
                            int first_bad;  // first plane (offset from xb) not finished yet
                            for (;;) {
                                const bool bad = mine && (int)(ld_acquire_u32_gpu(fp) - need) < 0;
                                first_bad = (int)__reduce_min_sync(0xffffffffu, (unsigned)(bad ? pe : npl));
                                if (first_bad > 0) break;
                                int stop = 0;
                                if (lane == 0 && (*s_abort || globaltimer_ns() - t0 > kWaitLimitNs)) stop = 1;
                                if (__shfl_sync(0xffffffffu, stop, 0)) break;
                            }
                            if (first_bad == 0) {
                                if (lane == 0) *s_abort = 1;
                                ok = false;
                                break;
                            }
                            ready = xb + first_bad - 1;
                            __syncwarp();
                            asm volatile("fence.proxy.async.global;" ::: "memory");
                        }
                        if (lane == 0) {
                            const int64_t row = (int64_t)xb * c.sx + (int64_t)o * (TC_SUB * TC_OUT);
                            unsigned char* dst = ring + (size_t)s * c.block_bytes;
                            mbar_arrive_expect_tx(&full[s], c.block_bytes);
    #pragma unroll
                            for (int h = 0; h < 2; ++h)
                                bulk_g2s(dst + h * c.rows_bytes, c.in[l] + ((int64_t)h * c.plane_rows + row) * 16,
                                         c.rows_bytes, &full[s]);
                            *s_issued = q + 1;
                        }
                    }
                    k = run_end;
                }
            }
        }
    } else if (warp <= TC_ISSUERS) {
        // ---------- MMA warps: warp 1 + u issues, for window u % TC_SUB, the 3 dy MMAs of the input
        // planes of parity u / TC_SUB (counted from the run's first input plane) ---------------------
        // Two threads accumulate into the same window's chunks (the tensor pipe executes one SM's
        // MMAs in order).  Output plane P receives input planes P - 1, P + 1 from one issuer and P
        // from the other, so each issuer commits accfull[P] after its last contribution to P: at
        // input P (its own parity) and at input P + 1 (the other parity) -- TC_ISSUERS arrivals
        // per plane.  An issuer waits for a chunk to be drained before it first writes it; the chunk
        // of plane xi was first written by the other issuer (input xi - 1), so the issuer of input xi
        // waits on planes xi and xi + 1 (the wait on an already completed phase returns at once).
        if (lane == 0) {
            const int u = warp - 1;
            const int j = u % TC_SUB, par = u / TC_SUB;
            const uint32_t wbase = smem_u32(wsm);
            const uint32_t rbase = smem_u32(ring);
            const uint32_t dwin = tmem + (uint32_t)j * TC_WIN_COLS;
            int it0 = 0;  // step number (CTA order) of the current run's first output plane
            int q0 = 0;   // block sequence number of the run's first input plane (x0 - 1)
            bool ok = true;
            for (int l = 0; l < NL && ok; ++l)
            for (int64_t k = k_begin; k < k_end && ok;) {
                const int o = (int)(k / c.nx);
                const int x0 = (int)(k % c.nx) + 1;
                const int64_t run_end = min(k_end, (int64_t)(o + 1) * c.nx);
                const int x1 = (int)((run_end - 1) % c.nx) + 1;
                for (int xi = x0 - 1 + par; xi <= x1 + 1; xi += TC_ISSUE_PAR) {
                    const int q = q0 + (xi - x0 + 1);
                    // output planes this input feeds inside the run; the chunks of planes lo..hi must
                    // be free before this thread's first write to each
                    const int lo = max(x0, xi - 1), hi = min(x1, xi + 1);
                    ok = tc_wait(&full[q % NS], (q / NS) & 1, s_abort);
                    for (int pl = max(lo, xi); ok && pl <= hi; ++pl) {
                        const int sh = it0 + (pl - x0);
                        ok = tc_wait(&accempty[sh % TC_RING], (sh / TC_RING) & 1, s_abort);
                    }
                    // the window's MMAs go out in block order, alternating between its two issuers, so a
                    // plane's three contributions are summed in the same order in every launch
                    if (TC_ISSUE_PAR > 1 && ok) ok = tc_wait_seq(s_seq + j, q, s_abort);
                    if (!ok) {
                        *s_abort = 1;
                        break;
                    }
                    tc_fence_after();
                    const int np = hi - lo + 1;                 // planes fed (1..3)
                    const int clo = (it0 + (lo - x0)) % TC_RING;  // chunk of plane lo
                    const int n1 = min(np, TC_RING - clo);      // planes before the ring wraps
                    const uint32_t boff = (uint32_t)((lo - (xi - 1)) * TC_CHUNK * 16);  // B rows of plane lo
                    const uint32_t arow0 = rbase + (uint32_t)(q % NS) * c.block_bytes + (uint32_t)(j * TC_OUT) * 16u;
#pragma unroll
                    for (int g = 0; g < 3; ++g) {
                        const uint64_t adesc = umma_desc(arow0 + (uint32_t)(g * c.sy) * 16u, c.rows_bytes, 128);
                        const uint32_t b0 = wbase + (uint32_t)(l * TC_W_BYTES + g * TC_WB_DY) + boff;
                        tc_mma(dwin + (uint32_t)(clo * TC_CHUNK), adesc, umma_desc(b0, TC_WB_KHALF, 128),
                               tc_idesc(n1 * TC_CHUNK), 1u);
                        if (n1 < np)
                            tc_mma(dwin, adesc, umma_desc(b0 + (uint32_t)(n1 * TC_CHUNK * 16), TC_WB_KHALF, 128),
                                   tc_idesc((np - n1) * TC_CHUNK), 1u);
                    }
                    tc_commit(&empty[q % NS]);  // the block is not read again by this thread
                    // this thread's last contributions: plane xi - 1 (other parity) and plane xi (own)
                    if (xi - 1 >= x0 && xi - 1 <= x1) tc_commit(&accfull[(it0 + (xi - 1 - x0)) % TC_RING]);
                    if (TC_ISSUE_PAR > 1 && xi >= x0 && xi <= x1) tc_commit(&accfull[(it0 + (xi - x0)) % TC_RING]);
                    if (TC_ISSUE_PAR > 1) {
                        tc_fence_before();
                        st_release_cta(s_seq + j, q + 1);
                    }
                }
                it0 += (int)(run_end - k);
                q0 += (int)(run_end - k) + 2;
                k = run_end;
            }
            tc_commit(done);  // arrives once every MMA this thread issued has completed
        }
    } else if (warp < TC_EPI_WARP0 + TC_EPI_GROUPS * 4) {
        // --------------------------------- epilogue warps --------------------------------------------
        // group = par * TC_SUB + window: the groups of parity `par` drain the items it with
        // it % TC_EPI_PAR == par, so the TMEM loads, exchange and stores of consecutive items overlap
        const int quarter = warp & 3;                  // TMEM lanes 32*quarter .. +31 belong to this warp
        const int group = (warp - TC_EPI_WARP0) >> 2;
        const int win = group % TC_SUB, par = group / TC_SUB;
        const int i = quarter * 32 + lane;             // row of the 128-row window
        const uint32_t usx = (uint32_t)c.sx, usy = (uint32_t)c.sy;
        const uint32_t tq = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)win * TC_WIN_COLS;
        float* xg = xchg + group * (2 * 4 * 2 * 16);
        if (feat) {
            // features phase: the 16 input channels of every output row of this CTA's items, written
            // to in[0]; then each item's counter gets its first 8
            const int et = threadIdx.x - 32 * TC_EPI_WARP0;
            constexpr int NT = TC_EPI_GROUPS * 128, RU = 4;  // threads, rows per thread and pass
            const int64_t nrows = (int64_t)nit * (TC_SUB * TC_OUT);
            unsigned char* fo = const_cast<unsigned char*>(c.in[0]);
            for (int64_t t0 = et; t0 < nrows; t0 += RU * NT) {
                // RU rows per pass: all their loads are issued before any is used
                uint32_t up[RU];
                int64_t vox[RU];
                bool ok[RU];
#pragma unroll
                for (int u = 0; u < RU; ++u) {
                    const int64_t t = t0 + (int64_t)u * NT;
                    const int64_t k = k_begin + t / (TC_SUB * TC_OUT);
                    const uint32_t xk = (uint32_t)(k % c.nx) + 1u;
                    up[u] = xk * usx + usy + (uint32_t)(k / c.nx) * (uint32_t)(TC_SUB * TC_OUT) + 1u +
                            (uint32_t)(t % (TC_SUB * TC_OUT));
                    const uint32_t xq = fastdiv(up[u], c.div_sx);
                    const uint32_t rem = up[u] - xq * usx;
                    const uint32_t yq = fastdiv(rem, c.div_sy);
                    const uint32_t zq = rem - yq * usy;
                    ok[u] = t < nrows && xq == xk && yq - 1u < (uint32_t)c.ny && zq - 1u < (uint32_t)c.nz;
                    vox[u] = ok[u] ? ((int64_t)(xq - 1) * c.ny + (yq - 1)) * (int64_t)c.nz + (zq - 1) : 0;
                }
                NetNodeIn nin[RU];
#pragma unroll
                for (int u = 0; u < RU; ++u) net_node_load(c.ncomp, vox[u], c.r, c.dinv, c.chat, c.mask, nin[u]);
#pragma unroll
                for (int u = 0; u < RU; ++u) {
                    if (!ok[u]) continue;
                    float f[16];
                    net_node_compute(c.ncomp, nin[u], f);
                    uint32_t pk[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(f[2 * q], f[2 * q + 1]);
                        pk[q] = *reinterpret_cast<const uint32_t*>(&h2);
                    }
                    *reinterpret_cast<uint4*>(fo + (int64_t)up[u] * 16) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    *reinterpret_cast<uint4*>(fo + (c.plane_rows + (int64_t)up[u]) * 16) =
                        make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
            }
            // every writer orders its stores for the other CTAs' bulk copies (async proxy) before the
            // counters are raised
            asm volatile("fence.proxy.async.global;" ::: "memory");
            __threadfence();
            asm volatile("bar.sync %0, %1;" ::"r"(TC_BAR_EPI_ALL), "r"(TC_EPI_GROUPS * 128) : "memory");
            if (et == 0) {
                __threadfence();
                for (int64_t k = k_begin; k < k_end; ++k) atomicAdd(c.flags + k, 8u);
            }
        }
        // the accumulator chunks start at zero (every MMA accumulates); the parity-0 groups clear them
        // and give the first "drained" arrival of every chunk
        if (par == 0) {
            for (int a = 0; a < TC_RING; ++a) {
#pragma unroll
                for (int h = 0; h < 3; ++h) tc_st16_zero(tq + (uint32_t)(a * TC_CHUNK + 16 * h));
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            tc_fence_before();
            __syncwarp();
            if (lane == 0)
                for (int a = 0; a < TC_RING; ++a) mbar_arrive1(&accempty[a]);
        }
        int xp = 0;  // exchange buffer parity
        for (int it = par; it < NL * nit; it += TC_EPI_PAR) {
            const int l = NET ? it / nit : 0;
            const int64_t k = k_begin + (it - l * nit);
            const bool last_layer = NOUT > 0 && (!NET || l == NL - 1);
            const int a = it % TC_RING;
            const uint32_t xk = (uint32_t)(k % c.nx) + 1u;
            // row of lane 0 of window 0: one row before the item's first output row
            const uint32_t q0 = xk * usx + usy + (uint32_t)(k / c.nx) * (uint32_t)(TC_SUB * TC_OUT);
            int ok = 1;
            if (lane == 0) ok = tc_wait(&accfull[a], (it / TC_RING) & 1, s_abort) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok && lane == 0) s_gabort[group] = 1;
            // the group's four warps decide together: the flag only changes before this barrier
            epi_group_barrier(group);
            if (s_gabort[group]) {
                if (lane == 0) *s_abort = 1;
                break;
            }
            tc_fence_after();
            __syncwarp();
            float* xb = xg + xp * (4 * 2 * 16);
            const uint32_t taddr = tq + (uint32_t)(a * TC_CHUNK);
            // voxel of row p (rows < 2^31: checked on the host); rows of the next x-plane belong to the
            // next item of the column
            const uint32_t up = q0 + (uint32_t)(win * TC_OUT + i);
            const uint32_t xq = fastdiv(up, c.div_sx);
            const uint32_t rem = up - xq * usx;
            const uint32_t yq = fastdiv(rem, c.div_sy);
            const uint32_t zq = rem - yq * usy;
            const bool valid = i >= 1 && i <= TC_OUT && xq == xk && yq - 1u < (uint32_t)c.ny && zq - 1u < (uint32_t)c.nz;
            const int64_t vox = ((int64_t)(xq - 1) * c.ny + (yq - 1)) * (int64_t)c.nz + (zq - 1);
            if (last_layer) {
                // last layer: output channels 0..NOUT-1 of the node's NOUT interleaved dofs
                constexpr int NO = NOUT > 0 ? NOUT : 1;
                float zm[NO], z0[NO], zp[NO];
#pragma unroll
                for (int q = 0; q < NO; ++q) {
                    zm[q] = tc_ld1(taddr + q);
                    z0[q] = tc_ld1(taddr + 16 + q);
                    zp[q] = tc_ld1(taddr + 32 + q);
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                // the values are in registers: zero the chunk for the plane TC_RING items later and give
                // it back to the MMA issuers before the exchange and the stores
#pragma unroll
                for (int h = 0; h < 3; ++h) tc_st16_zero(taddr + (uint32_t)(16 * h));
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive1(&accempty[a]);
#pragma unroll
                for (int q = 0; q < NO; ++q) {
                    if (lane == 31) xb[(quarter * 2 + 0) * 16 + q] = zm[q];
                    if (lane == 0) xb[(quarter * 2 + 1) * 16 + q] = zp[q];
                }
                epi_group_barrier(group);
#pragma unroll
                for (int q = 0; q < NO; ++q) {
                    float lo = __shfl_up_sync(0xffffffffu, zm[q], 1);
                    float hi = __shfl_down_sync(0xffffffffu, zp[q], 1);
                    if (lane == 0 && quarter > 0) lo = xb[((quarter - 1) * 2 + 0) * 16 + q];
                    if (lane == 31 && quarter < 3) hi = xb[((quarter + 1) * 2 + 1) * 16 + q];
                    if (valid) {
                        const int64_t d = vox * NO + q;
                        float o = lo + z0[q] + hi;
                        if (c.mask && c.mask[vox] != 0.f) o = 0.f;
                        if (c.dinv) o += c.omega * c.dinv[d] * c.r[d];
                        c.w[d] = o;
                    }
                }
            } else {
                float zm[16], z0[16], zp[16];
                tc_ld16(taddr, zm);
                tc_ld16(taddr + 16, z0);
                tc_ld16(taddr + 32, zp);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                // the values are in registers: zero the chunk for the plane TC_RING items later and give
                // it back to the MMA issuers before the exchange and the stores
#pragma unroll
                for (int h = 0; h < 3; ++h) tc_st16_zero(taddr + (uint32_t)(16 * h));
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive1(&accempty[a]);
                float4* lo_dst = reinterpret_cast<float4*>(xb + (quarter * 2 + 0) * 16);
                float4* hi_dst = reinterpret_cast<float4*>(xb + (quarter * 2 + 1) * 16);
                if (lane == 31) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) lo_dst[u] = make_float4(zm[4 * u], zm[4 * u + 1], zm[4 * u + 2], zm[4 * u + 3]);
                }
                if (lane == 0) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) hi_dst[u] = make_float4(zp[4 * u], zp[4 * u + 1], zp[4 * u + 2], zp[4 * u + 3]);
                }
                epi_group_barrier(group);
                float lo[16], hi[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) {
                    lo[u] = __shfl_up_sync(0xffffffffu, zm[u], 1);
                    hi[u] = __shfl_down_sync(0xffffffffu, zp[u], 1);
                }
                if (lane == 0 && quarter > 0) {
                    const float4* src = reinterpret_cast<const float4*>(xb + ((quarter - 1) * 2 + 0) * 16);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float4 v = src[u];
                        lo[4 * u] = v.x; lo[4 * u + 1] = v.y; lo[4 * u + 2] = v.z; lo[4 * u + 3] = v.w;
                    }
                }
                if (lane == 31 && quarter < 3) {
                    const float4* src = reinterpret_cast<const float4*>(xb + ((quarter + 1) * 2 + 1) * 16);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float4 v = src[u];
                        hi[4 * u] = v.x; hi[4 * u + 1] = v.y; hi[4 * u + 2] = v.z; hi[4 * u + 3] = v.w;
                    }
                }
                if (valid) {
                    uint32_t pk[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const __nv_bfloat162 h2 =
                            __floats2bfloat162_rn(fmaxf(lo[2 * u] + z0[2 * u] + hi[2 * u], 0.f),
                                                  fmaxf(lo[2 * u + 1] + z0[2 * u + 1] + hi[2 * u + 1], 0.f));
                        pk[u] = *reinterpret_cast<const uint32_t*>(&h2);
                    }
                    const int64_t pr = up;
                    unsigned char* ob = c.out[l];
                    *reinterpret_cast<uint4*>(ob + pr * 16) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    *reinterpret_cast<uint4*>(ob + (c.plane_rows + pr) * 16) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
                if (fused) {
                    // this warp's rows of the item are stored: one of the step's 8 arrivals for the counter
                    // warp, once that warp has taken the step TC_FLAG_RING earlier off the same barrier
                    int fok = 1;
                    if (lane == 0) fok = tc_wait_seq_gt(s_flagged, it - TC_FLAG_RING, s_abort) ? 1 : 0;
                    __syncwarp();
                    if (lane == 0) {
                        if (fok)
                            mbar_arrive1(&stored[it % TC_FLAG_RING]);
                        else
                            *s_abort = 1;
                    }
                }
            }
            xp ^= 1;
        }
    } else if (NET) {
        // ------------ counter warp (whole-network launch): raises an item's counter by 8 once the 8
        // epilogue warps of one of its hidden-layer steps have stored their rows, several steps per fence,
        // so the epilogue never waits for its stores to reach the other CTAs ----------------------------
        if (lane == 0) {
            const int total = (NL - 1) * nit;
            int g0 = 0;
            while (g0 < total) {
                if (!tc_wait(&stored[g0 % TC_FLAG_RING], (g0 / TC_FLAG_RING) & 1, s_abort)) {
                    *s_abort = 1;
                    break;
                }
                int g1 = g0 + 1;
                while (g1 < total && g1 - g0 < TC_FLAG_RING &&
                       mbar_try_wait(&stored[g1 % TC_FLAG_RING], (g1 / TC_FLAG_RING) & 1))
                    ++g1;
                // the rows stored before the arrivals this thread acquired become visible at gpu scope
                // before the counters move
                __threadfence();
                asm volatile("fence.proxy.async.global;" ::: "memory");
                for (int g = g0; g < g1; ++g) atomicAdd(c.flags + k_begin + g % nit, 8u);
                st_release_cta(s_flagged, g1);
                g0 = g1;
            }
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
        if (fused) {
            // the last CTA to finish closes the launch: the next one's stages start 8 * stages higher
            __threadfence();
            if (atomicAdd(c.epoch + 1, 1u) == gridDim.x - 1) {
                c.epoch[1] = 0u;
                __threadfence();
                atomicAdd(c.epoch, 1u);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

// features in the planar padded bf16 layout (interior rows only); ncomp = 1 or 3 (see node_features in
// gb_convnet.cu: the same channels)
__global__ void k_features_planar(int ncomp, int nx, int ny, int nz, int64_t plane_rows, const float* __restrict__ r,
                                  const float* __restrict__ dinv, const float* __restrict__ chat,
                                  const float* __restrict__ mask, unsigned char* __restrict__ out)
{
    pdl_enter();
    // 3-D launch: 32 z-consecutive nodes x 8 y-rows per block, one x-plane per grid z index
    const int z = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    const int x = (int)blockIdx.z;
    if (z < nz && y < ny) {
        const int64_t sy = nz + 2, sx = (int64_t)(ny + 2) * sy;
        const int64_t v = ((int64_t)x * ny + y) * nz + z;
        const int64_t p = (x + 1) * sx + (y + 1) * sy + (z + 1);
        float f[16];
        net_node_features(ncomp, v, r, dinv, chat, mask, f);
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

// grid geometry, work items and the shared-memory ring of a launch of nlayers layers; *smem = its
// dynamic shared memory
static int tc_setup(TcConv& c, int nx, int ny, int nz, int nlayers, size_t* smem)
{
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
    const size_t fixed = (size_t)nlayers * TC_W_BYTES + TC_XCHG_BYTES + 512;
    c.slots = (int)std::min<size_t>(TC_MAX_SLOTS, (TC_SMEM_LIMIT - fixed) / c.block_bytes);
    if (c.slots < TC_MIN_SLOTS) {
        gb::set_error("conv3_fwd_tc: grid too long in z (nz = %d) for the staged x-plane blocks", nz);
        return GB_ERR_UNSUPPORTED;
    }
    c.nlayers = nlayers;
    *smem = (size_t)c.slots * c.block_bytes + fixed;
    return GB_OK;
}

static int tc_set_smem_attr()
{
    // one-time per process: the largest dynamic shared memory any variant may use
    static bool attr_set = false;
    if (!attr_set) {
        void (*const kernels[])(const TcConv) = {k_conv3_tc<0, false>, k_conv3_tc<1, false>, k_conv3_tc<3, false>,
                                                 k_conv3_tc<1, true>, k_conv3_tc<3, true>};
        for (auto kern : kernels)
            GB_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM_LIMIT));
        attr_set = true;
    }
    return GB_OK;
}

}  // namespace gb

using namespace gb;

GB_API int64_t gb_conv3_planar_rows(int nx, int ny, int nz) { return planar_rows(nx, ny, nz); }

GB_API int gb_net_features_planar(int ncomp, int nx, int ny, int nz, const float* r, const float* dinv,
                                  const float* chat, const float* mask, void* out, cudaStream_t stream)
{
    const int64_t n = (int64_t)nx * ny * nz;
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "net_features_planar: ncomp must be 1 or 3");
    if (n <= 0) return GB_OK;
    GB_REQUIRE((uintptr_t)out % 16 == 0, "net_features_planar: output must be 16-byte aligned");
    GB_REQUIRE(nx <= 65535, "net_features_planar: grid too long in x");
    const dim3 grid((unsigned)ceil_div(nz, 32), (unsigned)ceil_div(ny, 8), (unsigned)nx);
    GB_CHECK_CUDA(launch_pdl(k_features_planar, grid, dim3(32, 8, 1), 0, stream, ncomp, nx, ny, nz,
                             planar_rows(nx, ny, nz), r, dinv, chat, mask, static_cast<unsigned char*>(out)));
    return GB_OK;
}

// One 16 -> 16 layer (last = 0: ReLU, planar bf16 output) or the last layer (last = 1: output channel 0
// only, w = omega dinv r + (mask ? 0 : out) in fp32; last = 3: channels 0..2 into the 3 interleaved dofs
// of each node, w[3v + c] = omega dinv[3v + c] r[3v + c] + (mask[v] ? 0 : out[v][c])).  in/out: planar padded bf16 buffers of
// 2 * gb_conv3_planar_rows() rows of 16 bytes whose border rows are zero; Wt: [27][16][16] bf16.
GB_API int gb_conv3_fwd_tc(int nx, int ny, int nz, int last, const void* in, const void* Wt, void* out, float* w,
                           const float* r, const float* dinv, const float* mask, float omega, int* status,
                           cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1, "conv3_fwd_tc: empty grid");
    GB_REQUIRE((uintptr_t)in % 16 == 0 && (uintptr_t)Wt % 16 == 0, "conv3_fwd_tc: in/Wt must be 16-byte aligned");
    GB_REQUIRE(last == 0 || last == 1 || last == 3, "conv3_fwd_tc: last must be 0, 1 or 3");
    GB_REQUIRE(last ? (w != nullptr && (dinv == nullptr || r != nullptr)) : (out != nullptr && (uintptr_t)out % 16 == 0),
               "conv3_fwd_tc: missing output");
    GB_REQUIRE(status != nullptr, "conv3_fwd_tc: status word required");
    TcConv c{};
    size_t smem = 0;
    if (int rc = tc_setup(c, nx, ny, nz, 1, &smem)) return rc;
    c.in[0] = static_cast<const unsigned char*>(in);
    c.Wt[0] = static_cast<const __nv_bfloat16*>(Wt);
    c.out[0] = static_cast<unsigned char*>(out);
    c.w = w;
    c.r = r;
    c.dinv = dinv;
    c.mask = mask;
    c.omega = omega;
    c.status = status;
    if (int rc = tc_set_smem_attr()) return rc;
    // one CTA per SM: it holds all 512 TMEM columns
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(c.nitems, (int64_t)sm_count()));
    if (last == 3)
        GB_CHECK_CUDA(launch_pdl(k_conv3_tc<3, false>, grid, TC_THREADS, smem, stream, c));
    else if (last)
        GB_CHECK_CUDA(launch_pdl(k_conv3_tc<1, false>, grid, TC_THREADS, smem, stream, c));
    else
        GB_CHECK_CUDA(launch_pdl(k_conv3_tc<0, false>, grid, TC_THREADS, smem, stream, c));
    return GB_OK;
}

// Work items (per-item completion counters) of the whole-network launch on an nx x ny x nz grid.
GB_API int64_t gb_convnet_tc_items(int nx, int ny, int nz)
{
    if (nx < 1 || ny < 1 || nz < 1) return 0;
    return ceil_div<int64_t>((int64_t)(ny - 1) * (nz + 2) + nz, TC_SUB * TC_OUT) * nx;
}

// The whole learned smoother in one cooperative launch: the features of (r, dinv, chat, mask) into
// act[0] (as gb_net_features_planar; chat = null: act[0] already holds them), hidden layers l = 0 .. nlayers - 2 from act[l] into act[l + 1]
// (ReLU), and the last layer from act[nlayers - 1] into w (as gb_conv3_fwd_tc with last = ncomp).
// A CTA stages an input x-plane of layer l once the items whose rows it spans have finished layer
// l - 1 on that plane: flags[item] counts their completed stages (8 arrivals per stage, one per
// epilogue warp), epoch[0] the completed launches, so the counters are never cleared.
//   act:   nlayers planar buffers of 2 * gb_conv3_planar_rows() rows of 16 bytes, border rows zero
//   Wt:    nlayers [27][16][16] bf16 weight blocks
//   flags: gb_convnet_tc_items() uint32 counters, epoch: 2 uint32, both zero before the first launch;
//          consecutive launches on one stream may share them, concurrent launches may not, and every
//          launch that shares them must use the same nlayers
// Unsupported (GB_ERR_UNSUPPORTED, nothing launched) when the device cannot hold one CTA per work
// item or SM at once.
GB_API int gb_convnet_fwd_tc(int nx, int ny, int nz, int ncomp, int nlayers, void* const* act, const void* const* Wt,
                             float* w, const float* r, const float* dinv, const float* chat, const float* mask,
                             float omega, unsigned int* flags, unsigned int* epoch, int* status, cudaStream_t stream)
{
    GB_REQUIRE(nx >= 1 && ny >= 1 && nz >= 1, "convnet_fwd_tc: empty grid");
    GB_REQUIRE(ncomp == 1 || ncomp == 3, "convnet_fwd_tc: ncomp must be 1 or 3");
    GB_REQUIRE(nlayers >= 2 && nlayers <= TC_MAX_LAYERS, "convnet_fwd_tc: 2 to %d layers", TC_MAX_LAYERS);
    GB_REQUIRE(act && Wt && w && r && dinv && flags && epoch && status, "convnet_fwd_tc: missing argument");
    for (int l = 0; l < nlayers; ++l)
        GB_REQUIRE(act[l] && Wt[l] && (uintptr_t)act[l] % 16 == 0 && (uintptr_t)Wt[l] % 16 == 0,
                   "convnet_fwd_tc: buffers and weights must be 16-byte aligned");
    TcConv c{};
    size_t smem = 0;
    if (int rc = tc_setup(c, nx, ny, nz, nlayers, &smem)) return rc;
    // an x-plane block spans 2 span + 1 columns, whose counters one poll reads
    const int64_t span = ((int64_t)c.sy + 2 + TC_SUB * TC_OUT - 1) / (TC_SUB * TC_OUT);
    GB_REQUIRE(2 * span + 1 <= TC_POLL, "convnet_fwd_tc: grid too long in z (nz = %d)", nz);
    for (int l = 0; l < nlayers; ++l) {
        c.in[l] = static_cast<const unsigned char*>(act[l]);
        c.Wt[l] = static_cast<const __nv_bfloat16*>(Wt[l]);
        c.out[l] = l + 1 < nlayers ? static_cast<unsigned char*>(act[l + 1]) : nullptr;
    }
    c.w = w;
    c.r = r;
    c.dinv = dinv;
    c.mask = mask;
    c.omega = omega;
    c.status = status;
    c.flags = flags;
    c.epoch = epoch;
    c.chat = chat;
    c.ncomp = ncomp;
    if (int rc = tc_set_smem_attr()) return rc;
    void (*kern)(const TcConv) = ncomp == 3 ? k_conv3_tc<3, true> : k_conv3_tc<1, true>;
    // every CTA waits on other CTAs' items: all of them must be resident (cooperative launch)
    int per_sm = 0, coop = 0, dev = 0;
    GB_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TC_NET_THREADS, smem));
    GB_CHECK_CUDA(cudaGetDevice(&dev));
    GB_CHECK_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(c.nitems, (int64_t)sm_count()));
    if (!coop || per_sm < 1 || grid > per_sm * sm_count()) {
        gb::set_error("convnet_fwd_tc: the device cannot hold the whole-network launch's CTAs at once");
        return GB_ERR_UNSUPPORTED;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(TC_NET_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kern, (const TcConv)c));
    return GB_OK;
}
