// The DTFE surrogate's kernels: a 3-D convolutional network that maps a
// cloud-in-cell density grid to the DTFE density grid (log(1 + rho / mean)).
//
// Layout: activations chunk-planar, [c / 8][voxel][8 channels] (channel c of
// voxel v at ((c / 8) * V + v) * 8 + c % 8, voxel index (z * Y + y) * X + x),
// bf16, or FP32 for the f32 outputs; weights bf16 as [tap][c_out][c_in]
// (tap = (dz*3 + dy)*3 + dx for offsets dz, dy, dx in -1..1), with an FP32
// master copy for the update.  Channel counts are multiples of 16 (inputs)
// and 8 (outputs); X is a multiple of 16.  A plane of 8 channels is then one
// contiguous run along x, which is what the tensor-memory kernel's copies
// fetch.
//
// conv3d forward (and the data gradient, the same product with the weights
// flipped and transposed) is an implicit GEMM on the tensor cores.  For 16 or
// 32 channels in and out it runs on tcgen05 (k_conv3d_fwd_tc: TMA-fed slabs,
// tensor-memory accumulators, warp-specialised); other channel counts, and
// tessgpu_conv3d_set_engine(1), use mma.sync m16n8k16 (k_conv3d_fwd: a warp
// takes 16 consecutive voxels of one x row and every output channel, each tap
// and 16-channel slice of the input one k-step, A fragments read straight from
// the input).  The weight gradient reduces over voxels on the CUDA cores
// (FP32), per tap, with the block's voxel slice staged in shared memory.
#include <cuda.h>   // CUtensorMap and its encoder's types (the encoder comes through the runtime)
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "../../include/tess2_gb300.h"
#include "tc_common.cuh"

namespace {

using namespace tcg;

constexpr int MAX_COUT = 64;   // output channels per warp tile (8 n-tiles)

// element index of channel c of voxel v in the chunk-planar layout
__device__ __forceinline__ long long plidx(long long v, int c, long long V)
{
    return ((long long)(c >> 3) * V + v) * 8 + (c & 7);
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p)
{
    return *reinterpret_cast<const uint32_t*>(p);
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// y[v][co] = act(sum_{tap, ci} x[v + tap][ci] w[tap][co][ci] + bias[co]); act = relu when relu != 0.
// y_bf16 and/or y_f32 (either may be null) receive the result.
template <int NT>   // n-tiles of 8 output channels
__global__ void __launch_bounds__(128) k_conv3d_fwd(const __nv_bfloat16* __restrict__ x, int X, int Y, int Z, int cin,
                                                    const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias,
                                                    int relu, __nv_bfloat16* y_bf16, float* y_f32)
{
    const int lane = threadIdx.x & 31;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long tiles = (long long)X / 16 * Y * Z;
    if (warp >= tiles)
        return;
    const int cout = NT * 8;
    const int xt = (int)(warp % (X / 16));
    const int yy = (int)((warp / (X / 16)) % Y);
    const int zz = (int)(warp / ((long long)(X / 16) * Y));
    const int x0 = xt * 16;
    const int gid = lane >> 2, tig = lane & 3;
    const long long V = (long long)X * Y * Z;
    float acc[NT][4];
#pragma unroll
    for (int n = 0; n < NT; ++n)
        acc[n][0] = acc[n][1] = acc[n][2] = acc[n][3] = 0.0f;
    for (int tap = 0; tap < 27; ++tap)
    {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        const int sz = zz + dz, sy = yy + dy;
        const bool row_ok = sz >= 0 && sz < Z && sy >= 0 && sy < Y;
        const int xa = x0 + gid + dx, xb = x0 + gid + 8 + dx;
        const bool oka = row_ok && xa >= 0 && xa < X, okb = row_ok && xb >= 0 && xb < X;
        const long long va = oka ? ((long long)sz * Y + sy) * X + xa : 0;
        const long long vb = okb ? ((long long)sz * Y + sy) * X + xb : 0;
        for (int c = 0; c < cin; c += 16)
        {
            uint32_t a[4];
            a[0] = oka ? ld_pair(x + plidx(va, c + tig * 2, V)) : 0u;
            a[1] = okb ? ld_pair(x + plidx(vb, c + tig * 2, V)) : 0u;
            a[2] = oka ? ld_pair(x + plidx(va, c + 8 + tig * 2, V)) : 0u;
            a[3] = okb ? ld_pair(x + plidx(vb, c + 8 + tig * 2, V)) : 0u;
#pragma unroll
            for (int n = 0; n < NT; ++n)
            {
                const __nv_bfloat16* wr = w + ((long long)tap * cout + n * 8 + gid) * cin + c + tig * 2;
                uint32_t b[2] = { ld_pair(wr), ld_pair(wr + 8) };
                mma_bf16(acc[n], a, b);
            }
        }
    }
    const long long v0 = ((long long)zz * Y + yy) * X + x0;
#pragma unroll
    for (int n = 0; n < NT; ++n)
    {
        const int co = n * 8 + tig * 2;
        float r[4] = { acc[n][0], acc[n][1], acc[n][2], acc[n][3] };
        if (bias)
        {
            r[0] += bias[co]; r[1] += bias[co + 1];
            r[2] += bias[co]; r[3] += bias[co + 1];
        }
        if (relu)
#pragma unroll
            for (int i = 0; i < 4; ++i) r[i] = fmaxf(r[i], 0.0f);
        const long long va = v0 + gid, vb = v0 + gid + 8;
        if (y_bf16)
        {
            *reinterpret_cast<__nv_bfloat162*>(y_bf16 + plidx(va, co, V)) = __floats2bfloat162_rn(r[0], r[1]);
            *reinterpret_cast<__nv_bfloat162*>(y_bf16 + plidx(vb, co, V)) = __floats2bfloat162_rn(r[2], r[3]);
        }
        if (y_f32)
        {
            *reinterpret_cast<float2*>(y_f32 + plidx(va, co, V)) = make_float2(r[0], r[1]);
            *reinterpret_cast<float2*>(y_f32 + plidx(vb, co, V)) = make_float2(r[2], r[3]);
        }
    }
}

// ---------------------------------------------------------------------------
// the same forward pass on the 5th-generation tensor cores (tcgen05)
// ---------------------------------------------------------------------------
// A tile is 128 consecutive voxels x0 .. x0 + 127 of one x row (the M of one
// MMA; positions past X are computed and dropped) x c_out (its N).  One
// persistent CTA per SM keeps all 27 taps' weights in shared memory (K-major
// core-matrix layout: 8 rows x 16 bytes per core matrix).  Per (dz, dy) a tile
// needs one slab: positions x0 - 1 .. x0 + 128 of the x row shifted by
// (dy, dz), stored as c_in / 8 planes of 16-byte rows; the three taps
// dx = -1, 0, 1 read that slab at row offsets 0, 1, 2 (start addresses 16
// bytes apart in the shared-memory descriptor).  Tiles go in groups of four
// on consecutive y rows of one (x range, z), one per MMA warp; for each dz the
// group's six input rows y0 - 1 .. y0 + 4 are one slab each and serve up to
// three tiles (as dy = +1, 0, -1), so a group loads 18 slabs instead of 36 and
// an input row is fetched 4.5 times per output tile instead of 27.  Warp
// roles, synchronised through mbarriers only (no block-wide barrier in the
// loop):
//   warps 4-5  TMA (alternate slabs of a group): per slab one
//              cp.async.bulk.tensor copy per plane (box 8 channels x 130
//              positions of a 5-D view (8, X, Y, Z, c_in / 8) of the
//              chunk-planar input: 2,080 contiguous bytes); positions outside
//              the grid (the x halo, rows past y or z) arrive as zeros without
//              a memory read; the buffer's "full" barrier completes on the
//              copies' bytes, its "empty" barrier on three arrivals (one commit
//              per consuming tile, the loader standing in for absent ones);
//   warps 6-9  MMA (one tile of each group each; warp 6 allocates tensor
//              memory): the whole warp runs the loop (so the descriptors stay
//              warp-uniform) and its elected lane issues tcgen05.mma
//              (kind::f16, bf16 x bf16 -> f32) for each slab, commits them to
//              the buffer's "empty" barrier and the finished tile to its
//              accumulator's "full" barrier (two sets of four accumulators
//              alternate between groups);
//   warps 0-3  epilogue: tcgen05.ld of row tid (warp w reads lanes 32w..),
//              release the accumulators, bias, ReLU, store the rows inside X.
// Every wait is bounded; a timed-out wait raises an abort flag that ends every
// role's loop, the kernel reports it in *err, waits for the copies in flight
// and its MMAs (bounded) and frees its tensor memory.
constexpr int TC_M = 128;      // GEMM rows per tile
constexpr int TC_SLAB = 136;   // rows per slab plane (>= 130, a multiple of 8)
constexpr int TC_PLANE = TC_SLAB * 16;
#ifndef TESSGPU_CONV_TILES
#define TESSGPU_CONV_TILES 4
#endif
constexpr int TC_T = TESSGPU_CONV_TILES;   // tiles per group = MMA-issuing warps
constexpr int TC_LOADERS = 2;              // TMA warps
constexpr int TC_TMA_WARP = 4, TC_MMA_WARP = 4 + TC_LOADERS;
constexpr int TC_THREADS = 32 * (4 + TC_LOADERS + TC_T);   // epilogue, TMA, MMA warps
constexpr int TC_BOX = 130;            // positions per slab plane a TMA copy writes
constexpr int TC_SMEM = 227 * 1024;    // dynamic shared memory a CTA may opt into

template <int COUT, int CIN>
struct TcLayout
{
    static constexpr int TAPB = COUT * CIN * 2;    // one tap's weights
    static constexpr int WBYTES = 27 * TAPB;
    static constexpr int SBYTES = (CIN / 8) * TC_PLANE;
    static constexpr int FIT = (TC_SMEM - WBYTES - 512) / SBYTES;
    static constexpr int STAGES = FIT < 40 ? FIT : 40;
    static constexpr int BAR = WBYTES + STAGES * SBYTES;   // mbarriers, tensor-memory address, abort flag
    // full[STAGES], empty[STAGES], acc_full[2][TC_T], acc_empty[2], fin
    static constexpr int OFF_FULL = BAR, OFF_EMPTY = BAR + 8 * STAGES, OFF_ACCF = BAR + 16 * STAGES,
                         OFF_ACCE = OFF_ACCF + 16 * TC_T, OFF_FIN = OFF_ACCE + 16, OFF_TMEM = OFF_FIN + 8,
                         OFF_ABORT = OFF_TMEM + 4, OFF_LAST = OFF_ABORT + 4, OFF_BIAS = OFF_LAST + 4 * STAGES;
    static constexpr int TOTAL = OFF_BIAS + 4 * COUT;
    // two sets of TC_T accumulators of COUT columns; a power of two >= 32
    static constexpr int ACOLS = 2 * TC_T * COUT;   // two sets of TC_T accumulators
    static constexpr int TCOLS = ACOLS <= 32 ? 32 : (ACOLS <= 64 ? 64 : (ACOLS <= 128 ? 128 : (ACOLS <= 256 ? 256 : 512)));
    static_assert(ACOLS <= 512, "tensor memory");
    static_assert(STAGES >= 3, "shared memory too small for the slab ring");
    static_assert(TOTAL <= TC_SMEM, "shared memory");
};

template <int COUT, int CIN>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_conv3d_fwd_tc(const __grid_constant__ CUtensorMap xmap, int X, int Y, int Z,
                    const __nv_bfloat16* __restrict__ w, const float* __restrict__ bias, int relu,
                    __nv_bfloat16* y_bf16, float* y_f32, int* err)
{
    using L = TcLayout<COUT, CIN>;
    constexpr int CH = CIN / 8;   // 16-byte chunks per row
    constexpr int S = L::STAGES;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // group q: TC_T tiles on consecutive y rows of one (x range, z): xt = q % per_row,
    // yb = (q / per_row) % nyb, z = q / (per_row * nyb); tile t covers x0 = xt * 128 .. of row
    // y = yb * TC_T + t (t < Tg = min(TC_T, Y - yb * TC_T))
    const int per_row = (X + TC_M - 1) / TC_M;
    const int nyb = (Y + TC_T - 1) / TC_T;
    const int groups = per_row * nyb * Z;   // < 2^31, checked by the launcher
    const long long V = (long long)X * Y * Z;
    const int NG = (int)blockIdx.x < groups ? (groups - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t slab_a = s_base + L::WBYTES;   // buffer b at slab_a + b * SBYTES
    const uint32_t full0 = s_base + L::OFF_FULL, empty0 = s_base + L::OFF_EMPTY;
    const uint32_t accf0 = s_base + L::OFF_ACCF, acce0 = s_base + L::OFF_ACCE, fin = s_base + L::OFF_FIN;
    volatile int* abort = reinterpret_cast<volatile int*>(smem + L::OFF_ABORT);
    float* sbias = reinterpret_cast<float*>(smem + L::OFF_BIAS);
    int* last_slab = reinterpret_cast<int*>(smem + L::OFF_LAST);   // per ring slot: the last slab copied into it

    // all taps' weights -> shared memory: row co of tap t, chunk c at
    // t * TAPB + (co / 8) * (CH * 128) + c * 128 + (co % 8) * 16
    const uint4* wg = reinterpret_cast<const uint4*>(w);
    for (int i = tid; i < 27 * COUT * CH; i += TC_THREADS)
    {
        const int t = i / (COUT * CH), rem = i % (COUT * CH), r = rem / CH, c = rem % CH;
        *reinterpret_cast<uint4*>(smem + t * L::TAPB + (r / 8) * (CH * 128) + c * 128 + (r % 8) * 16) = wg[i];
    }
    if (tid < COUT) sbias[tid] = bias ? bias[tid] : 0.0f;
    for (int b = tid; b < S; b += TC_THREADS) last_slab[b] = -1;
    if (tid == 0)
    {
        for (int b = 0; b < S; ++b)
        {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * b));   // expect_tx + copies
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 3;" ::"r"(empty0 + 8 * b));    // three uses
        }
        for (int a = 0; a < 2 * TC_T; ++a)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(accf0 + 8 * a));     // one commit
        for (int a = 0; a < 2; ++a)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(acce0 + 8 * a));   // 128 epilogue threads
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(fin), "n"(TC_T));   // one commit per MMA warp
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == TC_MMA_WARP)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_base + L::OFF_TMEM),
                     "r"(L::TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tbase = *reinterpret_cast<const volatile uint32_t*>(smem + L::OFF_TMEM);

    // A group's tiles share their slabs: for each dz the R = Tg + 2 input rows
    // y0 - 1 .. y0 + Tg (y0 = yb * TC_T) are one slab each, used by up to three
    // tiles (as dy = +1, 0, -1), so a group of four loads 18 slabs, not 36.
    // Slabs run in the order (group, dz, row), one ring position each; a slab's
    // "empty" barrier expects three arrivals: one commit per consuming tile and
    // the rest from the loader.
    if (warp >= TC_TMA_WARP && warp < TC_TMA_WARP + TC_LOADERS)
    {
        // ---- TMA (tiles t = w, w + TC_LOADERS, .. of each group): per slab one copy per 8-channel
        // plane; positions outside the grid arrive as zeros ----
        const int w = warp - TC_TMA_WARP;
        const bool leader = elect_one();
        const uint64_t map = reinterpret_cast<uint64_t>(&xmap);
        if (leader) asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
        bool stop = false;
        int mbase = 0;   // the group's first slab
        for (int G = 0; G < NG && !stop; ++G)
        {
            const int q = (int)blockIdx.x + G * (int)gridDim.x;
            const int xt = q % per_row, yb = (q / per_row) % nyb, z = q / (per_row * nyb);
            const int Tg = min(TC_T, Y - yb * TC_T), R = Tg + 2;
            const int x0 = xt * TC_M, y0 = yb * TC_T;
            for (int j = w; j < 3 * R && !stop; j += TC_LOADERS)
            {
                const int dz = j / R - 1, rho = j % R;   // input row y0 - 1 + rho of plane z + dz
                const int m = mbase + j, b = m % S;
                if (m >= S && !warp_wait(empty0 + 8 * b, (uint32_t)((m / S - 1) & 1), abort))
                {
                    stop = true;
                    break;
                }
                // tiles using this row: t in [rho - 2, rho] within the group
                const int ncons = min(Tg - 1, rho) - max(0, rho - 2) + 1;
                if (leader)
                {
                    last_slab[b] = m;
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full0 + 8 * b),
                                 "r"((uint32_t)(CH * TC_BOX * 16))
                                 : "memory");
#pragma unroll
                    for (int c = 0; c < CH; ++c)
                        asm volatile(
                            "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                            " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(slab_a + b * L::SBYTES + c * TC_PLANE),
                            "l"(map), "r"(0), "r"(x0 - 1), "r"(y0 - 1 + rho), "r"(z + dz), "r"(c), "r"(full0 + 8 * b)
                            : "memory");
                    for (int k = ncons; k < 3; ++k) mbar_arrive(empty0 + 8 * b);   // absent consumers
                }
                __syncwarp();
            }
            mbase += 3 * R;
        }
    }
    else if (warp >= TC_MMA_WARP)
    {
        // ---- MMA issue (tile t = warp - TC_MMA_WARP of each group): the whole warp runs the loop
        // (descriptors stay warp-uniform), the elected lane issues every tcgen05.mma and commit ----
        const int ti = warp - TC_MMA_WARP;
        // D f32; A, B bf16, both K-major; N = COUT, M = 128
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);
        const bool leader = elect_one();
        // descriptors as a base plus a byte offset / 16 in the start-address field (shared memory
        // addresses stay below 2^18, so the 14-bit field never carries)
        const uint64_t adesc0 = umma_sdesc(slab_a, TC_PLANE, 128);
        const uint64_t bdesc0 = umma_sdesc(s_base, 128, CH * 128);
        bool go = true;
        int mbase = 0;   // the group's first slab
        for (int G = 0; G < NG && go; ++G)
        {
            const int q = (int)blockIdx.x + G * (int)gridDim.x;
            const int yb = (q / per_row) % nyb;
            const int Tg = min(TC_T, Y - yb * TC_T), R = Tg + 2, A = G & 1;
            // the epilogue has read this accumulator set's tiles of group G - 2
            if (G >= 2 && !warp_wait(acce0 + 8 * A, (uint32_t)(((G - 2) >> 1) & 1), abort)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t dcol = tbase + (uint32_t)((A * TC_T + ti) * COUT);
            // a warp without a tile in a short group still commits (nothing) to its accumulator's
            // barrier, so that every slot completes one phase per group
            for (int g = 0; g < 9 && go && ti < Tg; ++g)
            {
                const int n = mbase + (g / 3) * R + ti + g % 3, b = n % S;   // row y0 + ti + dy
                go = warp_wait(full0 + 8 * b, (uint32_t)((n / S) & 1), abort);
                if (!go) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                for (int sh = 0; sh < 3; ++sh)
#pragma unroll
                    for (int ks = 0; ks < CIN / 16; ++ks)
                    {
                        const int tap = g * 3 + sh;
                        const uint64_t db = bdesc0 + (uint64_t)((tap * L::TAPB + ks * 256) >> 4);
                        const uint64_t da =
                            adesc0 + (uint64_t)((b * L::SBYTES + sh * 16 + ks * 2 * TC_PLANE) >> 4);
                        const uint32_t acc = (g > 0 || sh > 0 || ks > 0) ? 1u : 0u;
                        if (leader)
                            asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dcol),
                                         "l"(da), "l"(db), "r"(idesc), "r"(acc));
                    }
                if (leader)
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     empty0 + 8 * b)
                                 : "memory");
                __syncwarp();
            }
            if (!go) break;
            if (leader)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 accf0 + 8 * (A * TC_T + ti))
                             : "memory");
            __syncwarp();
            mbase += 3 * R;
        }
        // every MMA issued has completed once fin's first phase does
        if (leader)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(fin)
                         : "memory");
        __syncwarp();
        mbar_wait_bounded(fin, 0u);
        __syncwarp();
    }
    else
    {
        // ---- epilogue (warps 0-3: tensor-memory lanes 32 warp .. 32 warp + 31) ----
        for (int G = 0; G < NG; ++G)
        {
            const int q = (int)blockIdx.x + G * (int)gridDim.x;
            const int xt = q % per_row, yb = (q / per_row) % nyb, z = q / (per_row * nyb);
            const int Tg = min(TC_T, Y - yb * TC_T), A = G & 1;
            bool ok = true;
            for (int t = 0; t < Tg && ok; ++t)
            {
                bool ready = false;
                if (lane == 0)
                    ready = mbar_wait_or_abort(accf0 + 8 * (A * TC_T + t), (uint32_t)((G >> 1) & 1), abort);
                ok = __shfl_sync(0xffffffffu, ready ? 1 : 0, 0) != 0;
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                uint32_t acc[COUT];
                const uint32_t taddr =
                    tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)((A * TC_T + t) * COUT);
#pragma unroll
                for (int c = 0; c < COUT; c += 16)
                    tmem_ld16(taddr + c, acc + c);
                asm volatile("tcgen05.wait::ld.sync.aligned;");
                if (t == Tg - 1)
                {
                    // every accumulator of the group is read: hand the set back to the MMA warps
                    asm volatile("tcgen05.fence::before_thread_sync;");
                    mbar_arrive(acce0 + 8 * A);
                }
                const int ox = xt * TC_M + tid;
                if (ox < X)
                {
                    const long long vox = ((long long)z * Y + yb * TC_T + t) * X + ox;
                    float f[COUT];
#pragma unroll
                    for (int c = 0; c < COUT; ++c)
                    {
                        f[c] = __uint_as_float(acc[c]) + sbias[c];
                        if (relu) f[c] = fmaxf(f[c], 0.0f);
                    }
                    // chunk-planar: 8 channels (16 or 32 bytes) per plane, consecutive threads adjacent
                    if (y_bf16)
#pragma unroll
                        for (int c = 0; c < COUT; c += 8)
                            *reinterpret_cast<uint4*>(y_bf16 + ((c >> 3) * V + vox) * 8) =
                                make_uint4(pack_bf16(f[c], f[c + 1]), pack_bf16(f[c + 2], f[c + 3]),
                                           pack_bf16(f[c + 4], f[c + 5]), pack_bf16(f[c + 6], f[c + 7]));
                    if (y_f32)
#pragma unroll
                        for (int c = 0; c < COUT; c += 8)
                        {
                            float4* o = reinterpret_cast<float4*>(y_f32 + ((c >> 3) * V + vox) * 8);
                            o[0] = make_float4(f[c], f[c + 1], f[c + 2], f[c + 3]);
                            o[1] = make_float4(f[c + 4], f[c + 5], f[c + 6], f[c + 7]);
                        }
                }
            }
            if (!ok) break;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // no copy may still be landing in shared memory when the CTA exits (after an abort the MMA
    // warps may not have consumed every slab): wait for the last copy into each slot
    for (int b = tid; b < S; b += TC_THREADS)
    {
        const int m = last_slab[b];
        if (m >= 0) mbar_wait_bounded(full0 + 8 * b, (uint32_t)((m / S) & 1));
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicExch(err, 1);
    if (warp == TC_MMA_WARP)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(L::TCOLS));
}

// ---------------------------------------------------------------------------
// the weight gradient on the tensor cores (tcgen05)
// ---------------------------------------------------------------------------
// dw[tap][co][ci] += sum_v dy[v][co] x[v + tap][ci].  A tile is 128 voxels
// x0 .. x0 + 127 of one x row; for the tap (dz, dy, dx) its share is
// sum_r dyT[r][co] slab[r + dx + 1][ci], with dyT the tile of the output
// gradient (zero past X) and slab positions x0 - 1 .. x0 + 128 of the input row
// shifted by (dy, dz), both chunk-planar.  As one MMA per 16 rows r: D[co][ci]
// with A = dyT (M = 128: c_out rows and zero planes up to 128), B = the slab
// read from row dx + 1 (N = c_in), both MN-major straight from the planes
// (LBO = 8 rows, SBO = one plane).  A CTA takes one dz (blockIdx.x % 3) and
// keeps the nine taps of that dz in tensor memory across all of its tiles (9
// accumulators of c_in columns); at the end warps 0-3 read them (lane = c_out)
// and add them to dw, one atomic per weight and CTA.  Warp 4 loads a tile
// (the dyT planes and three slabs) by TMA into one of two stages while warp 5
// issues the previous tile's 72 MMAs.  Waits are bounded as in the forward
// kernel.
constexpr int WG_TILE = 128;
constexpr int WG_APLANE = WG_TILE * 16;            // one plane of dyT
constexpr int WG_ABYTES = 16 * WG_APLANE;          // 16 planes: M = 128 (unused planes stay zero)
constexpr int WG_THREADS_TC = 192;                 // warps 0-3 epilogue, 4 TMA, 5 MMA
constexpr int WG_MIN_SMEM = 120 * 1024;            // one CTA per SM (its tensor memory is the SM's half)

template <int COUT, int CIN>
struct WgLayout
{
    static constexpr int CH = CIN / 8;
    static constexpr int SBYTES = CH * TC_PLANE;             // one slab
    static constexpr int STAGE = WG_ABYTES + 3 * SBYTES;     // dyT + the three slabs of a dz
    static constexpr int BAR = 2 * STAGE;                    // full[2], empty[2], fin, tmem, abort, last[2]
    static constexpr int OFF_FULL = BAR, OFF_EMPTY = BAR + 16, OFF_FIN = BAR + 32, OFF_TMEM = BAR + 40,
                         OFF_ABORT = BAR + 44, OFF_LAST = BAR + 48;
    static constexpr int USED = OFF_LAST + 8;
    static constexpr int TOTAL = USED > WG_MIN_SMEM ? USED : WG_MIN_SMEM;
    static constexpr int ACOLS = 9 * CIN;
    static constexpr int TCOLS = ACOLS <= 128 ? 128 : (ACOLS <= 256 ? 256 : 512);
    static constexpr uint32_t TX = (uint32_t)((COUT / 8) * WG_TILE * 16 + 3 * CH * TC_BOX * 16);
    static_assert(ACOLS <= 512, "tensor memory");
    static_assert(TOTAL <= TC_SMEM, "shared memory");
};

template <int COUT, int CIN>
__global__ void __launch_bounds__(WG_THREADS_TC, 1)
    k_conv3d_wgrad_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap dymap, int X,
                      int Y, int Z, float* dw, int* err)
{
    using L = WgLayout<COUT, CIN>;
    constexpr int CH = L::CH;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    const int per_row = (X + WG_TILE - 1) / WG_TILE;
    const int tiles = per_row * Y * Z;   // < 2^31, checked by the launcher
    const int dz = (int)(blockIdx.x % 3) - 1, lanes = (int)gridDim.x / 3, me = (int)blockIdx.x / 3;
    const int ntl = me < tiles ? (tiles - 1 - me) / lanes + 1 : 0;
    const uint32_t s_base = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t full0 = s_base + L::OFF_FULL, empty0 = s_base + L::OFF_EMPTY, fin = s_base + L::OFF_FIN;
    volatile int* abort = reinterpret_cast<volatile int*>(smem + L::OFF_ABORT);
    int* last = reinterpret_cast<int*>(smem + L::OFF_LAST);   // per stage: the last tile loaded into it

    // the dyT planes past c_out stay zero for the whole kernel
    for (int i = tid; i < 2 * (16 - COUT / 8) * WG_APLANE / 16; i += blockDim.x)
    {
        const int per = (16 - COUT / 8) * WG_APLANE / 16, s = i / per, j = i % per;
        reinterpret_cast<uint4*>(smem + s * L::STAGE + (COUT / 8) * WG_APLANE)[j] = make_uint4(0, 0, 0, 0);
    }
    if (tid < 2) last[tid] = -1;
    if (tid == 0)
    {
        for (int s = 0; s < 2; ++s)
        {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * s));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(empty0 + 8 * s));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fin));
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (warp == 5)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_base + L::OFF_TMEM),
                     "r"(L::TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tbase = *reinterpret_cast<const volatile uint32_t*>(smem + L::OFF_TMEM);
    bool ok = true;

    if (warp == 4)
    {
        // ---- TMA: per tile the dyT planes and, for dy = -1, 0, 1, the slab of row (y + dy, z + dz) ----
        const bool leader = elect_one();
        const uint64_t xm = reinterpret_cast<uint64_t>(&xmap), dm = reinterpret_cast<uint64_t>(&dymap);
        for (int k = 0; k < ntl; ++k)
        {
            const int s = k & 1;
            if (k >= 2 && !warp_wait(empty0 + 8 * s, (uint32_t)(((k - 2) >> 1) & 1), abort)) break;
            const int t = me + k * lanes, r = t / per_row, x0 = (t - r * per_row) * WG_TILE;
            const int y = r % Y, z = r / Y;
            const uint32_t st = s_base + s * L::STAGE;
            if (leader)
            {
                last[s] = k;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full0 + 8 * s),
                             "r"(L::TX)
                             : "memory");
#pragma unroll
                for (int p = 0; p < COUT / 8; ++p)
                    asm volatile(
                        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(st + p * WG_APLANE),
                        "l"(dm), "r"(0), "r"(x0), "r"(y), "r"(z), "r"(p), "r"(full0 + 8 * s)
                        : "memory");
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int c = 0; c < CH; ++c)
                        asm volatile(
                            "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                            " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(st + WG_ABYTES + d * L::SBYTES +
                                                                              c * TC_PLANE),
                            "l"(xm), "r"(0), "r"(x0 - 1), "r"(y + d - 1), "r"(z + dz), "r"(c), "r"(full0 + 8 * s)
                            : "memory");
            }
            __syncwarp();
        }
    }
    else if (warp == 5)
    {
        // ---- MMA: D[tap (dy, dx)][co][ci] += dyT^T slab, 8 MMAs of 16 rows per tap and tile ----
        // D f32; A, B bf16, both MN-major (bits 15, 16); N = CIN, M = 128
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                               ((uint32_t)(CIN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
        const bool leader = elect_one();
        const uint64_t adesc0 = umma_sdesc(s_base, 128, WG_APLANE);
        const uint64_t bdesc0 = umma_sdesc(s_base + WG_ABYTES, 128, TC_PLANE);
        for (int k = 0; k < ntl && ok; ++k)
        {
            const int s = k & 1;
            ok = warp_wait(full0 + 8 * s, (uint32_t)((k >> 1) & 1), abort);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int sh = 0; sh < 3; ++sh)
#pragma unroll
                    for (int ks = 0; ks < WG_TILE / 16; ++ks)
                    {
                        const uint64_t da = adesc0 + (uint64_t)((s * L::STAGE + ks * 256) >> 4);
                        const uint64_t db =
                            bdesc0 + (uint64_t)((s * L::STAGE + d * L::SBYTES + sh * 16 + ks * 256) >> 4);
                        const uint32_t acc = (k > 0 || ks > 0) ? 1u : 0u;
                        if (leader)
                            asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                                             tbase + (uint32_t)((d * 3 + sh) * CIN)),
                                         "l"(da), "l"(db), "r"(idesc), "r"(acc));
                    }
            if (leader)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 empty0 + 8 * s)
                             : "memory");
            __syncwarp();
        }
        if (leader)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(fin)
                         : "memory");
        __syncwarp();
        if (!mbar_wait_bounded(fin, 0u)) *abort = 1;
        __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // no copy may still be landing when the CTA reads or exits
    if (tid < 2 && last[tid] >= 0) mbar_wait_bounded(full0 + 8 * tid, (uint32_t)((last[tid] >> 1) & 1));
    __syncthreads();
    const bool good = *abort == 0;
    if (warp < 4 && good && ntl > 0)
    {
        // lane 32 warp + l = row co of every accumulator
        const int co = tid;
#pragma unroll 1
        for (int tap = 0; tap < 9; ++tap)
        {
            uint32_t v[CIN];
#pragma unroll
            for (int c = 0; c < CIN; c += 16)
                tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)(tap * CIN + c), v + c);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
            if (co < COUT)
            {
                float* out = dw + ((long long)((dz + 1) * 9 + tap) * COUT + co) * CIN;
#pragma unroll
                for (int c = 0; c < CIN; ++c) atomicAdd(out + c, __uint_as_float(v[c]));
            }
        }
    }
    if (tid == 0 && !good) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 5)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(L::TCOLS));
}

// db[co] += sum_v dy[v][co] (chunk-planar dy): block partial sums, one atomic per channel and block
__global__ void __launch_bounds__(256) k_bias_grad(const __nv_bfloat16* __restrict__ dy, long long V, int cout,
                                                   float* db)
{
    __shared__ float part[8][32];
    const int plane = blockIdx.y;   // 8 channels
    float acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    {
        const uint4 q = reinterpret_cast<const uint4*>(dy + ((long long)plane * V + v) * 8)[0];
        const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            const float2 f = __bfloat1622float2(h[i]);
            acc[2 * i] += f.x;
            acc[2 * i + 1] += f.y;
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
        float a = acc[i];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) part[i][wid] = a;
    }
    __syncthreads();
    if (threadIdx.x < 8)
    {
        float a = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += part[threadIdx.x][w];
        atomicAdd(&db[plane * 8 + threadIdx.x], a);
    }
}

// dw[tap][co][ci] += sum_v dy[v][co] x[v + tap][ci]; db[co] += sum_v dy[v][co]
// (FP32 accumulation).  Block: one tap, VB voxels of one x row band; thread
// (co, ci) pairs.
constexpr int VB = 128;
__global__ void __launch_bounds__(256) k_conv3d_wgrad(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ dy,
                                                      int X, int Y, int Z, int cin, int cout, float* dw, float* db)
{
    extern __shared__ float sm[];
    float* sdy = sm;                 // [VB][cout]
    float* sx = sm + VB * cout;      // [VB][cin]
    const int tap = blockIdx.y;
    const int dz = tap / 9 - 1, dy_ = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
    const long long V = (long long)X * Y * Z;
    const long long v0 = (long long)blockIdx.x * VB;
    for (int i = threadIdx.x; i < VB * cout; i += blockDim.x)
    {
        const long long v = v0 + i / cout;
        sdy[i] = v < V ? __bfloat162float(dy[plidx(v, i % cout, V)]) : 0.0f;
    }
    for (int i = threadIdx.x; i < VB * cin; i += blockDim.x)
    {
        const long long v = v0 + i / cin;
        float val = 0.0f;
        if (v < V)
        {
            const int xx = (int)(v % X), yy = (int)((v / X) % Y), zz = (int)(v / ((long long)X * Y));
            const int sx_ = xx + dx, sy = yy + dy_, sz = zz + dz;
            if (sx_ >= 0 && sx_ < X && sy >= 0 && sy < Y && sz >= 0 && sz < Z)
                val = __bfloat162float(x[plidx(((long long)sz * Y + sy) * X + sx_, i % cin, V)]);
        }
        sx[i] = val;
    }
    __syncthreads();
    for (int p = threadIdx.x; p < cout * cin; p += blockDim.x)
    {
        const int co = p / cin, ci = p % cin;
        float acc = 0.0f;
        for (int v = 0; v < VB; ++v)
            acc += sdy[v * cout + co] * sx[v * cin + ci];
        atomicAdd(&dw[((long long)tap * cout + co) * cin + ci], acc);
    }
    if (tap == 13 && db)
        for (int co = threadIdx.x; co < cout; co += blockDim.x)
        {
            float acc = 0.0f;
            for (int v = 0; v < VB; ++v)
                acc += sdy[v * cout + co];
            atomicAdd(&db[co], acc);
        }
}

// weights for the data gradient: wt[26 - tap][ci][co] = w[tap][co][ci] (bf16 from the FP32 master)
__global__ void k_flip_weights(const float* w, int cout, int cin, __nv_bfloat16* w_bf16, __nv_bfloat16* wt_bf16)
{
    const int n = 27 * cout * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int tap = i / (cout * cin), co = (i / cin) % cout, ci = i % cin;
        const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
        w_bf16[i] = v;
        wt_bf16[((26 - tap) * cin + ci) * cout + co] = v;
    }
}

// g (FP32, [V][c]) times relu'(y) (y the layer's bf16 output) -> bf16 gradient
__global__ void k_relu_grad(const float* g, const __nv_bfloat16* y, long long n, __nv_bfloat16* out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(__bfloat162float(y[i]) > 0.0f ? g[i] : 0.0f);
}

// Adam with bias correction (FP32 master weights)
__global__ void k_adam(float* w, const float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

int blocks_for(long long n, int t)
{
    long long b = (n + t - 1) / t;
    return (int)(b < 1 ? 1 : (b > 65535LL * 8 ? 65535LL * 8 : b));
}

__device__ int g_conv_err;   // raised by a tcgen05 kernel whose bounded wait ran out
int g_conv_engine = 0;       // 0: tcgen05 where the channel counts allow, 1: mma.sync only

template <int COUT, int CIN>
tessgpu_status launch_fwd_tc(const __nv_bfloat16* x, int X, int Y, int Z, const __nv_bfloat16* w, const float* bias,
                             int relu, __nv_bfloat16* yb, float* yf, cudaStream_t s)
{
    using L = TcLayout<COUT, CIN>;
    static int sms_of[64];   // SMs per device ordinal, once the kernel is set up there
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TESSGPU_ERR_CUDA;
    if (!sms_of[dev])
    {
        int optin = 0, sms = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (optin < L::TOTAL || sms <= 0) return TESSGPU_ERR_UNSUPPORTED;
        if (cudaFuncSetAttribute(k_conv3d_fwd_tc<COUT, CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, L::TOTAL) !=
            cudaSuccess)
            return TESSGPU_ERR_CUDA;
        sms_of[dev] = sms;
    }
    int* err = nullptr;
    if (cudaGetSymbolAddress((void**)&err, g_conv_err) != cudaSuccess) return TESSGPU_ERR_CUDA;
    const long long tiles = (long long)((X + TC_M - 1) / TC_M) * ((Y + TC_T - 1) / TC_T) * Z;   // groups
    const EncodeTiled encode = tensor_map_encoder();
    if (tiles >= (1LL << 31) || !encode || ((uintptr_t)x & 15)) return TESSGPU_ERR_UNSUPPORTED;
    // the chunk-planar input as (8 channels, X, Y, Z, CIN / 8 planes); a box is TC_BOX positions
    // of one plane, 2,080 contiguous bytes
    CUtensorMap xmap;
    const cuuint64_t dims[5] = { 8, (cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(CIN / 8) };
    const cuuint64_t strides[4] = { 16, (cuuint64_t)X * 16, (cuuint64_t)X * Y * 16, (cuuint64_t)X * Y * Z * 16 };
    const cuuint32_t box[5] = { 8, (cuuint32_t)TC_BOX, 1, 1, 1 };
    const cuuint32_t estride[5] = { 1, 1, 1, 1, 1 };
    if (encode(&xmap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void*)x, dims, strides, box, estride,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return TESSGPU_ERR_UNSUPPORTED;
    // one persistent CTA per SM (the slab ring fills its shared memory)
    const int grid = (int)(tiles < sms_of[dev] ? tiles : sms_of[dev]);
    k_conv3d_fwd_tc<COUT, CIN><<<grid, TC_THREADS, L::TOTAL, s>>>(xmap, X, Y, Z, w, bias, relu, yb, yf, err);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

// a chunk-planar activation (c channels) as (8 channels, X, Y, Z, c / 8); a box is rows positions of one plane
bool planar_map(CUtensorMap* map, const void* base, int X, int Y, int Z, int c, int rows)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode || ((uintptr_t)base & 15)) return false;
    const cuuint64_t dims[5] = { 8, (cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(c / 8) };
    const cuuint64_t strides[4] = { 16, (cuuint64_t)X * 16, (cuuint64_t)X * Y * 16, (cuuint64_t)X * Y * Z * 16 };
    const cuuint32_t box[5] = { 8, (cuuint32_t)rows, 1, 1, 1 };
    const cuuint32_t estride[5] = { 1, 1, 1, 1, 1 };
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int COUT, int CIN>
tessgpu_status launch_wgrad_tc(const __nv_bfloat16* x, const __nv_bfloat16* dy, int X, int Y, int Z, float* dw,
                               cudaStream_t s)
{
    using L = WgLayout<COUT, CIN>;
    static int sms_of[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TESSGPU_ERR_CUDA;
    if (!sms_of[dev])
    {
        int optin = 0, sms = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (optin < L::TOTAL || sms < 3) return TESSGPU_ERR_UNSUPPORTED;
        if (cudaFuncSetAttribute(k_conv3d_wgrad_tc<COUT, CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 L::TOTAL) != cudaSuccess)
            return TESSGPU_ERR_CUDA;
        sms_of[dev] = sms;
    }
    int* err = nullptr;
    if (cudaGetSymbolAddress((void**)&err, g_conv_err) != cudaSuccess) return TESSGPU_ERR_CUDA;
    const long long tiles = (long long)((X + WG_TILE - 1) / WG_TILE) * Y * Z;
    CUtensorMap xmap, dymap;
    if (tiles >= (1LL << 31) || !planar_map(&xmap, x, X, Y, Z, CIN, TC_BOX) ||
        !planar_map(&dymap, dy, X, Y, Z, COUT, WG_TILE))
        return TESSGPU_ERR_UNSUPPORTED;
    // one CTA per SM, a third of them per dz
    long long lanes = sms_of[dev] / 3;
    if (lanes > tiles) lanes = tiles;
    k_conv3d_wgrad_tc<COUT, CIN><<<(unsigned)(3 * lanes), WG_THREADS_TC, L::TOTAL, s>>>(xmap, dymap, X, Y, Z, dw,
                                                                                      err);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

}  // namespace

extern "C" tessgpu_status tessgpu_conv3d_set_engine(int engine)
{
    if (engine != 0 && engine != 1) return TESSGPU_ERR_INVALID;
    g_conv_engine = engine;
    return TESSGPU_OK;
}

extern "C" tessgpu_status tessgpu_conv3d_check(void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    int h = 0;
    const int zero = 0;
    if (cudaMemcpyFromSymbolAsync(&h, g_conv_err, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TESSGPU_ERR_CUDA;
    if (!h) return TESSGPU_OK;
    if (cudaMemcpyToSymbolAsync(g_conv_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TESSGPU_ERR_CUDA;
    return TESSGPU_ERR_TIMEOUT;
}

extern "C" tessgpu_status tessgpu_conv3d_fwd(const void* x, int X, int Y, int Z, int cin, int cout, const void* w,
                                             const float* bias, int relu, void* y_bf16, float* y_f32, void* stream)
{
    if (!x || !w || X <= 0 || Y <= 0 || Z <= 0 || X % 16 || cin <= 0 || cin % 16 || cout <= 0 || cout % 8 ||
        cout > MAX_COUT || (!y_bf16 && !y_f32))
        return TESSGPU_ERR_INVALID;
    const long long tiles = (long long)X / 16 * Y * Z;
    const int nb = (int)((tiles * 32 + 127) / 128);
    cudaStream_t s = (cudaStream_t)stream;
    const __nv_bfloat16* xx = (const __nv_bfloat16*)x;
    const __nv_bfloat16* ww = (const __nv_bfloat16*)w;
    __nv_bfloat16* yb = (__nv_bfloat16*)y_bf16;
    if (g_conv_engine == 0)
    {
        // TESSGPU_ERR_UNSUPPORTED (more than 2^31 tiles, no tensor-map encoder): the mma.sync kernel below
        tessgpu_status st = TESSGPU_ERR_UNSUPPORTED;
        if (cin == 16 && cout == 16) st = launch_fwd_tc<16, 16>(xx, X, Y, Z, ww, bias, relu, yb, y_f32, s);
        if (cin == 16 && cout == 32) st = launch_fwd_tc<32, 16>(xx, X, Y, Z, ww, bias, relu, yb, y_f32, s);
        if (cin == 32 && cout == 16) st = launch_fwd_tc<16, 32>(xx, X, Y, Z, ww, bias, relu, yb, y_f32, s);
        if (cin == 32 && cout == 32) st = launch_fwd_tc<32, 32>(xx, X, Y, Z, ww, bias, relu, yb, y_f32, s);
        if (st != TESSGPU_ERR_UNSUPPORTED) return st;
    }
    switch (cout / 8)
    {
    case 1: k_conv3d_fwd<1><<<nb, 128, 0, s>>>(xx, X, Y, Z, cin, ww, bias, relu, yb, y_f32); break;
    case 2: k_conv3d_fwd<2><<<nb, 128, 0, s>>>(xx, X, Y, Z, cin, ww, bias, relu, yb, y_f32); break;
    case 4: k_conv3d_fwd<4><<<nb, 128, 0, s>>>(xx, X, Y, Z, cin, ww, bias, relu, yb, y_f32); break;
    case 8: k_conv3d_fwd<8><<<nb, 128, 0, s>>>(xx, X, Y, Z, cin, ww, bias, relu, yb, y_f32); break;
    default: return TESSGPU_ERR_UNSUPPORTED;
    }
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_conv3d_wgrad(const void* x, const void* dy, int X, int Y, int Z, int cin, int cout,
                                               float* dw, float* db, void* stream)
{
    if (!x || !dy || !dw || X <= 0 || Y <= 0 || Z <= 0 || cin <= 0 || cout <= 0 || cin * cout > 64 * 64)
        return TESSGPU_ERR_INVALID;
    const long long V = (long long)X * Y * Z;
    cudaStream_t s = (cudaStream_t)stream;
    if (g_conv_engine == 0)
    {
        // tcgen05 for 16 or 32 channels in and out (TESSGPU_ERR_UNSUPPORTED: the FP32 kernel below)
        const __nv_bfloat16* xx = (const __nv_bfloat16*)x;
        const __nv_bfloat16* dd = (const __nv_bfloat16*)dy;
        tessgpu_status st = TESSGPU_ERR_UNSUPPORTED;
        if (cin == 16 && cout == 16) st = launch_wgrad_tc<16, 16>(xx, dd, X, Y, Z, dw, s);
        if (cin == 16 && cout == 32) st = launch_wgrad_tc<32, 16>(xx, dd, X, Y, Z, dw, s);
        if (cin == 32 && cout == 16) st = launch_wgrad_tc<16, 32>(xx, dd, X, Y, Z, dw, s);
        if (cin == 32 && cout == 32) st = launch_wgrad_tc<32, 32>(xx, dd, X, Y, Z, dw, s);
        if (st == TESSGPU_OK && db)
        {
            long long nb = (V + 255) / 256;
            if (nb > 256) nb = 256;
            k_bias_grad<<<dim3((unsigned)nb, (unsigned)(cout / 8)), 256, 0, s>>>(dd, V, cout, db);
            st = cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
        }
        if (st != TESSGPU_ERR_UNSUPPORTED) return st;
    }
    dim3 grid((unsigned)((V + VB - 1) / VB), 27);
    const size_t smem = sizeof(float) * VB * (cin + cout);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_conv3d_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_conv3d_wgrad<<<grid, 256, smem, s>>>((const __nv_bfloat16*)x, (const __nv_bfloat16*)dy, X, Y, Z, cin, cout, dw,
                                           db);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_conv3d_prepare_weights(const float* w, int cout, int cin, void* w_bf16,
                                                         void* wt_bf16, void* stream)
{
    if (!w || !w_bf16 || !wt_bf16 || cout <= 0 || cin <= 0) return TESSGPU_ERR_INVALID;
    const int n = 27 * cout * cin;
    k_flip_weights<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, cout, cin, (__nv_bfloat16*)w_bf16,
                                                                         (__nv_bfloat16*)wt_bf16);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_relu_grad(const float* g, const void* y, long long n, void* out, void* stream)
{
    if (!g || !y || !out || n < 0) return TESSGPU_ERR_INVALID;
    if (n)
        k_relu_grad<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(g, (const __nv_bfloat16*)y, n,
                                                                           (__nv_bfloat16*)out);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_adam(float* w, const float* g, float* m, float* v, int n, float lr, float b1, float b2,
                                       float eps, int step, void* stream)
{
    if (!w || !g || !m || !v || n < 0 || step < 1) return TESSGPU_ERR_INVALID;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    if (n)
        k_adam<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}
