// The DTFE surrogate's U-Net kernels: 3x3x3 convolutions of any channel count
// (multiples of 16 in, 32 out) on the 5th-generation tensor cores, for the
// forward pass and the data gradient (tcgen05 implicit GEMM, bf16 x bf16 ->
// FP32 in tensor memory), the weight gradient on the tensor cores too, and the
// U-Net's other steps: 2x2x2 average pooling, nearest upsampling into a
// concatenation buffer, their gradients, the 1x1 prediction head with its
// loss, bias gradients.
//
// Layout.  Activations chunk-planar as the rest of the surrogate: channel c of
// voxel v at ((c / 8) * V + v) * 8 + c % 8, voxel v = (z * Y + y) * X + x, bf16.
// A concatenation [a | b] is one buffer whose first planes hold a and the
// next ones b; producers write at a plane offset, so concatenating copies
// nothing.  Weights: an FP32 master [tap][c_out][c_in] (tap = (dz * 3 + dy) * 3
// + dx, offsets -1..1) packed to bf16 [tap][c_in / 8][c_out][8] for the
// forward pass and to [26 - tap][c_out / 8][c_in][8] for the data gradient
// (the same product with the weights flipped and transposed).
//
// Convolution (k_unet_conv): a tile is 128 consecutive voxels (M of one MMA)
// x NT output channels (N).  Per stage the TMA warp copies one K chunk of KC
// input channels for one (dz, dy) row of taps (SLAB: X a multiple of 128, the
// tile inside one x row; one slab of positions x0 - 1 .. x0 + 128 serves
// dx = -1, 0, 1 at start addresses 16 bytes apart) or for one tap (TAP: X of
// 16, 32 or 64, the tile = 128 / X whole x rows; the box starts at x = dx), and
// the matching weights, both by cp.async.bulk.tensor; positions outside the
// grid arrive as zeros.  The MMA warp issues tcgen05.mma per 16 channels into
// one of two tensor-memory accumulators; the four epilogue warps read the
// other (tcgen05.ld, lane = voxel), add the bias, apply ReLU or the ReLU mask
// of the data gradient, and store bf16 rows, consecutive threads on adjacent
// 16-byte chunks.
//
// Weight gradient (k_unet_wgrad): dw[tap][co][ci] = sum_v dy[v][co] x[v+tap][ci]
// with K = voxels: A = the output-gradient tile (M = 128 output channels,
// zero past c_out), B = the input slab (N = NTW input channels), both
// MN-major straight from the planes.  An item is (tap group, c_out tile,
// c_in tile, voxel chunk); its accumulators (3 or 1 taps x NTW columns) stay
// in tensor memory across the chunk's tiles and are added to dw once.
//
// Every wait is bounded (tc_common.cuh); a timed-out wait raises the CTA's
// abort flag, every role leaves its loop, the CTA waits for its copies and
// MMAs, frees its tensor memory and reports through tessgpu_unet_check.
#include <cstdlib>

#include "../../include/tess2_gb300.h"
#include "tc_common.cuh"

namespace {

using namespace tcg;

constexpr int U_THREADS = 192;        // warps 0-3 epilogue, 4 TMA, 5 MMA (+ tensor-memory allocation)
constexpr int U_SMEM = 227 * 1024;    // dynamic shared memory a CTA may opt into
constexpr int U_M = 128;              // voxels per tile
// every launch asks for at least this much shared memory, so that one CTA runs per SM:
// a CTA's tensor-memory allocation (up to all 512 columns) then never waits for another's
constexpr int U_MIN_SMEM = 116 * 1024;

__device__ int g_unet_err;            // raised by a kernel whose bounded wait ran out

__host__ __device__ constexpr int pow2_cols(int c)
{
    return c <= 32 ? 32 : (c <= 64 ? 64 : (c <= 128 ? 128 : (c <= 256 ? 256 : 512)));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tma5(uint32_t dst, uint64_t map, int c0, int c1, int c2, int c3, int c4, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
                 "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tma4(uint32_t dst, uint64_t map, int c0, int c1, int c2, int c3, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
                 "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ void expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t dcol, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dcol),
                 "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void bar_init(uint32_t bar, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

// instruction descriptor: D f32, A and B bf16, M = 128, N = n; mn: both operands MN-major
__host__ __device__ constexpr uint32_t idesc_f16(int n, bool mn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (mn ? (1u << 15) | (1u << 16) : 0u) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(U_M >> 4) << 24);
}

// ---------------------------------------------------------------------------
// convolution (forward and data gradient)
// ---------------------------------------------------------------------------
template <int NT, int KC, bool SLAB, int MT>
struct ConvLayout
{
    static constexpr int TB = SLAB ? 3 : 1;                  // taps per stage
    // one plane of a tile's input: TAP, 128 rows of 16 bytes; SLAB, the 128 rows x0 .. x0 + 127 at
    // byte 128 (a 128-byte-aligned box) with the halo rows x0 - 1 at 112 and x0 + 128 at 2176
    static constexpr int APLANE = SLAB ? 2304 : U_M * 16;
    static constexpr int AROW0 = SLAB ? 112 : 0;             // byte of the A operand's first row
    static constexpr int ABYTES = (KC / 8) * APLANE;         // one tile's input
    static constexpr int ASTRIDE = (ABYTES + 1023) / 1024 * 1024;
    static constexpr int BPLANE = NT * 16;                   // one plane of KC/8 of a tap's weights
    static constexpr int BTAP = (KC / 8) * BPLANE;
    static constexpr int BBYTES = TB * BTAP;
    static constexpr int BOFF = MT * ASTRIDE;
    static constexpr int STAGE = (BOFF + BBYTES + 1023) / 1024 * 1024;
    static constexpr int FIT = (U_SMEM - 1024) / STAGE;
    static constexpr int STAGES = FIT < 8 ? FIT : 8;
    static constexpr int BAR = STAGES * STAGE;
    // full[S], empty[S], accf[2], acce[2], fin, tensor-memory address, abort flag, last[S]
    static constexpr int OFF_FULL = BAR, OFF_EMPTY = BAR + 8 * STAGES, OFF_ACCF = BAR + 16 * STAGES,
                         OFF_ACCE = OFF_ACCF + 16, OFF_FIN = OFF_ACCE + 16, OFF_TMEM = OFF_FIN + 8,
                         OFF_ABORT = OFF_TMEM + 4, OFF_LAST = OFF_ABORT + 4;
    static constexpr int TOTAL = OFF_LAST + 4 * STAGES;
    static constexpr int TCOLS = pow2_cols(2 * MT * NT);     // two sets of MT accumulators of NT columns
    static constexpr int THREADS = 32 * (5 + MT);            // epilogue 0-3, TMA 4, MMA 5 .. 4 + MT
    // bytes the copies deliver per stage (the halo rows are stored by the TMA warp's lanes)
    static constexpr uint32_t TX = (uint32_t)(MT * (KC / 8) * U_M * 16 + BBYTES);
    static_assert(NT % 32 == 0 && NT >= 32 && NT <= 256, "N: a multiple of 32 up to 256");
    static_assert(KC % 16 == 0 && KC <= 64, "K chunk");
    static_assert(!SLAB || MT * (KC / 8) * 2 <= 32, "one halo row per lane");
    static_assert(2 * MT * NT <= 512, "tensor memory");
    static_assert(STAGES >= 2, "shared memory");
    static_assert(TOTAL <= U_SMEM, "shared memory");
};

struct ConvArgs
{
    const __nv_bfloat16* x;         // the input (cin channels), for the slab's halo rows
    int X, Y, Z;                    // grid (X a multiple of 128 for SLAB, X in {16, 32, 64} for TAP)
    int cin, cout;                  // cin a multiple of KC, cout a multiple of NT
    long long V;                    // X * Y * Z, a multiple of 128
    const float* bias;              // [cout] or null
    int relu;
    const __nv_bfloat16* mask;      // chunk-planar, cout channels, or null: out = acc when mask > 0, else 0
    __nv_bfloat16* y;               // chunk-planar output
    int y_plane0;                   // plane of y that output channel 0 goes to
    int* err;
};

template <int NT, int KC, bool SLAB, int MT>
__global__ void __launch_bounds__(ConvLayout<NT, KC, SLAB, MT>::THREADS, 1)
    k_unet_conv(const __grid_constant__ CUtensorMap amap, const __grid_constant__ CUtensorMap bmap, const ConvArgs p)
{
    using L = ConvLayout<NT, KC, SLAB, MT>;
    constexpr int S = L::STAGES;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mgroups = (int)(p.V / (U_M * MT));             // items of MT consecutive tiles
    const int items = mgroups * (p.cout / NT);               // < 2^31 (launcher)
    const int nkc = p.cin / KC;
    const int steps = (SLAB ? 9 : 27) * nkc;                 // stages per item
    const bool split = !SLAB && p.X == 64;                   // tile rows copied as two halves
    const int NI = (int)blockIdx.x < items ? (items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const uint32_t s_base = smem_u32(smem);
    const uint32_t full0 = s_base + L::OFF_FULL, empty0 = s_base + L::OFF_EMPTY;
    const uint32_t accf0 = s_base + L::OFF_ACCF, acce0 = s_base + L::OFF_ACCE, fin = s_base + L::OFF_FIN;
    volatile int* abort = reinterpret_cast<volatile int*>(smem + L::OFF_ABORT);
    int* last = reinterpret_cast<int*>(smem + L::OFF_LAST);   // per slot: the last stage copied into it

    for (int b = tid; b < S; b += L::THREADS) last[b] = -1;
    if (tid == 0)
    {
        for (int b = 0; b < S; ++b)
        {
            bar_init(full0 + 8 * b, SLAB ? 2 : 1);   // expect_tx + the copies' bytes (+ the halo rows)
            bar_init(empty0 + 8 * b, MT);            // one commit per MMA warp that read the slot
        }
        for (int a = 0; a < 2; ++a)
        {
            bar_init(accf0 + 8 * a, MT);     // one commit per MMA warp and item
            bar_init(acce0 + 8 * a, 128);    // the 128 epilogue threads
        }
        bar_init(fin, MT);
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

    if (warp == 4)
    {
        // ---- TMA: per stage the MT tiles' input boxes and the weights of their taps ----
        const bool leader = elect_one();
        const uint64_t am = reinterpret_cast<uint64_t>(&amap), bm = reinterpret_cast<uint64_t>(&bmap);
        if (leader)
        {
            asm volatile("prefetch.tensormap [%0];" ::"l"(am) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"(bm) : "memory");
        }
        // SLAB: lane l < 2 MT KC/8 keeps one halo row (tile t, plane q, side) in a register, loaded a
        // stage ahead so that its latency overlaps the wait for the next ring slot
        const int nh = MT * (KC / 8) * 2;
        const int ht = lane / (2 * (KC / 8)), hq = (lane >> 1) % (KC / 8), hside = lane & 1;
        auto halo_load = [&](int mg, int j) {
            uint4 h = make_uint4(0, 0, 0, 0);
            if (lane < nh)
            {
                const int g = j / nkc, kc = j - g * nkc;
                const long long v0 = ((long long)mg * MT + ht) * U_M;
                const int x0 = (int)(v0 % p.X);
                const long long r = v0 / p.X;
                const int y = (int)(r % p.Y) + g % 3 - 1, z = (int)(r / p.Y) + g / 3 - 1;
                const int x = hside ? x0 + U_M : x0 - 1;
                if (x >= 0 && x < p.X && y >= 0 && y < p.Y && z >= 0 && z < p.Z)
                    h = __ldg(reinterpret_cast<const uint4*>(p.x) + (long long)(kc * (KC / 8) + hq) * p.V +
                              ((long long)z * p.Y + y) * p.X + x);
            }
            return h;
        };
        bool stop = false;
        int step = 0;
        for (int k = 0; k < NI && !stop; ++k)
        {
            const int item = (int)blockIdx.x + k * (int)gridDim.x;
            const int n = item / mgroups, mg = item - n * mgroups;
            uint4 hrow = make_uint4(0, 0, 0, 0);
            if (SLAB) hrow = halo_load(mg, 0);
            for (int j = 0; j < steps; ++j, ++step)
            {
                const int b = step % S;
                if (step >= S && !warp_wait(empty0 + 8 * b, (uint32_t)((step / S - 1) & 1), abort))
                {
                    stop = true;
                    break;
                }
                const int g = j / nkc, kc = j - g * nkc;
                const int dz = SLAB ? g / 3 - 1 : g / 9 - 1;
                const int dy = SLAB ? g % 3 - 1 : (g / 3) % 3 - 1;
                const int dx = SLAB ? 0 : g % 3 - 1;
                const int tap0 = SLAB ? 3 * g : g;
                const uint32_t dst = s_base + b * L::STAGE;
                if (leader)
                {
                    last[b] = step;
                    expect_tx(full0 + 8 * b, L::TX);
#pragma unroll
                    for (int t = 0; t < MT; ++t)
                    {
                        const long long v0 = ((long long)mg * MT + t) * U_M;
                        const int x0 = (int)(v0 % p.X);
                        const long long r = v0 / p.X;
                        const int y0 = (int)(r % p.Y), z = (int)(r / p.Y);
                        const uint32_t ta = dst + t * L::ASTRIDE;
                        if (SLAB)
                        {
                            // per plane one box of 4 rows of 32 voxels (512 bytes each)
#pragma unroll
                            for (int q = 0; q < KC / 8; ++q)
                                tma5(ta + q * L::APLANE + 128, am, 0, x0 >> 5, y0 + dy, z + dz, kc * (KC / 8) + q,
                                     full0 + 8 * b);
                        }
                        else if (split)
                        {
                            // X = 64: each plane as two boxes of 32 voxels a row (M order: half, row, x)
                            for (int q = 0; q < KC / 8; ++q)
                                for (int h = 0; h < 2; ++h)
                                    tma4(ta + q * L::APLANE + h * 1024, am, 8 * dx + 256 * h, y0 + dy, z + dz,
                                         kc * (KC / 8) + q, full0 + 8 * b);
                        }
                        else
                            // X of 16 or 32: rows of X voxels x 8 channels; the box starts at x = dx and the
                            // x halo comes back as zeros
                            tma4(ta, am, 8 * dx, y0 + dy, z + dz, kc * (KC / 8), full0 + 8 * b);
                    }
                    tma4(dst + L::BOFF, bm, 0, n * (NT / 32), kc * (KC / 8), tap0, full0 + 8 * b);
                }
                if (SLAB)
                {
                    // the halo rows x0 - 1 and x0 + 128 of every tile and plane (zero outside the
                    // grid), made visible to the tensor cores; then the next stage's rows are loaded
                    if (lane < nh)
                        *reinterpret_cast<uint4*>(smem + (dst - s_base) + ht * L::ASTRIDE + hq * L::APLANE +
                                                  (hside ? 128 + U_M * 16 : 112)) = hrow;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(full0 + 8 * b);
                    if (j + 1 < steps) hrow = halo_load(mg, j + 1);
                }
                __syncwarp();
            }
        }
    }
    else if (warp >= 5)
    {
        // ---- MMA (warp 5 + t: tile t of each item): the whole warp runs the loop (warp-uniform
        // descriptors), one lane issues ----
        constexpr uint32_t idesc = idesc_f16(NT, false);
        const int t = warp - 5;
        const bool leader = elect_one();
        bool go = true;
        int step = 0;
        for (int k = 0; k < NI && go; ++k)
        {
            const int a = k & 1;
            // the epilogue has read this accumulator set's item k - 2
            if (k >= 2 && !warp_wait(acce0 + 8 * a, (uint32_t)(((k - 2) >> 1) & 1), abort)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t dcol = tbase + (uint32_t)((a * MT + t) * NT);
            for (int j = 0; j < steps; ++j, ++step)
            {
                const int b = step % S;
                go = warp_wait(full0 + 8 * b, (uint32_t)((step / S) & 1), abort);
                if (!go) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t abase = s_base + b * L::STAGE;
                const uint64_t ad = umma_sdesc(abase + t * L::ASTRIDE + L::AROW0, L::APLANE, 128);
                const uint64_t bd = umma_sdesc(abase + L::BOFF, L::BPLANE, 128);
#pragma unroll
                for (int sh = 0; sh < L::TB; ++sh)
#pragma unroll
                    for (int ks = 0; ks < KC / 16; ++ks)
                    {
                        const uint64_t da = ad + (uint64_t)((sh * 16 + ks * 2 * L::APLANE) >> 4);
                        const uint64_t db = bd + (uint64_t)((sh * L::BTAP + ks * 2 * L::BPLANE) >> 4);
                        if (leader) mma_f16(dcol, da, db, idesc, (j > 0 || sh > 0 || ks > 0) ? 1u : 0u);
                    }
                if (leader) commit(empty0 + 8 * b);
                __syncwarp();
            }
            if (!go) break;
            if (leader) commit(accf0 + 8 * a);
            __syncwarp();
        }
        // every MMA this warp issued has completed once fin's first phase does
        if (leader) commit(fin);
        __syncwarp();
        if (!mbar_wait_bounded(fin, 0u)) *abort = 1;
        __syncwarp();
    }
    else
    {
        // ---- epilogue (warps 0-3: tensor-memory lanes 32 warp .. 32 warp + 31 = voxels) ----
        for (int k = 0; k < NI; ++k)
        {
            const int item = (int)blockIdx.x + k * (int)gridDim.x;
            const int n = item / mgroups, mg = item - n * mgroups;
            const int a = k & 1;
            bool ready = false;
            if (lane == 0) ready = mbar_wait_or_abort(accf0 + 8 * a, (uint32_t)((k >> 1) & 1), abort);
            if (!__shfl_sync(0xffffffffu, ready ? 1 : 0, 0)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
            for (int t = 0; t < MT; ++t)
            {
                // tensor-memory lane tid = the tile's row tid: voxel tid, or for X = 64 (half, row, x)
                const int vt = split ? ((tid >> 5) & 1) * 64 + (tid >> 6) * 32 + (tid & 31) : tid;
                const long long v = ((long long)mg * MT + t) * U_M + vt;
                const uint32_t taddr = tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)((a * MT + t) * NT);
#pragma unroll 1
                for (int c0 = 0; c0 < NT; c0 += 32)
                {
                    uint32_t acc[32];
                    tmem_ld16(taddr + c0, acc);
                    tmem_ld16(taddr + c0 + 16, acc + 16);
                    asm volatile("tcgen05.wait::ld.sync.aligned;");
                    if (t == MT - 1 && c0 + 32 >= NT)
                    {
                        // this thread has read all of the set: hand it back to the MMA warps
                        asm volatile("tcgen05.fence::before_thread_sync;");
                        mbar_arrive(acce0 + 8 * a);
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                    {
                        const int ch = n * NT + c0 + 8 * q;   // first of the plane's 8 channels
                        float f[8];
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                        {
                            f[e] = __uint_as_float(acc[8 * q + e]) + (p.bias ? __ldg(p.bias + ch + e) : 0.0f);
                            if (p.relu) f[e] = fmaxf(f[e], 0.0f);
                        }
                        if (p.mask)
                        {
                            const uint4 mk =
                                __ldg(reinterpret_cast<const uint4*>(p.mask + ((long long)(ch >> 3) * p.V + v) * 8));
                            const __nv_bfloat16* mb = reinterpret_cast<const __nv_bfloat16*>(&mk);
#pragma unroll
                            for (int e = 0; e < 8; ++e)
                                if (!(__bfloat162float(mb[e]) > 0.0f)) f[e] = 0.0f;
                        }
                        *reinterpret_cast<uint4*>(p.y + ((long long)(p.y_plane0 + (ch >> 3)) * p.V + v) * 8) =
                            make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]),
                                       pack_bf16(f[6], f[7]));
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    // no copy may still be landing in shared memory when the CTA exits
    for (int b = tid; b < S; b += L::THREADS)
    {
        const int s = last[b];
        if (s >= 0) mbar_wait_bounded(full0 + 8 * b, (uint32_t)((s / S) & 1));
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicExch(p.err, 1);
    if (warp == 5)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(L::TCOLS));
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
// SLAB with RPT = 1: the tile is 128 voxels of one x row (X a multiple of 128); RPT = 2: two whole
// rows of X = 64.  The input slab keeps each row with a halo row before and after it; a 16-voxel
// K chunk never straddles two rows, so each MMA starts at its own row.
template <int NTW, bool SLAB, int RPT = 1>
struct WgradLayout
{
    static constexpr int TG = SLAB ? 3 : 1;                  // taps per item
    static constexpr int APLANE = U_M * 16;                  // one plane of the output-gradient tile
    static constexpr int ABYTES = 16 * APLANE;               // 16 planes: M = 128 output channels
    static constexpr int RBYTES = U_M / RPT * 16;            // one row of the tile, 16 bytes a voxel
    // row i of an input plane at byte ROWM0 + i ROWSTEP (128-byte aligned), its halo rows 16 bytes
    // before it and RBYTES after its start
    static constexpr int ROWSTEP = (RBYTES + 32 + 127) / 128 * 128;
    static constexpr int ROWM0 = 128;
    static constexpr int XPLANE =
        SLAB ? (ROWM0 + (RPT - 1) * ROWSTEP + RBYTES + 16 + 127) / 128 * 128 : U_M * 16;
    static constexpr int BBYTES = (NTW / 8) * XPLANE;
    static constexpr int BOFF = ABYTES;
    static constexpr int STAGE = (BOFF + BBYTES + 1023) / 1024 * 1024;
    static constexpr int FIT = (U_SMEM - 1024) / STAGE;
    static constexpr int STAGES = FIT < 4 ? FIT : 4;
    static constexpr int BAR = STAGES * STAGE;
    // full[S], empty[S], accf, acce, fin, tensor-memory address, abort flag, last[S]
    static constexpr int OFF_FULL = BAR, OFF_EMPTY = BAR + 8 * STAGES, OFF_ACCF = BAR + 16 * STAGES,
                         OFF_ACCE = OFF_ACCF + 8, OFF_FIN = OFF_ACCE + 8, OFF_TMEM = OFF_FIN + 8,
                         OFF_ABORT = OFF_TMEM + 4, OFF_LAST = OFF_ABORT + 4;
    static constexpr int TOTAL = OFF_LAST + 4 * STAGES;
    static constexpr int TCOLS = pow2_cols(TG * NTW);
    static constexpr uint32_t TX = (uint32_t)(ABYTES + (NTW / 8) * U_M * 16);   // the copies' bytes
    static_assert(NTW % 16 == 0 && NTW >= 16 && NTW <= 256, "N");
    static_assert(RPT == 1 || RPT == 2, "rows per tile");
    static_assert(!SLAB || RPT == 2 || NTW / 8 * 2 <= 32, "one halo row per lane");
    static_assert(TG * NTW <= 512, "tensor memory");
    static_assert(STAGES >= 2, "shared memory");
    static_assert(TOTAL <= U_SMEM, "shared memory");
};

struct WgradArgs
{
    const __nv_bfloat16* x;   // the input, for the slab's halo rows
    int merged;               // not SLAB: 1 = boxes of whole x rows (X <= 32), 0 = 16-byte rows (X = 64)
    int X, Y, Z;
    int cin, cout;
    long long V;
    int nch;        // voxel chunks per (tap group, c_out tile, c_in tile); <= V / 128
    float* dw;      // FP32 [27][cout][cin], accumulated into
    int* err;
};

template <int NTW, bool SLAB, int TS, int RPT>
__global__ void __launch_bounds__(U_THREADS, 1)
    k_unet_wgrad(const __grid_constant__ CUtensorMap dymap, const __grid_constant__ CUtensorMap xmap,
                 const WgradArgs p)
{
    using L = WgradLayout<NTW, SLAB, RPT>;
    constexpr bool HALO = SLAB && RPT == 1;   // halo rows from the grid; RPT = 2: whole rows, halos zero
    constexpr int S = L::STAGES;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mtiles = (int)(p.V / U_M);
    // SLAB: TS (dz, dy) pairs share M (128 / TS output channels each); otherwise one tap per group
    constexpr int CO_S = U_M / TS;           // rows of M per pair
    const int CT = (p.cout + 127) / 128, NTN = p.cin / NTW, NG = SLAB ? (9 + TS - 1) / TS : 27;
    const int items = NG * CT * NTN * p.nch;
    const int NI = (int)blockIdx.x < items ? (items - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const uint32_t s_base = smem_u32(smem);
    const uint32_t full0 = s_base + L::OFF_FULL, empty0 = s_base + L::OFF_EMPTY;
    const uint32_t accf = s_base + L::OFF_ACCF, acce = s_base + L::OFF_ACCE, fin = s_base + L::OFF_FIN;
    volatile int* abort = reinterpret_cast<volatile int*>(smem + L::OFF_ABORT);
    int* last = reinterpret_cast<int*>(smem + L::OFF_LAST);

    for (int b = tid; b < S; b += U_THREADS) last[b] = -1;
    if (tid == 0)
    {
        for (int b = 0; b < S; ++b)
        {
            bar_init(full0 + 8 * b, HALO ? 2 : 1);   // expect_tx + the copies (+ the halo rows)
            bar_init(empty0 + 8 * b, 1);
        }
        bar_init(accf, 1);
        bar_init(acce, 128);
        bar_init(fin, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (SLAB && RPT == 2)
    {
        // whole rows: every halo row lies outside the grid, zero for the whole kernel
        for (int i = tid; i < S * (NTW / 8) * RPT * 2; i += U_THREADS)
        {
            const int side = i & 1, r = (i >> 1) % RPT, q = (i >> 1) / RPT % (NTW / 8), b = (i >> 1) / RPT / (NTW / 8);
            *reinterpret_cast<uint4*>(smem + b * L::STAGE + L::BOFF + q * L::XPLANE + L::ROWM0 + r * L::ROWSTEP +
                                      (side ? L::RBYTES : -16)) = make_uint4(0, 0, 0, 0);
        }
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

    // item -> (tap group grp, c_out tile ct, c_in tile nt, chunk) and the chunk's tiles [m0, m1)
    // the tap group varies fastest: CTAs running at the same time read the same voxel chunk
    // (from L2 after the first), each for its own taps
    auto decode = [&](int item, int& grp, int& ct, int& nt, int& m0, int& m1) {
        grp = item % NG;
        int rest = item / NG;
        ct = rest % CT;
        rest /= CT;
        nt = rest % NTN;
        const int chunk = rest / NTN;
        m0 = (int)((long long)chunk * mtiles / p.nch);
        m1 = (int)((long long)(chunk + 1) * mtiles / p.nch);
    };

    if (warp == 4)
    {
        // ---- TMA: per tile the output-gradient planes of the c_out tile and the input box ----
        const bool leader = elect_one();
        const uint64_t dm = reinterpret_cast<uint64_t>(&dymap), xm = reinterpret_cast<uint64_t>(&xmap);
        if (leader)
        {
            asm volatile("prefetch.tensormap [%0];" ::"l"(dm) : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"(xm) : "memory");
        }
        // SLAB: lane l < 2 NTW/8 keeps one halo row (plane l / 2, side l % 2) of the input slab in a
        // register, loaded a tile ahead so that its latency overlaps the wait for the next slot
        const int nh = HALO ? (NTW / 8) * 2 : 0, hq = lane >> 1, hside = lane & 1;
        auto halo_load = [&](int m, int nt, int dy, int dz) {
            uint4 h = make_uint4(0, 0, 0, 0);
            if (lane < nh)
            {
                const long long v0 = (long long)m * U_M;
                const int x0 = (int)(v0 % p.X);
                const long long r = v0 / p.X;
                const int y = (int)(r % p.Y) + dy, z = (int)(r / p.Y) + dz, x = hside ? x0 + U_M : x0 - 1;
                if (x >= 0 && x < p.X && y >= 0 && y < p.Y && z >= 0 && z < p.Z)
                    h = __ldg(reinterpret_cast<const uint4*>(p.x) + (long long)(nt * (NTW / 8) + hq) * p.V +
                              ((long long)z * p.Y + y) * p.X + x);
            }
            return h;
        };
        bool stop = false;
        int step = 0;
        for (int k = 0; k < NI && !stop; ++k)
        {
            int grp, ct, nt, m0, m1;
            decode((int)blockIdx.x + k * (int)gridDim.x, grp, ct, nt, m0, m1);
            const int dz = grp / 9 - 1, dy = (grp / 3) % 3 - 1, dx = grp % 3 - 1;   // not SLAB: the tap
            uint4 hrow = make_uint4(0, 0, 0, 0);
            if (HALO) hrow = halo_load(m0, nt, 0, 0);
            for (int m = m0; m < m1; ++m, ++step)
            {
                const int b = step % S;
                if (step >= S && !warp_wait(empty0 + 8 * b, (uint32_t)((step / S - 1) & 1), abort))
                {
                    stop = true;
                    break;
                }
                const long long v0 = (long long)m * U_M;
                const int x0 = (int)(v0 % p.X);
                const long long r = v0 / p.X;
                const int y0 = (int)(r % p.Y), z = (int)(r / p.Y);
                const uint32_t dst = s_base + b * L::STAGE;
                if (leader)
                {
                    last[b] = step;
                    expect_tx(full0 + 8 * b, L::TX);
                    if (SLAB)
                    {
                        // with u = v + (dz, dy): dW[dz, dy, dx] = sum_u dy[u - (dz, dy)] x[u + dx].  Per pair
                        // of the group the output gradient shifted by whole rows (16 / TS planes, those past
                        // c_out read as zeros); the input slab of the tile's own row (its dx taps 16 bytes
                        // apart); both as boxes of 4 rows of 32 voxels (512-byte rows)
#pragma unroll
                        for (int jj = 0; jj < TS; ++jj)
                        {
                            const int pr = min(grp * TS + jj, 8);   // pairs past the ninth load the ninth again
                            tma5(dst + jj * (16 / TS) * L::APLANE, dm, 0, x0 >> 5, y0 - (pr % 3 - 1),
                                 z - (pr / 3 - 1), ct * 16, full0 + 8 * b);
                        }
#pragma unroll
                        for (int q = 0; q < NTW / 8; ++q)
#pragma unroll
                            for (int i = 0; i < RPT; ++i)
                                tma5(dst + L::BOFF + q * L::XPLANE + L::ROWM0 + i * L::ROWSTEP, xm, 0, x0 >> 5, y0 + i,
                                     z, nt * (NTW / 8) + q, full0 + 8 * b);
                    }
                    else if (p.merged)
                    {
                        // whole x rows (x and channel merged); the input box starts at x = dx, its x halo
                        // reads as zeros
                        tma4(dst, dm, 0, y0, z, ct * 16, full0 + 8 * b);
                        tma4(dst + L::BOFF, xm, 8 * dx, y0 + dy, z + dz, nt * (NTW / 8), full0 + 8 * b);
                    }
                    else
                    {
                        tma5(dst, dm, 0, x0, y0, z, ct * 16, full0 + 8 * b);
                        tma5(dst + L::BOFF, xm, 0, dx, y0 + dy, z + dz, nt * (NTW / 8), full0 + 8 * b);
                    }
                }
                if (HALO)
                {
                    if (lane < nh)
                        *reinterpret_cast<uint4*>(smem + (dst - s_base) + L::BOFF + hq * L::XPLANE +
                                                  (hside ? 128 + U_M * 16 : 112)) = hrow;
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(full0 + 8 * b);
                    if (m + 1 < m1) hrow = halo_load(m + 1, nt, 0, 0);
                }
                __syncwarp();
            }
        }
    }
    else if (warp == 5)
    {
        // ---- MMA: D[tap][co][ci] += dyT x, 8 MMAs of 16 voxels per tap and tile ----
        constexpr uint32_t idesc = idesc_f16(NTW, true);
        const bool leader = elect_one();
        bool go = true;
        int step = 0;
        for (int k = 0; k < NI && go; ++k)
        {
            int grp, ct, nt, m0, m1;
            decode((int)blockIdx.x + k * (int)gridDim.x, grp, ct, nt, m0, m1);
            // the epilogue has read item k - 1's accumulators
            if (k >= 1 && !warp_wait(acce, (uint32_t)((k - 1) & 1), abort)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            for (int m = m0; m < m1; ++m, ++step)
            {
                const int b = step % S;
                go = warp_wait(full0 + 8 * b, (uint32_t)((step / S) & 1), abort);
                if (!go) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t abase = s_base + b * L::STAGE;
                const uint64_t ad = umma_sdesc(abase, 128, L::APLANE);
                // SLAB: K chunk ks (16 voxels) lies in row ks / (8 / RPT) of the tile; its slab rows start
                // at that row's halo row, plus 16 bytes per dx
                const uint64_t bd = umma_sdesc(abase + L::BOFF + (SLAB ? L::ROWM0 - 16 : 0), 128, L::XPLANE);
#pragma unroll
                for (int sh = 0; sh < L::TG; ++sh)
#pragma unroll
                    for (int ks = 0; ks < U_M / 16; ++ks)
                    {
                        constexpr int KPR = 8 / RPT;   // K chunks per row
                        const int boff = SLAB ? (ks / KPR) * L::ROWSTEP + (ks % KPR) * 256 : ks * 256;
                        const uint64_t da = ad + (uint64_t)((ks * 256) >> 4);
                        const uint64_t db = bd + (uint64_t)((sh * 16 + boff) >> 4);
                        if (leader)
                            mma_f16(tbase + (uint32_t)(sh * NTW), da, db, idesc, (m > m0 || ks > 0) ? 1u : 0u);
                    }
                if (leader) commit(empty0 + 8 * b);
                __syncwarp();
            }
            if (!go) break;
            if (leader) commit(accf);
            __syncwarp();
        }
        if (leader) commit(fin);
        __syncwarp();
        if (!mbar_wait_bounded(fin, 0u)) *abort = 1;
        __syncwarp();
    }
    else
    {
        // ---- epilogue: lane 32 warp + l = output channel of the c_out tile; add to dw ----
        for (int k = 0; k < NI; ++k)
        {
            int grp, ct, nt, m0, m1;
            decode((int)blockIdx.x + k * (int)gridDim.x, grp, ct, nt, m0, m1);
            bool ready = false;
            if (lane == 0) ready = mbar_wait_or_abort(accf, (uint32_t)(k & 1), abort);
            if (!__shfl_sync(0xffffffffu, ready ? 1 : 0, 0)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            // lane tid: SLAB, pair grp * TS + tid / CO_S and output channel ct * 128 + tid % CO_S
            const int pr = SLAB ? grp * TS + tid / CO_S : 0;
            const int co = ct * 128 + tid % CO_S;
#pragma unroll 1
            for (int sh = 0; sh < L::TG; ++sh)
            {
                const int tap = SLAB ? 3 * pr + sh : grp;
#pragma unroll 1
                for (int c0 = 0; c0 < NTW; c0 += 16)
                {
                    uint32_t v[16];
                    tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)(sh * NTW + c0), v);
                    asm volatile("tcgen05.wait::ld.sync.aligned;");
                    if (co < p.cout && (!SLAB || pr < 9))
                    {
                        float* out = p.dw + ((long long)tap * p.cout + co) * p.cin + nt * NTW + c0;
#pragma unroll
                        for (int c = 0; c < 16; ++c) atomicAdd(out + c, __uint_as_float(v[c]));
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(acce);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    for (int b = tid; b < S; b += U_THREADS)
    {
        const int s = last[b];
        if (s >= 0) mbar_wait_bounded(full0 + 8 * b, (uint32_t)((s / S) & 1));
    }
    __syncthreads();
    if (tid == 0 && *abort) atomicExch(p.err, 1);
    if (warp == 5)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(L::TCOLS));
}

// ---------------------------------------------------------------------------
// the other steps (CUDA cores; HBM-bound)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void unpack8(const uint4& u, float* f)
{
    const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
    for (int e = 0; e < 8; ++e) f[e] = __bfloat162float(h[e]);
}

__device__ __forceinline__ uint4 pack8(const float* f)
{
    return make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
}

// the coarse voxel of fine voxel v, and the fine voxels of coarse voxel u
__device__ __forceinline__ long long coarse_of(long long v, int X, int Y)
{
    const int x = (int)(v % X);
    const long long r = v / X;
    const int y = (int)(r % Y), z = (int)(r / Y);
    return ((long long)(z >> 1) * (Y >> 1) + (y >> 1)) * (X >> 1) + (x >> 1);
}

__device__ __forceinline__ long long fine_of(long long u, int X, int Y, int child)
{
    const int hx = X >> 1, hy = Y >> 1;
    const int x = (int)(u % hx);
    const long long r = u / hx;
    const int y = (int)(r % hy), z = (int)(r / hy);
    return ((long long)(2 * z + (child >> 2)) * Y + 2 * y + ((child >> 1) & 1)) * X + 2 * x + (child & 1);
}

// y[u] = mean of x over the 8 fine voxels of u (X, Y, Z: the fine grid)
__global__ void k_pool(const __nv_bfloat16* __restrict__ x, int X, int Y, int Z, int planes,
                       __nv_bfloat16* __restrict__ y)
{
    const long long V = (long long)X * Y * Z, U = V / 8, n = U * planes;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const int pl = (int)(i / U);
        const long long u = i - (long long)pl * U;
        float s[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
#pragma unroll
        for (int c = 0; c < 8; ++c)
        {
            float f[8];
            unpack8(__ldg(reinterpret_cast<const uint4*>(x + ((long long)pl * V + fine_of(u, X, Y, c)) * 8)), f);
#pragma unroll
            for (int e = 0; e < 8; ++e) s[e] += f[e];
        }
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] *= 0.125f;
        reinterpret_cast<uint4*>(y)[(long long)pl * U + u] = pack8(s);
    }
}

// dx[v] = (act[v] > 0) ? skip[v] + dy[coarse(v)] / 8 : 0 (skip: planes skip_plane0.. of a
// concatenation gradient, or null); X, Y, Z: the fine grid
__global__ void k_pool_grad(const __nv_bfloat16* __restrict__ dy, const __nv_bfloat16* __restrict__ skip,
                            int skip_plane0, const __nv_bfloat16* __restrict__ act, int X, int Y, int Z, int planes,
                            __nv_bfloat16* __restrict__ dx)
{
    const long long V = (long long)X * Y * Z, U = V / 8, n = V * planes;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const int pl = (int)(i / V);
        const long long v = i - (long long)pl * V;
        float g[8], a[8];
        unpack8(__ldg(reinterpret_cast<const uint4*>(dy) + (long long)pl * U + coarse_of(v, X, Y)), g);
        unpack8(__ldg(reinterpret_cast<const uint4*>(act) + i), a);
        float s[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
        if (skip) unpack8(__ldg(reinterpret_cast<const uint4*>(skip) + (long long)(skip_plane0 + pl) * V + v), s);
#pragma unroll
        for (int e = 0; e < 8; ++e) s[e] = a[e] > 0.0f ? s[e] + 0.125f * g[e] : 0.0f;
        reinterpret_cast<uint4*>(dx)[i] = pack8(s);
    }
}

// y[planes y_plane0 ..][v] = x[coarse(v)] (X, Y, Z: the fine grid)
__global__ void k_upsample(const __nv_bfloat16* __restrict__ x, int X, int Y, int Z, int planes,
                           __nv_bfloat16* __restrict__ y, int y_plane0)
{
    const long long V = (long long)X * Y * Z, U = V / 8, n = V * planes;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const int pl = (int)(i / V);
        const long long v = i - (long long)pl * V;
        reinterpret_cast<uint4*>(y)[(long long)(y_plane0 + pl) * V + v] =
            __ldg(reinterpret_cast<const uint4*>(x) + (long long)pl * U + coarse_of(v, X, Y));
    }
}

// dx[u] = sum of dy (planes dy_plane0 ..) over the 8 fine voxels of u (X, Y, Z: the fine grid)
__global__ void k_upsample_grad(const __nv_bfloat16* __restrict__ dy, int dy_plane0, int X, int Y, int Z, int planes,
                                __nv_bfloat16* __restrict__ dx)
{
    const long long V = (long long)X * Y * Z, U = V / 8, n = U * planes;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const int pl = (int)(i / U);
        const long long u = i - (long long)pl * U;
        float s[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
#pragma unroll
        for (int c = 0; c < 8; ++c)
        {
            float f[8];
            unpack8(__ldg(reinterpret_cast<const uint4*>(dy) + (long long)(dy_plane0 + pl) * V + fine_of(u, X, Y, c)), f);
#pragma unroll
            for (int e = 0; e < 8; ++e) s[e] += f[e];
        }
        reinterpret_cast<uint4*>(dx)[i] = pack8(s);
    }
}

// the network's input: channel 0 of 16 = field, the rest 0 (plane 1 must be zero already)
__global__ void k_input(const float* __restrict__ field, long long V, __nv_bfloat16* __restrict__ x)
{
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    {
        const float f[8] = { field[v], 0, 0, 0, 0, 0, 0, 0 };
        reinterpret_cast<uint4*>(x)[v] = pack8(f);
    }
}

// Where the particles sit inside the voxels: each particle goes to its nearest
// grid point g (x fastest), u = (p - g) / step in [-1/2, 1/2] per axis, and
// the voxel sums MOMENT_PLANES planes of V floats: [0] the count, [1..3] the
// sums of u_x, u_y, u_z, [4..9] of u_x u_x, u_y u_y, u_z u_z, u_x u_y,
// u_x u_z, u_y u_z.  A cloud-in-cell grid cannot tell where in a voxel its
// particles are; the DTFE field between them depends on it.
constexpr int MOMENT_PLANES = 10;

__global__ void k_cell_moments(const float* __restrict__ xyz, long long n, float3 g0, float3 inv, int X, int Y, int Z,
                               float* __restrict__ m)
{
    const long long V = (long long)X * Y * Z;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const float fx = (xyz[3 * i] - g0.x) * inv.x;
        const float fy = (xyz[3 * i + 1] - g0.y) * inv.y;
        const float fz = (xyz[3 * i + 2] - g0.z) * inv.z;
        const int ix = __float2int_rn(fx), iy = __float2int_rn(fy), iz = __float2int_rn(fz);
        if (ix < 0 || ix >= X || iy < 0 || iy >= Y || iz < 0 || iz >= Z)
            continue;   // nearest grid point outside the grid
        const float ux = fx - ix, uy = fy - iy, uz = fz - iz;
        float* c = m + ((long long)iz * Y + iy) * X + ix;
        atomicAdd(c, 1.0f);
        atomicAdd(c + V, ux);
        atomicAdd(c + 2 * V, uy);
        atomicAdd(c + 3 * V, uz);
        atomicAdd(c + 4 * V, ux * ux);
        atomicAdd(c + 5 * V, uy * uy);
        atomicAdd(c + 6 * V, uz * uz);
        atomicAdd(c + 7 * V, ux * uy);
        atomicAdd(c + 8 * V, ux * uz);
        atomicAdd(c + 9 * V, uy * uz);
    }
}

// The network's 16 input channels from the field and the voxel moments:
// 0 field, 1 log(1 + count), 2-4 twice the mean offset, 5-10 twelve times the
// offsets' central second moments (xx, yy, zz, xy, xz, yz; a uniform spread
// over the voxel gives 1 on the diagonal), 11-15 zero.  Empty voxels give
// zeros, a single particle zero second moments.
__global__ void k_input_moments(const float* __restrict__ field, const float* __restrict__ m, long long V,
                                __nv_bfloat16* __restrict__ x)
{
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    {
        const float n = m[v];
        float f[16] = { field[v], log1pf(n) };
        if (n > 0.0f)
        {
            const float r = 1.0f / n;
            const float mx = m[V + v] * r, my = m[2 * V + v] * r, mz = m[3 * V + v] * r;
            f[2] = 2.0f * mx;
            f[3] = 2.0f * my;
            f[4] = 2.0f * mz;
            if (n > 1.0f)
            {
                f[5] = 12.0f * (m[4 * V + v] * r - mx * mx);
                f[6] = 12.0f * (m[5 * V + v] * r - my * my);
                f[7] = 12.0f * (m[6 * V + v] * r - mz * mz);
                f[8] = 12.0f * (m[7 * V + v] * r - mx * my);
                f[9] = 12.0f * (m[8 * V + v] * r - mx * mz);
                f[10] = 12.0f * (m[9 * V + v] * r - my * mz);
            }
        }
        reinterpret_cast<uint4*>(x)[v] = pack8(f);
        reinterpret_cast<uint4*>(x)[V + v] = pack8(f + 8);
    }
}

// pred[v] = field[v] + b + sum_c w[c] act[c][v]; with a target: loss += sum (pred - target)^2 (block
// partial sums, one atomic per block)
__global__ void __launch_bounds__(256) k_head(const __nv_bfloat16* __restrict__ act, int c, const float* __restrict__ w,
                                              const float* __restrict__ field, long long V, float* __restrict__ pred,
                                              const float* __restrict__ target, double* loss)
{
    __shared__ double part[8];
    double l = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    {
        float s = field[v] + w[c];
        for (int pl = 0; pl < c / 8; ++pl)
        {
            float f[8];
            unpack8(__ldg(reinterpret_cast<const uint4*>(act) + (long long)pl * V + v), f);
#pragma unroll
            for (int e = 0; e < 8; ++e) s = fmaf(w[8 * pl + e], f[e], s);
        }
        pred[v] = s;
        if (target)
        {
            const double d = (double)s - (double)target[v];
            l += d * d;
        }
    }
    if (!target || !loss) return;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += part[i];
        atomicAdd(loss, t);
    }
}

// gradient of scale * sum (pred - target)^2 through the head: g = 2 scale (pred - target);
// dact[c][v] = (act > 0) ? w[c] g : 0; dw[c] += sum_v g act[c][v], dw[c_count] += sum_v g
__global__ void __launch_bounds__(256) k_head_grad(const __nv_bfloat16* __restrict__ act, int c,
                                                   const float* __restrict__ w, const float* __restrict__ pred,
                                                   const float* __restrict__ target, long long V, float scale,
                                                   __nv_bfloat16* __restrict__ dact, float* dw)
{
    __shared__ float part[8][33];
    float acc[33];
    for (int i = 0; i <= 32; ++i) acc[i] = 0.0f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    {
        const float g = 2.0f * scale * (pred[v] - target[v]);
        acc[32] += g;
        for (int pl = 0; pl < c / 8; ++pl)
        {
            float f[8], d[8];
            unpack8(__ldg(reinterpret_cast<const uint4*>(act) + (long long)pl * V + v), f);
#pragma unroll
            for (int e = 0; e < 8; ++e)
            {
                acc[8 * pl + e] += g * f[e];
                d[e] = f[e] > 0.0f ? w[8 * pl + e] * g : 0.0f;
            }
            reinterpret_cast<uint4*>(dact)[(long long)pl * V + v] = pack8(d);
        }
    }
    const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
    for (int i = 0; i <= 32; ++i)
    {
        float s = acc[i];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (ln == 0) part[wid][i] = s;
    }
    __syncthreads();
    if (threadIdx.x <= 32 && (threadIdx.x < c || threadIdx.x == 32))
    {
        float s = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += part[i][threadIdx.x];
        atomicAdd(dw + (threadIdx.x == 32 ? c : threadIdx.x), s);
    }
}

// db[co] += sum_v dy[v][co]: one block per (plane, voxel slice), one atomic per channel and block
__global__ void __launch_bounds__(256) k_unet_bias_grad(const __nv_bfloat16* __restrict__ dy, long long V, float* db)
{
    __shared__ float part[8][8];
    const int pl = blockIdx.y;
    float acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    {
        float f[8];
        unpack8(__ldg(reinterpret_cast<const uint4*>(dy) + (long long)pl * V + v), f);
#pragma unroll
        for (int e = 0; e < 8; ++e) acc[e] += f[e];
    }
    const int wid = threadIdx.x >> 5, ln = threadIdx.x & 31;
#pragma unroll
    for (int e = 0; e < 8; ++e)
    {
        float s = acc[e];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (ln == 0) part[wid][e] = s;
    }
    __syncthreads();
    if (threadIdx.x < 8)
    {
        float s = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += part[i][threadIdx.x];
        atomicAdd(db + 8 * pl + threadIdx.x, s);
    }
}

// FP32 master [tap][co][ci] -> bf16 forward [tap][ci/8][co][8] and data-gradient [26-tap][co/8][ci][8]
__global__ void k_pack_weights(const float* __restrict__ w, int cout, int cin, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wb)
{
    const int n = 27 * cout * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int tap = i / (cout * cin), co = (i / cin) % cout, ci = i % cin;
        const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
        wf[(((long long)tap * (cin / 8) + ci / 8) * cout + co) * 8 + ci % 8] = v;
        wb[(((long long)(26 - tap) * (cout / 8) + co / 8) * cin + ci) * 8 + co % 8] = v;
    }
}

int grid_1d(long long n, int t)
{
    long long b = (n + t - 1) / t;
    return (int)(b < 1 ? 1 : (b > 152LL * 32 ? 152LL * 32 : b));
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int smem_of(int total)
{
    return total > U_MIN_SMEM ? total : U_MIN_SMEM;
}

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// a chunk-planar activation of c channels as (8 channels, X, Y, Z, c / 8), box (8, bx, by, 1, bp)
bool act_map(CUtensorMap* map, const void* base, int X, int Y, int Z, int c, int bx, int by, int bp)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode || ((uintptr_t)base & 15)) return false;
    const cuuint64_t dims[5] = { 8, (cuuint64_t)X, (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(c / 8) };
    const cuuint64_t strides[4] = { 16, (cuuint64_t)X * 16, (cuuint64_t)X * Y * 16, (cuuint64_t)X * Y * Z * 16 };
    const cuuint32_t box[5] = { 8, (cuuint32_t)bx, (cuuint32_t)by, 1, (cuuint32_t)bp };
    const cuuint32_t estride[5] = { 1, 1, 1, 1, 1 };
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// an activation (X a multiple of 32) as (256 = 32 voxels x 8 channels, X / 32, Y, Z, c / 8), box
// (256, min(X, 128) / 32, by, 1, bp): bp planes of by rows of up to 128 voxels, in 512-byte rows
bool row_map(CUtensorMap* map, const void* base, int X, int Y, int Z, int c, int bp = 1, int by = 1)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode || ((uintptr_t)base & 15) || X % 32) return false;
    const cuuint64_t dims[5] = { 256, (cuuint64_t)(X / 32), (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(c / 8) };
    const cuuint64_t strides[4] = { 512, (cuuint64_t)X * 16, (cuuint64_t)X * Y * 16, (cuuint64_t)X * Y * Z * 16 };
    const cuuint32_t box[5] = { 256, (cuuint32_t)(X < 128 ? X / 32 : 4), (cuuint32_t)by, 1, (cuuint32_t)bp };
    const cuuint32_t estride[5] = { 1, 1, 1, 1, 1 };
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// an activation with X of 16, 32 or 64 as (8 X = x and channel merged, Y, Z, c / 8): a box of
// 128 / X rows (X <= 32: all of a row, bp planes; X = 64: half a row, one plane); a box starting at
// x = -1 or ending at x = X reads zeros there (the x halo)
bool merged_map(CUtensorMap* map, const void* base, int X, int Y, int Z, int c, int bp)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode || ((uintptr_t)base & 15) || (X != 16 && X != 32 && X != 64)) return false;
    const cuuint64_t dims[4] = { (cuuint64_t)(8 * X), (cuuint64_t)Y, (cuuint64_t)Z, (cuuint64_t)(c / 8) };
    const cuuint64_t strides[3] = { (cuuint64_t)X * 16, (cuuint64_t)X * Y * 16, (cuuint64_t)X * Y * Z * 16 };
    const cuuint32_t box[4] = { (cuuint32_t)(X == 64 ? 256 : 8 * X), (cuuint32_t)(U_M / X), 1,
                                (cuuint32_t)(X == 64 ? 1 : bp) };
    const cuuint32_t estride[4] = { 1, 1, 1, 1 };
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// packed weights [27][cin/8][cout][8] as (256 = 32 output channels x 8, cout / 32, cin / 8, 27), box
// (256, nt / 32, kc / 8, tb): 512-byte rows, landing as [tap][plane][nt][8] like a box of 16-byte rows
bool weight_map(CUtensorMap* map, const void* base, int cin, int cout, int nt, int kc, int tb)
{
    const EncodeTiled encode = tensor_map_encoder();
    if (!encode || ((uintptr_t)base & 15) || cout % 32 || nt % 32) return false;
    const cuuint64_t dims[4] = { 256, (cuuint64_t)(cout / 32), (cuuint64_t)(cin / 8), 27 };
    const cuuint64_t strides[3] = { 512, (cuuint64_t)cout * 16, (cuuint64_t)(cin / 8) * cout * 16 };
    const cuuint32_t box[4] = { 256, (cuuint32_t)(nt / 32), (cuuint32_t)(kc / 8), (cuuint32_t)tb };
    const cuuint32_t estride[4] = { 1, 1, 1, 1 };
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estride,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int NT, int KC, bool SLAB, int MT>
tessgpu_status launch_conv(const void* x, const void* w, const ConvArgs& a, cudaStream_t s)
{
    using L = ConvLayout<NT, KC, SLAB, MT>;
    static bool ready[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TESSGPU_ERR_CUDA;
    if (!ready[dev])
    {
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (optin < smem_of(L::TOTAL)) return TESSGPU_ERR_UNSUPPORTED;
        if (cudaFuncSetAttribute(k_unet_conv<NT, KC, SLAB, MT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem_of(L::TOTAL)) != cudaSuccess)
            return TESSGPU_ERR_CUDA;
        ready[dev] = true;
    }
    CUtensorMap amap, bmap;
    if (!(SLAB ? row_map(&amap, x, a.X, a.Y, a.Z, a.cin) : merged_map(&amap, x, a.X, a.Y, a.Z, a.cin, KC / 8)) ||
        !weight_map(&bmap, w, a.cin, a.cout, NT, KC, L::TB))
        return TESSGPU_ERR_UNSUPPORTED;
    const long long items = a.V / (U_M * MT) * (a.cout / NT);
    const int sms = sm_count();
    const int grid = (int)(items < sms ? items : sms);
    k_unet_conv<NT, KC, SLAB, MT><<<grid, L::THREADS, smem_of(L::TOTAL), s>>>(amap, bmap, a);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

template <int NTW, bool SLAB, int TS, int RPT>
tessgpu_status launch_wgrad(const void* x, const void* dy, WgradArgs a, cudaStream_t s)
{
    using L = WgradLayout<NTW, SLAB, RPT>;
    static bool ready[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return TESSGPU_ERR_CUDA;
    if (!ready[dev])
    {
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (optin < smem_of(L::TOTAL)) return TESSGPU_ERR_UNSUPPORTED;
        if (cudaFuncSetAttribute(k_unet_wgrad<NTW, SLAB, TS, RPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem_of(L::TOTAL)) != cudaSuccess)
            return TESSGPU_ERR_CUDA;
        ready[dev] = true;
    }
    CUtensorMap dymap, xmap;
    a.merged = !SLAB && a.X <= 32;
    bool ok;
    if (SLAB)
        ok = row_map(&dymap, dy, a.X, a.Y, a.Z, a.cout, 16 / TS, RPT) && row_map(&xmap, x, a.X, a.Y, a.Z, a.cin, 1, 1);
    else if (a.merged)
        ok = merged_map(&dymap, dy, a.X, a.Y, a.Z, a.cout, 16) && merged_map(&xmap, x, a.X, a.Y, a.Z, a.cin, NTW / 8);
    else
        ok = act_map(&dymap, dy, a.X, a.Y, a.Z, a.cout, a.X, U_M / a.X, 16) &&
             act_map(&xmap, x, a.X, a.Y, a.Z, a.cin, a.X, U_M / a.X, NTW / 8);
    if (!ok) return TESSGPU_ERR_UNSUPPORTED;
    const int sms = sm_count();
    const long long mt = a.V / U_M;
    const long long base = (long long)(SLAB ? (9 + TS - 1) / TS : 27) * ((a.cout + 127) / 128) * (a.cin / NTW);
    long long nch = (2LL * sms + base - 1) / base;
    if (nch > mt) nch = mt;
    if (nch < 1) nch = 1;
    a.nch = (int)nch;
    const long long items = base * nch;
    const int grid = (int)(items < sms ? items : sms);
    k_unet_wgrad<NTW, SLAB, TS, RPT><<<grid, U_THREADS, smem_of(L::TOTAL), s>>>(dymap, xmap, a);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

bool unet_grid_ok(int X, int Y, int Z)
{
    if (X <= 0 || Y <= 0 || Z <= 0) return false;
    if (X % 128 == 0) return true;   // slab tiles (one x row)
    return (X == 16 || X == 32 || X == 64) && Y % (U_M / X) == 0;   // tiles of whole x rows
}

int unet_tiles_env()
{
    const char* e = getenv("TESSGPU_UNET_TILES");
    return e ? atoi(e) : 0;
}

int* err_flag()
{
    int* e = nullptr;
    return cudaGetSymbolAddress((void**)&e, g_unet_err) == cudaSuccess ? e : nullptr;
}

}  // namespace

extern "C" tessgpu_status tessgpu_unet_conv(const void* x, int X, int Y, int Z, int cin, const void* w, int cout,
                                            const float* bias, int relu, const void* mask, void* y, int y_plane0,
                                            void* stream)
{
    if (!x || !w || !y || !unet_grid_ok(X, Y, Z) || cin <= 0 || cin % 16 || cout <= 0 || cout % 32 || y_plane0 < 0 ||
        (long long)X * Y * Z / U_M * (cout / 32) >= (1LL << 31))
        return TESSGPU_ERR_INVALID;
    int* err = err_flag();
    if (!err) return TESSGPU_ERR_CUDA;
    ConvArgs a;
    a.x = (const __nv_bfloat16*)x;
    a.X = X; a.Y = Y; a.Z = Z;
    a.cin = cin; a.cout = cout;
    a.V = (long long)X * Y * Z;
    a.bias = bias; a.relu = relu;
    a.mask = (const __nv_bfloat16*)mask;
    a.y = (__nv_bfloat16*)y;
    a.y_plane0 = y_plane0;
    a.err = err;
    cudaStream_t s = (cudaStream_t)stream;
    const bool slab = X % 128 == 0;
    // N tile: all output channels up to 256, else the largest of 256, 192, 128, 96, 64, 32 dividing c_out
    int nt = 32;
    for (int c : { 256, 192, 128, 96, 64 })
        if (cout % c == 0)
        {
            nt = c;
            break;
        }
    const int kc = cin % 64 == 0 && !slab ? 64 : (cin % 32 == 0 ? 32 : 16);
    // tiles per item: four (N = 32) or two (N = 64) MMA-issuing warps on tiles that share the weights'
    // stage, when the tile count divides; TESSGPU_UNET_TILES=1 forces one
    const long long mtiles = a.V / U_M;
    int mt = nt == 32 ? 4 : (nt == 64 ? 2 : 1);
    if (mtiles % mt || unet_tiles_env() == 1) mt = 1;
#define UC(NT_, KC_, SL_, MT_)                                                                                         \
    if (nt == NT_ && kc == KC_ && slab == SL_ && mt == MT_) return launch_conv<NT_, KC_, SL_, MT_>(x, w, a, s);
    UC(32, 16, true, 4) UC(32, 32, true, 4) UC(64, 32, true, 2) UC(96, 32, true, 1) UC(128, 32, true, 1)
    UC(192, 32, true, 1) UC(256, 32, true, 1)
    UC(32, 16, false, 4) UC(32, 32, false, 4) UC(64, 32, false, 2) UC(96, 32, false, 1) UC(128, 32, false, 1)
    UC(192, 32, false, 1) UC(256, 32, false, 1)
    UC(32, 64, false, 4) UC(64, 64, false, 2) UC(96, 64, false, 1) UC(128, 64, false, 1) UC(192, 64, false, 1)
    UC(256, 64, false, 1)
    UC(32, 16, true, 1) UC(32, 32, true, 1) UC(64, 32, true, 1) UC(32, 16, false, 1) UC(32, 32, false, 1)
    UC(64, 32, false, 1) UC(32, 64, false, 1) UC(64, 64, false, 1)
#undef UC
    return TESSGPU_ERR_UNSUPPORTED;
}

extern "C" tessgpu_status tessgpu_unet_wgrad(const void* x, const void* dy, int X, int Y, int Z, int cin, int cout,
                                             float* dw, float* db, void* stream)
{
    if (!x || !dy || !dw || !unet_grid_ok(X, Y, Z) || cin <= 0 || cin % 16 || cout <= 0 || cout % 8)
        return TESSGPU_ERR_INVALID;
    int* err = err_flag();
    if (!err) return TESSGPU_ERR_CUDA;
    WgradArgs a;
    a.X = X; a.Y = Y; a.Z = Z;
    a.cin = cin; a.cout = cout;
    a.V = (long long)X * Y * Z;
    a.nch = 1;
    a.dw = dw;
    a.err = err;
    cudaStream_t s = (cudaStream_t)stream;
    // slab form: X a multiple of 128 (a tile in one x row) or X = 64 (a tile of two whole rows)
    const bool slab = X % 128 == 0 || X == 64;
    const int rpt = X == 64 ? 2 : 1;
    // N tile over the input channels: all of them up to 128 (slab: three taps share tensor memory) or 256
    // slab form: output channels of 16, 32 or 64 leave room in M for 8, 4 or 2 (dz, dy) pairs
    const int ts = slab && (cout == 16 || cout == 32 || cout == 64) ? 128 / cout : 1;
    int ntw = 16;
    const int cap = slab ? 128 : 256;
    for (int c : { 256, 192, 128, 96, 64, 32, 16 })
        if (c <= cap && cin % c == 0)
        {
            ntw = c;
            break;
        }
    tessgpu_status st = TESSGPU_ERR_UNSUPPORTED;
    a.x = (const __nv_bfloat16*)x;
    a.merged = 0;
#define UW(N_, SL_, T_, R_)                                                                                        \
    else if (ntw == N_ && slab == SL_ && ts == T_ && rpt == R_) st = launch_wgrad<N_, SL_, T_, R_>(x, dy, a, s);
    if (false) {}
    UW(16, true, 1, 1) UW(32, true, 1, 1) UW(64, true, 1, 1) UW(96, true, 1, 1) UW(128, true, 1, 1)
    UW(16, true, 2, 1) UW(32, true, 2, 1) UW(64, true, 2, 1) UW(96, true, 2, 1) UW(128, true, 2, 1)
    UW(16, true, 4, 1) UW(32, true, 4, 1) UW(64, true, 4, 1) UW(96, true, 4, 1) UW(128, true, 4, 1)
    UW(16, true, 8, 1) UW(32, true, 8, 1) UW(64, true, 8, 1) UW(96, true, 8, 1) UW(128, true, 8, 1)
    UW(16, true, 1, 2) UW(32, true, 1, 2) UW(64, true, 1, 2) UW(96, true, 1, 2) UW(128, true, 1, 2)
    UW(16, true, 2, 2) UW(32, true, 2, 2) UW(64, true, 2, 2) UW(96, true, 2, 2) UW(128, true, 2, 2)
    UW(16, true, 4, 2) UW(32, true, 4, 2) UW(64, true, 4, 2) UW(96, true, 4, 2) UW(128, true, 4, 2)
    UW(16, true, 8, 2) UW(32, true, 8, 2) UW(64, true, 8, 2) UW(96, true, 8, 2) UW(128, true, 8, 2)
    UW(16, false, 1, 1) UW(32, false, 1, 1) UW(64, false, 1, 1) UW(96, false, 1, 1) UW(128, false, 1, 1)
    UW(192, false, 1, 1) UW(256, false, 1, 1)
#undef UW
    if (st != TESSGPU_OK || !db) return st;
    const long long V = a.V;
    long long nb = (V + 255) / 256;
    if (nb > 128) nb = 128;
    k_unet_bias_grad<<<dim3((unsigned)nb, (unsigned)(cout / 8)), 256, 0, s>>>((const __nv_bfloat16*)dy, V, db);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_pack_weights(const float* w, int cout, int cin, void* w_fwd, void* w_bwd,
                                                    void* stream)
{
    if (!w || !w_fwd || !w_bwd || cout <= 0 || cin <= 0 || cout % 8 || cin % 8) return TESSGPU_ERR_INVALID;
    const int n = 27 * cout * cin;
    k_pack_weights<<<grid_1d(n, 256), 256, 0, (cudaStream_t)stream>>>(w, cout, cin, (__nv_bfloat16*)w_fwd,
                                                                      (__nv_bfloat16*)w_bwd);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_pool(const void* x, int X, int Y, int Z, int c, void* y, void* stream)
{
    if (!x || !y || X <= 0 || Y <= 0 || Z <= 0 || X % 2 || Y % 2 || Z % 2 || c <= 0 || c % 8)
        return TESSGPU_ERR_INVALID;
    const long long n = (long long)X * Y * Z / 8 * (c / 8);
    k_pool<<<grid_1d(n, 256), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)x, X, Y, Z, c / 8,
                                                               (__nv_bfloat16*)y);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_pool_grad(const void* dy, const void* skip, int skip_plane0, const void* act,
                                                 int X, int Y, int Z, int c, void* dx, void* stream)
{
    if (!dy || !act || !dx || X <= 0 || Y <= 0 || Z <= 0 || X % 2 || Y % 2 || Z % 2 || c <= 0 || c % 8 ||
        skip_plane0 < 0)
        return TESSGPU_ERR_INVALID;
    const long long n = (long long)X * Y * Z * (c / 8);
    k_pool_grad<<<grid_1d(n, 256), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16*)dy, (const __nv_bfloat16*)skip, skip_plane0, (const __nv_bfloat16*)act, X, Y, Z, c / 8,
        (__nv_bfloat16*)dx);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_upsample(const void* x, int X, int Y, int Z, int c, void* y, int y_plane0,
                                                void* stream)
{
    if (!x || !y || X <= 0 || Y <= 0 || Z <= 0 || X % 2 || Y % 2 || Z % 2 || c <= 0 || c % 8 || y_plane0 < 0)
        return TESSGPU_ERR_INVALID;
    const long long n = (long long)X * Y * Z * (c / 8);
    k_upsample<<<grid_1d(n, 256), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)x, X, Y, Z, c / 8,
                                                                  (__nv_bfloat16*)y, y_plane0);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_upsample_grad(const void* dy, int dy_plane0, int X, int Y, int Z, int c,
                                                     void* dx, void* stream)
{
    if (!dy || !dx || X <= 0 || Y <= 0 || Z <= 0 || X % 2 || Y % 2 || Z % 2 || c <= 0 || c % 8 || dy_plane0 < 0)
        return TESSGPU_ERR_INVALID;
    const long long n = (long long)X * Y * Z / 8 * (c / 8);
    k_upsample_grad<<<grid_1d(n, 256), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)dy, dy_plane0, X, Y, Z,
                                                                       c / 8, (__nv_bfloat16*)dx);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_input(const float* field, long long V, void* x, void* stream)
{
    if (!field || !x || V <= 0) return TESSGPU_ERR_INVALID;
    k_input<<<grid_1d(V, 256), 256, 0, (cudaStream_t)stream>>>(field, V, (__nv_bfloat16*)x);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_cell_moments(const float* xyz, long long n, const float* grid_min,
                                                    const float* grid_step, int X, int Y, int Z, float* moments,
                                                    void* stream)
{
    if ((n > 0 && !xyz) || n < 0 || !grid_min || !grid_step || !moments || X <= 0 || Y <= 0 || Z <= 0)
        return TESSGPU_ERR_INVALID;
    for (int d = 0; d < 3; ++d)
        if (!(grid_step[d] > 0.0f)) return TESSGPU_ERR_INVALID;
    const long long V = (long long)X * Y * Z;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(moments, 0, sizeof(float) * MOMENT_PLANES * V, s) != cudaSuccess) return TESSGPU_ERR_CUDA;
    if (n > 0)
        k_cell_moments<<<grid_1d(n, 256), 256, 0, s>>>(
            xyz, n, make_float3(grid_min[0], grid_min[1], grid_min[2]),
            make_float3(1.0f / grid_step[0], 1.0f / grid_step[1], 1.0f / grid_step[2]), X, Y, Z, moments);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_input_moments(const float* field, const float* moments, long long V, void* x,
                                                     void* stream)
{
    if (!field || !moments || !x || V <= 0) return TESSGPU_ERR_INVALID;
    k_input_moments<<<grid_1d(V, 256), 256, 0, (cudaStream_t)stream>>>(field, moments, V, (__nv_bfloat16*)x);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_head(const void* act, int c, const float* w, const float* field, long long V,
                                            float* pred, const float* target, double* loss, void* stream)
{
    if (!act || !w || !field || !pred || V <= 0 || c <= 0 || c % 8 || c > 32) return TESSGPU_ERR_INVALID;
    k_head<<<grid_1d(V, 256), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)act, c, w, field, V, pred, target,
                                                              loss);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_head_grad(const void* act, int c, const float* w, const float* pred,
                                                 const float* target, long long V, float scale, void* dact, float* dw,
                                                 void* stream)
{
    if (!act || !w || !pred || !target || !dact || !dw || V <= 0 || c <= 0 || c % 8 || c > 32)
        return TESSGPU_ERR_INVALID;
    k_head_grad<<<grid_1d(V, 256), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)act, c, w, pred, target, V,
                                                                   scale, (__nv_bfloat16*)dact, dw);
    return cudaGetLastError() == cudaSuccess ? TESSGPU_OK : TESSGPU_ERR_CUDA;
}

extern "C" tessgpu_status tessgpu_unet_check(void* stream)
{
    cudaStream_t s = (cudaStream_t)stream;
    int h = 0;
    const int zero = 0;
    if (cudaMemcpyFromSymbolAsync(&h, g_unet_err, sizeof(int), 0, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TESSGPU_ERR_CUDA;
    if (!h) return TESSGPU_OK;
    if (cudaMemcpyToSymbolAsync(g_unet_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TESSGPU_ERR_CUDA;
    return TESSGPU_ERR_TIMEOUT;
}
