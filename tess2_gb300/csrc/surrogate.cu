// The DTFE surrogate's kernels: a 3-D convolutional network that maps a
// cloud-in-cell density grid to the DTFE density grid (log(1 + rho / mean)).
//
// Layout: activations channels-last, bf16, voxel index (z * Y + y) * X + x,
// channel fastest; weights bf16 as [tap][c_out][c_in] (tap = (dz*3 + dy)*3 + dx
// for offsets dz, dy, dx in -1..1), with an FP32 master copy for the update.
// Channel counts are multiples of 16 (inputs) and 8 (outputs); X is a
// multiple of 16.
//
// conv3d forward (and the data gradient, the same product with the weights
// flipped and transposed) is an implicit GEMM on the tensor cores:
// mma.sync m16n8k16 bf16 x bf16 -> f32.  A warp takes 16 consecutive voxels
// of one x row and every output channel; each tap and 16-channel slice of the
// input is one k-step, its A fragment read straight from the input (zero
// outside the grid) and its B fragment from the weights.  The weight gradient
// reduces over voxels on the CUDA cores (FP32), per tap, with the block's
// voxel slice staged in shared memory.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "../../include/tess2_gb300.h"

namespace {

constexpr int MAX_COUT = 64;   // output channels per warp tile (8 n-tiles)

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
            a[0] = oka ? ld_pair(x + va * cin + c + tig * 2) : 0u;
            a[1] = okb ? ld_pair(x + vb * cin + c + tig * 2) : 0u;
            a[2] = oka ? ld_pair(x + va * cin + c + 8 + tig * 2) : 0u;
            a[3] = okb ? ld_pair(x + vb * cin + c + 8 + tig * 2) : 0u;
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
            *reinterpret_cast<__nv_bfloat162*>(y_bf16 + va * cout + co) = __floats2bfloat162_rn(r[0], r[1]);
            *reinterpret_cast<__nv_bfloat162*>(y_bf16 + vb * cout + co) = __floats2bfloat162_rn(r[2], r[3]);
        }
        if (y_f32)
        {
            y_f32[va * cout + co] = r[0]; y_f32[va * cout + co + 1] = r[1];
            y_f32[vb * cout + co] = r[2]; y_f32[vb * cout + co + 1] = r[3];
        }
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
        sdy[i] = v < V ? __bfloat162float(dy[v * cout + i % cout]) : 0.0f;
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
                val = __bfloat162float(x[(((long long)sz * Y + sy) * X + sx_) * cin + i % cin]);
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

}  // namespace

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
    dim3 grid((unsigned)((V + VB - 1) / VB), 27);
    const size_t smem = sizeof(float) * VB * (cin + cout);
    cudaStream_t s = (cudaStream_t)stream;
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
