// DTFE vertex densities without any device allocation.
//
// Some callers cannot allocate GPU memory when they need the densities: an
// analysis step running in situ inside a simulation whose own allocator has
// reserved the device memory up front, or code that must not call cudaMalloc
// / cudaFree because those can synchronise the whole device and stall the
// simulation's streams.  This entry point serves them: the caller passes its
// inputs and the output already in device memory, and the only scratch (the
// per-vertex star-volume sums) lives in a fixed array compiled into the
// library.
//
// That array, noalloc_star_sums, holds TESSGPU_NOALLOC_MAX_PARTICLES 64-bit
// sums (16 MiB); every GPU that loads the library keeps it until the process
// exits.  All calls share it and it keeps the last call's contents, so each
// call clears the part it uses first; two calls that overlap on the GPU (on
// different streams or host threads) race on it and must be serialised by
// the caller.
//
// The first call on a device looks up the array's device address there
// (cudaGetSymbolAddress, with that device current); make that first call
// before any stream capture.
//
// The arithmetic is that of the DTFE path in dtfe.cu: 6V per tet in FP32
// (FP64 when the FP32 error bound exceeds tau |6V|, or in FP64 mode), summed
// exactly as fixed-point integers, rho = 24 m / sum.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include "../../include/tess2_gb300.h"

static __device__ __align__(256) unsigned long long noalloc_star_sums[TESSGPU_NOALLOC_MAX_PARTICLES];
static __device__ __align__(256) int noalloc_flags[8];

namespace {

constexpr float kEps32 = 5.9604645e-08f;   // 2^-24
constexpr float kTau = 4.0e-5f;            // the DTFE path's FP64 fix-up threshold
constexpr int kMaxDevices = 64;

__device__ __forceinline__ double vol6_f64(const float* a, const float* b, const float* c, const float* d)
{
    const double e[3][3] = { { (double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2] },
                             { (double)c[0] - a[0], (double)c[1] - a[1], (double)c[2] - a[2] },
                             { (double)d[0] - a[0], (double)d[1] - a[1], (double)d[2] - a[2] } };
    return e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) + e[0][1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
}

__device__ __forceinline__ float vol6_f32(const float* a, const float* b, const float* c, const float* d, float& bound)
{
    const float e1x = b[0] - a[0], e1y = b[1] - a[1], e1z = b[2] - a[2];
    const float e2x = c[0] - a[0], e2y = c[1] - a[1], e2z = c[2] - a[2];
    const float e3x = d[0] - a[0], e3y = d[1] - a[1], e3z = d[2] - a[2];
    const float m1a = e2y * e3z, m1b = e2z * e3y;
    const float m2a = e2z * e3x, m2b = e2x * e3z;
    const float m3a = e2x * e3y, m3b = e2y * e3x;
    const float det = e1x * (m1a - m1b) + e1y * (m2a - m2b) + e1z * (m3a - m3b);
    const float perm = fabsf(e1x) * (fabsf(m1a) + fabsf(m1b)) + fabsf(e1y) * (fabsf(m2a) + fabsf(m2b)) +
                       fabsf(e1z) * (fabsf(m3a) + fabsf(m3b));
    bound = 10.0f * kEps32 * perm;
    return det;
}

// one thread per tet, reading tess2's tet_t records and x,y,z particles directly
__global__ void k_noalloc_star(const float* xyz, int np, const int* tets, int nt, int mode, double scale,
                               unsigned long long* sums, int* flags)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
    {
        const int* r = tets + 8 * (size_t)t;
        const int v[4] = { r[0], r[1], r[2], r[3] };
        if (v[0] < 0 || v[0] >= np || v[1] < 0 || v[1] >= np || v[2] < 0 || v[2] >= np || v[3] < 0 || v[3] >= np)
        {
            atomicExch(&flags[0], 1);
            continue;
        }
        const float* p0 = xyz + 3 * (size_t)v[0];
        const float* p1 = xyz + 3 * (size_t)v[1];
        const float* p2 = xyz + 3 * (size_t)v[2];
        const float* p3 = xyz + 3 * (size_t)v[3];
        double vol;
        if (mode == TESSGPU_MODE_FP64)
            vol = fabs(vol6_f64(p0, p1, p2, p3));
        else
        {
            float bound;
            const float d = vol6_f32(p0, p1, p2, p3, bound);
            vol = bound > kTau * fabsf(d) ? fabs(vol6_f64(p0, p1, p2, p3)) : (double)fabsf(d);
        }
        const unsigned long long q = (unsigned long long)__double2ll_rn(vol * scale);
        for (int k = 0; k < 4; ++k)
            atomicAdd(&sums[v[k]], q);
    }
}

__global__ void k_noalloc_rho(const unsigned long long* sums, int np, float mass, double inv_scale, float* rho,
                              int* flags)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < np; v += gridDim.x * blockDim.x)
    {
        const long long w = (long long)sums[v];
        if (w < 0)
            atomicExch(&flags[1], 1);
        const double s = (double)w * inv_scale;
        rho[v] = s > 0.0 ? (float)(24.0 * (double)mass / s) : 0.0f;
    }
}

std::mutex g_setup_mutex;
unsigned long long* g_sums_addr[kMaxDevices];
int* g_flags_addr[kMaxDevices];

}  // namespace

extern "C" tessgpu_status tessgpu_dtfe_densities_noalloc(const float* d_particles, int num_particles,
                                                         const int* d_tets, int num_tets, const float* bounds6,
                                                         float mass, int mode, float* d_rho, void* stream)
{
    if (num_particles < 0 || num_tets < 0 || !bounds6 || (mode != TESSGPU_MODE_MIXED && mode != TESSGPU_MODE_FP64) ||
        (num_particles && (!d_particles || !d_rho)) || (num_tets && !d_tets))
        return TESSGPU_ERR_INVALID;
    if (num_particles > TESSGPU_NOALLOC_MAX_PARTICLES)
    {
        fprintf(stderr, "tessgpu_dtfe_densities_noalloc: %d particles exceed the fixed scratch of %d\n",
                num_particles, TESSGPU_NOALLOC_MAX_PARTICLES);
        return TESSGPU_ERR_INVALID;
    }
    if (num_particles == 0)
        return TESSGPU_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return TESSGPU_ERR_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices)
        return TESSGPU_ERR_UNSUPPORTED;
    unsigned long long* sums;
    int* flags;
    {
        // the symbol's device address on this device (host code cannot use
        // the symbol itself: it names a host-side stand-in)
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_sums_addr[dev])
        {
            void* a = nullptr;
            void* f = nullptr;
            if (cudaGetSymbolAddress(&a, noalloc_star_sums) != cudaSuccess ||
                cudaGetSymbolAddress(&f, noalloc_flags) != cudaSuccess)
            {
                cudaGetLastError();
                return TESSGPU_ERR_CUDA;
            }
            g_sums_addr[dev] = (unsigned long long*)a;
            g_flags_addr[dev] = (int*)f;
        }
        sums = g_sums_addr[dev];
        flags = g_flags_addr[dev];
    }
    // fixed-point scale: any 6V star sum stays below 2^62 (as in the batch path)
    double vbox = 48.0;
    for (int i = 0; i < 3; ++i)
        vbox *= fmax((double)bounds6[3 + i] - (double)bounds6[i], 1e-30);
    const int bits = 61 - (int)std::ceil(std::log2(vbox));
    const double scale = std::ldexp(1.0, bits);

    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(sums, 0, sizeof(unsigned long long) * (size_t)num_particles, s) != cudaSuccess ||
        cudaMemsetAsync(flags, 0, sizeof(int) * 8, s) != cudaSuccess)
        return TESSGPU_ERR_CUDA;
    if (num_tets)
    {
        const int nb = (int)std::min<long long>((num_tets + 255) / 256, 8192);
        k_noalloc_star<<<nb, 256, 0, s>>>(d_particles, num_particles, d_tets, num_tets, mode, scale, sums, flags);
    }
    const int nb2 = (int)std::min<long long>((num_particles + 255) / 256, 8192);
    k_noalloc_rho<<<nb2, 256, 0, s>>>(sums, num_particles, mass, 1.0 / scale, d_rho, flags);
    int h[2] = { 0, 0 };
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return TESSGPU_ERR_CUDA;
    if (h[0])
        return TESSGPU_ERR_BAD_MESH;
    if (h[1])
        return TESSGPU_ERR_UNSUPPORTED;
    return TESSGPU_OK;
}
