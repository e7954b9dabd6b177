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
// That array, noalloc_star_sums, holds TESSGPU_NOALLOC_MAX_PARTICLES star
// sums of two 64-bit words each (32 MiB); every GPU that loads the library
// keeps it until the process exits.  All calls share it and it keeps the last call's contents, so each
// call clears the part it uses first; two calls that overlap on the GPU (on
// different streams or host threads) race on it and must be serialised by
// the caller.
//
// Host code cannot pass the array's symbol to a kernel: in host code the name
// is a host-side stand-in, not a device address.  Every call therefore looks
// up the array's address on the current device with cudaGetSymbolAddress
// (nothing is cached, so a device reset or a different current context never
// leaves a stale address behind).  A call synchronises its stream and reads a
// status word back, so it cannot be recorded into a CUDA graph.
//
// The arithmetic is the DTFE path's (dtfe_common.cuh, shared with dtfe.cu):
// 6V per tet in FP32 (FP64 when the FP32 error bound exceeds tau |6V|, or in
// FP64 mode), summed exactly as fixed-point integers (one 64-bit word in
// mixed mode, two in FP64 mode), rho = 24 m / sum.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include "../../include/tess2_gb300.h"
#include "dtfe_common.cuh"

static __device__ __align__(256) tg::StarSum noalloc_star_sums[TESSGPU_NOALLOC_MAX_PARTICLES];
static __device__ __align__(256) int noalloc_flags[8];

namespace {

using tg::StarSum;
using tg::tet_abs_vol6;

// one thread per tet, reading tess2's tet_t records and x,y,z particles directly
__global__ void k_noalloc_star(const float* xyz, int np, const int* tets, int nt, int mode, double scale,
                               StarSum* sums, int* flags)
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
        float3 a[4];
        for (int k = 0; k < 4; ++k)
        {
            const float* q = xyz + 3 * (size_t)v[k];
            a[k] = make_float3(q[0], q[1], q[2]);
        }
        const double vol = tet_abs_vol6(mode == TESSGPU_MODE_FP64, a[0], a[1], a[2], a[3], nullptr);
        const bool two = mode == TESSGPU_MODE_FP64;
        unsigned long long qh, ql;
        tg::star_term(vol, scale, two, qh, ql);
        for (int k = 0; k < 4; ++k)
        {
            if (two)
                atomicAdd(&sums[v[k]].hi, qh);
            atomicAdd(&sums[v[k]].lo, ql);
        }
    }
}

__global__ void k_noalloc_rho(const StarSum* sums, int np, float mass, double inv_scale, float* rho, int* flags)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < np; v += gridDim.x * blockDim.x)
    {
        const StarSum w = sums[v];
        if (tg::star_overflow(w.hi, w.lo))
            atomicExch(&flags[1], 1);
        const double s = tg::star_value(w.hi, w.lo, inv_scale);
        rho[v] = s > 0.0 ? (float)(24.0 * (double)mass / s) : 0.0f;
    }
}

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
    // the scratch arrays' device addresses on the current device
    void* sums_addr = nullptr;
    void* flags_addr = nullptr;
    if (cudaGetSymbolAddress(&sums_addr, noalloc_star_sums) != cudaSuccess ||
        cudaGetSymbolAddress(&flags_addr, noalloc_flags) != cudaSuccess)
    {
        cudaGetLastError();
        return TESSGPU_ERR_CUDA;
    }
    StarSum* sums = (StarSum*)sums_addr;
    int* flags = (int*)flags_addr;
    const double scale = tg::star_sum_scale(bounds6, bounds6 + 3, mode == TESSGPU_MODE_FP64);

    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(sums, 0, sizeof(StarSum) * (size_t)num_particles, s) != cudaSuccess ||
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
