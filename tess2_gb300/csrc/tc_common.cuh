// Helpers shared by the tcgen05 kernels (surrogate.cu, unet.cu): shared-memory
// matrix descriptors, bounded mbarrier waits, tensor-memory loads, bf16
// packing, and the tensor-map encoder taken from the driver through the
// runtime (no link against libcuda).
//
// Bounded waits: a pipeline wait gives up after 2 s of %globaltimer time and
// raises the CTA's abort flag, so a stalled role ends every loop instead of
// hanging the GPU; the waits for work already issued (copies landing, MMAs
// completing) before a CTA frees tensor memory and exits allow 30 s.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace tcg {

__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;   // stride between core matrices along K
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;   // stride between 8-row groups
    d |= (uint64_t)1 << 46;                       // descriptor version; base offset 0; no swizzle
    return d;
}

// the thread sleeps in try_wait until the phase completes or about 50 us pass
__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(mbar), "r"(parity), "n"(50000)
                 : "memory");
    return done != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr uint64_t TC_WAIT_NS = 2000000000ull;   // a wait gives up after 2 s of wall time

// bounded wait (2 s of wall time, whatever the kernel's speed); gives up when
// another role raised the abort flag, and raises it when the bound runs out
__device__ __forceinline__ bool mbar_wait_or_abort(uint32_t mbar, uint32_t parity, volatile int* abort)
{
    const uint64_t t0 = global_ns();
    for (int it = 0; it < (1 << 26); ++it)
    {
        if (mbar_try(mbar, parity)) return true;
        if (*abort) return false;
        if (global_ns() - t0 > TC_WAIT_NS) break;
    }
    *abort = 1;
    return false;
}

// The waits for work already issued -- the last copy into each ring slot and
// the commit of every MMA -- before the CTA frees its tensor memory and
// exits.  A copy of a valid box always lands and an issued MMA always
// completes, so these run long only when the kernel itself is slowed (an
// instrumented profiler replay serialises and slows it by orders of
// magnitude); giving up early there is the one way this kernel could free
// tensor memory or exit with asynchronous work still writing to it, so they
// allow 30 s, not the 2 s of the pipeline's waits.
constexpr uint64_t TC_DRAIN_NS = 30000000000ull;

// bounded wait that ignores the abort flag (draining copies and MMAs before exit)
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity)
{
    const uint64_t t0 = global_ns();
    for (int it = 0; it < (1 << 30); ++it)
    {
        if (mbar_try(mbar, parity)) return true;
        if (global_ns() - t0 > TC_DRAIN_NS) break;
    }
    return false;
}

// the same outcome on every lane of the warp
__device__ __forceinline__ bool warp_wait(uint32_t mbar, uint32_t parity, volatile int* abort)
{
    return __all_sync(0xffffffffu, mbar_wait_or_abort(mbar, parity, abort));
}

// true on one lane of the (fully active) warp
__device__ __forceinline__ bool elect_one()
{
    uint32_t e;
    asm volatile("{\n\t.reg .pred P;\n\telect.sync _|P, 0xffffffff;\n\tselp.u32 %0, 1, 0, P;\n\t}" : "=r"(e));
    return e != 0;
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, through the runtime (no link against libcuda)
inline EncodeTiled tensor_map_encoder()
{
    static EncodeTiled fn = nullptr;
    if (!fn)
    {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiled)p;
        cudaGetLastError();
    }
    return fn;
}

}  // namespace tcg
