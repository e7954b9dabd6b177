// Arithmetic shared by every DTFE entry point (the batch and host-buffer
// paths in dtfe.cu / api.cu and the allocation-free densities in noalloc.cu),
// so that all of them round the same way: the FP32 tet volume with its error
// bound, the FP64 volume, the threshold above which mixed mode recomputes a
// tet in FP64, and the fixed-point scale of the star-volume sums.
//
// Translation units that include this are built with -fmad=false: the error
// bound of tet_vol6_f32 assumes that no multiply-add is contracted.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace tg {

constexpr float EPS32 = 5.9604645e-08f;            // 2^-24
constexpr double EPS64 = 1.1102230246251565e-16;   // 2^-53

// mixed mode: a tet whose FP32 error bound exceeds DTFE_TAU * |6V| is
// recomputed in FP64
constexpr float DTFE_TAU = 4.0e-5f;

// 6 * signed volume of tet (a0, a1, a2, a3) in FP64: exact differences of the
// float coordinates, one rounding per product and sum
__host__ __device__ __forceinline__ double tet_vol6_f64(float3 a0, float3 a1, float3 a2, float3 a3)
{
    double e[3][3] = { { (double)a1.x - a0.x, (double)a1.y - a0.y, (double)a1.z - a0.z },
                       { (double)a2.x - a0.x, (double)a2.y - a0.y, (double)a2.z - a0.z },
                       { (double)a3.x - a0.x, (double)a3.y - a0.y, (double)a3.z - a0.z } };
    return e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) + e[0][1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
}

// FP32 6V with a bound on its rounding error (Shewchuk's orient3d bound over
// the translated coordinates, padded)
__host__ __device__ __forceinline__ float tet_vol6_f32(float3 a0, float3 a1, float3 a2, float3 a3, float& bound)
{
    float e1x = a1.x - a0.x, e1y = a1.y - a0.y, e1z = a1.z - a0.z;
    float e2x = a2.x - a0.x, e2y = a2.y - a0.y, e2z = a2.z - a0.z;
    float e3x = a3.x - a0.x, e3y = a3.y - a0.y, e3z = a3.z - a0.z;
    float m1a = e2y * e3z, m1b = e2z * e3y;
    float m2a = e2z * e3x, m2b = e2x * e3z;
    float m3a = e2x * e3y, m3b = e2y * e3x;
    float det = e1x * (m1a - m1b) + e1y * (m2a - m2b) + e1z * (m3a - m3b);
    float perm = fabsf(e1x) * (fabsf(m1a) + fabsf(m1b)) + fabsf(e1y) * (fabsf(m2a) + fabsf(m2b)) +
                 fabsf(e1z) * (fabsf(m3a) + fabsf(m3b));
    bound = 10.0f * EPS32 * perm;
    return det;
}

// |6V| as the star-volume sums take it: FP64 in FP64 mode or when the FP32
// bound is too loose, else the FP32 value; *fixed (may be null) counts the
// tets recomputed in FP64
__device__ __forceinline__ double tet_abs_vol6(int mode_fp64, float3 a0, float3 a1, float3 a2, float3 a3,
                                               unsigned long long* fixed)
{
    if (mode_fp64)
        return fabs(tet_vol6_f64(a0, a1, a2, a3));
    float bound;
    const float d = tet_vol6_f32(a0, a1, a2, a3, bound);
    if (bound > DTFE_TAU * fabsf(d))
    {
        if (fixed) ++*fixed;
        return fabs(tet_vol6_f64(a0, a1, a2, a3));
    }
    return (double)fabsf(d);
}

// Star-volume sums W_v = sum of 6V over v's tets, as exact fixed-point
// integers: every term is rounded once to a multiple of the quantum 1/scale
// (scale a power of two) and the terms are added with 64-bit integer
// atomics, so the sums are exact and independent of the order of the
// additions, and W (hence rho) is bit-reproducible.
//
// Mixed mode: one 64-bit word (lo), scale such that any sum stays below
// 2^62 -- a quantum of 2^-55 for a unit box, finer than the FP32 volumes it
// sums.  FP64 mode: up to 101 bits in two words -- the term q = 6V * scale is
// split into hi = floor(q / 2^40) and lo = q - hi * 2^40, summed separately
// (a lo sum of up to 2^24 terms stays below 2^64, the hi sum of any star
// below 2^61) -- a quantum of 2^-95 for a unit box, so even the smallest tets
// of a dense clump keep FP64 accuracy.
struct StarSum
{
    unsigned long long hi, lo;
};
constexpr double STAR_LO = 1099511627776.0;   // 2^40

__host__ __device__ __forceinline__ void star_term(double vol6, double scale, bool two_words, unsigned long long& hi,
                                                   unsigned long long& lo)
{
    const double x = vol6 * scale;            // exact (power-of-two scale)
    if (!two_words)
    {
        hi = 0;
        lo = (unsigned long long)rint(x);
        return;
    }
    const double h = floor(x / STAR_LO);      // exact
    hi = (unsigned long long)h;
    lo = (unsigned long long)rint(x - h * STAR_LO);   // the difference is exact; rint rounds q's fraction
}

__host__ __device__ __forceinline__ double star_value(unsigned long long hi, unsigned long long lo, double inv_scale)
{
    return ((double)hi * STAR_LO + (double)lo) * inv_scale;
}

// true when a sum left the range its scale was chosen for
__host__ __device__ __forceinline__ bool star_overflow(unsigned long long hi, unsigned long long lo)
{
    return hi >= (1ull << 62) || lo >= (1ull << 63);
}

// the fixed-point scale: 2^bits with any 6V sum of up to 8x the data box
// below 2^62 (one word, mixed mode) or 2^101 (two words, FP64 mode)
inline double star_sum_scale(const float* dmin, const float* dmax, bool two_words)
{
    double vbox = 48.0;
    for (int i = 0; i < 3; ++i)
    {
        const double ext = (double)dmax[i] - (double)dmin[i];
        vbox *= ext > 1e-30 ? ext : 1e-30;
    }
    const int bits = (two_words ? 101 : 61) - (int)ceil(log2(vbox));
    return ldexp(1.0, bits);
}

}  // namespace tg
