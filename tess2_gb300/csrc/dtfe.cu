// DTFE: vertex densities from Delaunay star volumes and tet-linear
// interpolation onto the grid.  The reference has no DTFE; this follows
// Schaap & van de Weygaert (2000): rho_v = (D+1) m / W_v with W_v the summed
// volume of the tets around v, and the grid value is the barycentric
// interpolation of rho in the tet that contains the grid point (0 outside
// every tet).
//
// Point-in-tet decisions are exact.  A grid point p belongs to tet t when the
// symbolically perturbed point p + (e, e^2, e^3) lies strictly inside t, with
// orientation signs of the float32 inputs evaluated exactly.  That makes the
// tets a partition of the triangulated region (one owner per grid point,
// never two, no holes) and gives the same owner as any exact evaluation.
// Each decision is taken by the cheapest test that can certify it:
//   1. the barycentric numerator in working precision with a rigorous error
//      bound (FP32 in mixed mode, FP64 in FP64 mode),
//   2. the orientation determinant in FP64 with Shewchuk's orient3d bound,
//   3. exact expansion arithmetic (Dekker two-product + Shewchuk
//      grow-expansion), and for an exact zero the perturbation's sign.
//
// Mixed mode computes volumes and interpolation weights in FP32 and
// recomputes, in FP64, every tet whose FP32 error bound relative to its
// volume exceeds tau.  FP64 mode computes everything in FP64.
//
// Compiled with -fmad=false: FMAs appear only where written (fmaf/fma), so
// the error bounds below hold as derived.
#include "kernels.h"
#include <float.h>
#include <math.h>

namespace tg {

constexpr unsigned FULL = 0xffffffffu;
constexpr float EPS32 = 5.9604645e-08f;      // 2^-24
constexpr double EPS64 = 1.1102230246251565e-16;  // 2^-53

__device__ __forceinline__ int find_blk(const BlockDesc* b, int nb, int t)
{
    int lo = 0, hi = nb - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (b[mid].t_off <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// exact predicates for float32 inputs
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e)
{
    double x = __dadd_rn(a, b);
    double bv = __dsub_rn(x, a);
    double av = __dsub_rn(x, bv);
    e = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
    s = x;
}

// sign of the exact sum of n doubles (grow-expansion with zero elimination)
__device__ __noinline__ int exact_sign(const double* t, int n)
{
    double e[48];
    int m = 0;
    for (int i = 0; i < n; ++i)
    {
        double q = t[i];
        int k = 0;
        for (int j = 0; j < m; ++j)
        {
            double hi, lo;
            two_sum(q, e[j], hi, lo);
            if (lo != 0.0)
                e[k++] = lo;
            q = hi;
        }
        if (q != 0.0)
            e[k++] = q;
        m = k;
    }
    return m == 0 ? 0 : (e[m - 1] > 0.0 ? 1 : -1);
}

__device__ __forceinline__ int add_triple(double* t, int n, double s, float x, float y, float z)
{
    double xy = (double)x * (double)y;          // exact: 48 significant bits
    double hi = __dmul_rn(xy, (double)z);
    double lo = fma(xy, (double)z, -hi);        // exact remainder
    t[n] = s * hi;
    t[n + 1] = s * lo;
    return n + 2;
}

__device__ __forceinline__ int add_det3(double* t, int n, double s, const float* u, const float* v, const float* w)
{
    n = add_triple(t, n, s, u[0], v[1], w[2]);
    n = add_triple(t, n, -s, u[0], v[2], w[1]);
    n = add_triple(t, n, s, u[1], v[2], w[0]);
    n = add_triple(t, n, -s, u[1], v[0], w[2]);
    n = add_triple(t, n, s, u[2], v[0], w[1]);
    n = add_triple(t, n, -s, u[2], v[1], w[0]);
    return n;
}

// exact sign of O(x,y,z,p) = det[y-x; z-x; p-x]
//   = det3(y,z,p) - det3(x,z,p) + det3(x,y,p) - det3(x,y,z)
__device__ __noinline__ int orient_exact(const float* x, const float* y, const float* z, const float* p)
{
    double t[48];
    int n = 0;
    n = add_det3(t, n, 1.0, y, z, p);
    n = add_det3(t, n, -1.0, x, z, p);
    n = add_det3(t, n, 1.0, x, y, p);
    n = add_det3(t, n, -1.0, x, y, z);
    return exact_sign(t, n);
}

// FP64 evaluation with Shewchuk's orient3d error bound, exact when uncertain
__device__ __noinline__ int orient_filtered(const float* x, const float* y, const float* z, const float* p)
{
    double adx = (double)x[0] - p[0], ady = (double)x[1] - p[1], adz = (double)x[2] - p[2];
    double bdx = (double)y[0] - p[0], bdy = (double)y[1] - p[1], bdz = (double)y[2] - p[2];
    double cdx = (double)z[0] - p[0], cdy = (double)z[1] - p[1], cdz = (double)z[2] - p[2];
    double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    double cdxady = cdx * ady, adxcdy = adx * cdy;
    double adxbdy = adx * bdy, bdxady = bdx * ady;
    double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    double perm = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) + (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz) +
                  (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    double bound = (7.0 + 56.0 * EPS64) * EPS64 * perm;
    // det[x-p; y-p; z-p] = -O(x,y,z,p)
    if (det > bound) return -1;
    if (-det > bound) return 1;
    return orient_exact(x, y, z, p);
}

// exact sign of component j of (y-x) x (z-x)
__device__ __noinline__ int face_normal_sign(const float* x, const float* y, const float* z, int j)
{
    int a = (j + 1) % 3, b = (j + 2) % 3;
    double t[6];
    t[0] = (double)y[a] * z[b];
    t[1] = -(double)y[a] * x[b];
    t[2] = -(double)x[a] * z[b];
    t[3] = -(double)y[b] * z[a];
    t[4] = (double)y[b] * x[a];
    t[5] = (double)x[b] * z[a];
    return exact_sign(t, 6);
}

__constant__ int c_face_of[4][3] = { {1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2} };
__constant__ int c_face_sigma[4] = { -1, 1, -1, 1 };

// exact sign of N_k(p) (the barycentric numerator of vertex k, D_k in the
// oracle) with the perturbation's tie-break; multiplied by s = sign(V6) the
// result is > 0 exactly when the perturbed point is on vertex k's side
__device__ __noinline__ int numerator_sign_exact(const float a[4][3], int k, const float* p)
{
    const float* x = a[c_face_of[k][0]];
    const float* y = a[c_face_of[k][1]];
    const float* z = a[c_face_of[k][2]];
    int o = orient_filtered(x, y, z, p);
    for (int j = 0; j < 3 && o == 0; ++j)
        o = face_normal_sign(x, y, z, j);
    return c_face_sigma[k] * o;
}

// ---------------------------------------------------------------------------
// star volumes and densities
// ---------------------------------------------------------------------------
__device__ __forceinline__ double tet_vol6_f64(float3 a0, float3 a1, float3 a2, float3 a3)
{
    double e[3][3] = { { (double)a1.x - a0.x, (double)a1.y - a0.y, (double)a1.z - a0.z },
                       { (double)a2.x - a0.x, (double)a2.y - a0.y, (double)a2.z - a0.z },
                       { (double)a3.x - a0.x, (double)a3.y - a0.y, (double)a3.z - a0.z } };
    return e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) + e[0][1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
}

// FP32 6*volume with a bound on its rounding error (Shewchuk's orient3d bound
// over the translated coordinates, padded)
__device__ __forceinline__ float tet_vol6_f32(float3 a0, float3 a1, float3 a2, float3 a3, float& bound)
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

__global__ void k_star_volumes(int mode, const BlockDesc* blocks, int nb, int total, const float4* pos,
                               const int4* tv, double* W, float tau, Status* st)
{
    unsigned long long nfix = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        const int4 vi = __ldg(&tv[t]);
        const float3 a0 = ld3(pos, vi.x), a1 = ld3(pos, vi.y), a2 = ld3(pos, vi.z), a3 = ld3(pos, vi.w);
        double vol;
        if (mode == TESSGPU_MODE_FP64)
            vol = fabs(tet_vol6_f64(a0, a1, a2, a3)) / 6.0;
        else
        {
            float bound;
            const float d = tet_vol6_f32(a0, a1, a2, a3, bound);
            if (bound > tau * fabsf(d))
            {
                vol = fabs(tet_vol6_f64(a0, a1, a2, a3)) / 6.0;
                nfix++;
            }
            else
                vol = (double)(fabsf(d) / 6.0f);
        }
        // FP64 sums in L2: the float32 terms add exactly for the usual exponent spread
        atomicAdd(&W[vi.x], vol);
        atomicAdd(&W[vi.y], vol);
        atomicAdd(&W[vi.z], vol);
        atomicAdd(&W[vi.w], vol);
    }
    for (int o = 16; o > 0; o >>= 1)
        nfix += __shfl_xor_sync(FULL, nfix, o);
    if ((threadIdx.x & 31) == 0 && nfix)
        atomicAdd(&st->fp64_tets, nfix);
}

__global__ void k_densities(const double* W, int n, float mass, float* rho32, double* rho64)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    {
        const double w = W[v];
        const double r = w > 0.0 ? 4.0 * (double)mass / w : 0.0;
        rho32[v] = (float)r;
        rho64[v] = r;
    }
}

// ---------------------------------------------------------------------------
// rasterisation, one thread per tet
// ---------------------------------------------------------------------------
// first grid index whose position is >= x (positions are x_i = i*step + gmin in float)
__device__ __forceinline__ int first_at_or_above(float x, float gmin, float step, int lo, int hi)
{
    float f = (x - gmin) / step;
    f = fminf(fmaxf(f, (float)lo - 2.0f), (float)hi + 2.0f);
    int i = (int)floorf(f);
    while (i > lo && (float)(i - 1) * step + gmin >= x) --i;
    while (i <= hi && (float)i * step + gmin < x) ++i;
    return i < lo ? lo : i;
}

template <typename T> struct Real;
template <> struct Real<float>
{
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float abs_(float a) { return fabsf(a); }
    static constexpr float eps = EPS32;
};
template <> struct Real<double>
{
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
    static __device__ __forceinline__ double abs_(double a) { return fabs(a); }
    static constexpr double eps = EPS64;
};

// barycentric numerators N_k(p) = (p - a[base_k]) . c_k in working type T
//   k=1..3: base a0, c1 = e2 x e3, c2 = e3 x e1, c3 = e1 x e2   (e_k = a_k - a0)
//   k=0:    base a1, c0 = (a3 - a1) x (a2 - a1)
// N_0 + N_1 + N_2 + N_3 = 6V, and N_k equals the oracle's D_k.  B_k bounds
// |computed N_k - exact N_k| for every p with lo <= p <= hi: the error of the
// float differences and cross product (6 eps on the two products) times |q|,
// plus 4 eps |c| |q| for the difference p - base and the three-term dot.
template <typename T>
__device__ __forceinline__ void cross_bound(T ux, T uy, T uz, T vx, T vy, T vz, const T* Q, T* c, T& B)
{
    const T eps = Real<T>::eps;
    const T p0a = uy * vz, p0b = uz * vy;
    const T p1a = uz * vx, p1b = ux * vz;
    const T p2a = ux * vy, p2b = uy * vx;
    c[0] = p0a - p0b;
    c[1] = p1a - p1b;
    c[2] = p2a - p2b;
    const T b0 = Q[0] * (6 * eps * (Real<T>::abs_(p0a) + Real<T>::abs_(p0b)) + 4 * eps * Real<T>::abs_(c[0]));
    const T b1 = Q[1] * (6 * eps * (Real<T>::abs_(p1a) + Real<T>::abs_(p1b)) + 4 * eps * Real<T>::abs_(c[1]));
    const T b2 = Q[2] * (6 * eps * (Real<T>::abs_(p2a) + Real<T>::abs_(p2b)) + 4 * eps * Real<T>::abs_(c[2]));
    B = (b0 + b1 + b2) * (T)1.001 + (T)FLT_MIN;
}

template <typename T>
__device__ __forceinline__ void numerators_setup(const float a[4][3], const float* lo, const float* hi,
                                                 T c[4][3], T Bk[4])
{
    const T eps = Real<T>::eps;
    T Q0[3], Q1[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        const T l = lo[d], h = hi[d];
        Q0[d] = fmax(Real<T>::abs_(l - (T)a[0][d]), Real<T>::abs_(h - (T)a[0][d])) * ((T)1 + 4 * eps);
        Q1[d] = fmax(Real<T>::abs_(l - (T)a[1][d]), Real<T>::abs_(h - (T)a[1][d])) * ((T)1 + 4 * eps);
    }
    const T e1x = (T)a[1][0] - (T)a[0][0], e1y = (T)a[1][1] - (T)a[0][1], e1z = (T)a[1][2] - (T)a[0][2];
    const T e2x = (T)a[2][0] - (T)a[0][0], e2y = (T)a[2][1] - (T)a[0][1], e2z = (T)a[2][2] - (T)a[0][2];
    const T e3x = (T)a[3][0] - (T)a[0][0], e3y = (T)a[3][1] - (T)a[0][1], e3z = (T)a[3][2] - (T)a[0][2];
    const T f1x = (T)a[3][0] - (T)a[1][0], f1y = (T)a[3][1] - (T)a[1][1], f1z = (T)a[3][2] - (T)a[1][2];
    const T f2x = (T)a[2][0] - (T)a[1][0], f2y = (T)a[2][1] - (T)a[1][1], f2z = (T)a[2][2] - (T)a[1][2];
    cross_bound<T>(f1x, f1y, f1z, f2x, f2y, f2z, Q1, c[0], Bk[0]);
    cross_bound<T>(e2x, e2y, e2z, e3x, e3y, e3z, Q0, c[1], Bk[1]);
    cross_bound<T>(e3x, e3y, e3z, e1x, e1y, e1z, Q0, c[2], Bk[2]);
    cross_bound<T>(e1x, e1y, e1z, e2x, e2y, e2z, Q0, c[3], Bk[3]);
}

// sign of 6V of tet (a0,a1,a2,a3): FP64 filter, then exact
__device__ __noinline__ int tet_sign(float a00, float a01, float a02, float a10, float a11, float a12,
                                     float a20, float a21, float a22, float a30, float a31, float a32)
{
    const float a[4][3] = { { a00, a01, a02 }, { a10, a11, a12 }, { a20, a21, a22 }, { a30, a31, a32 } };
    return orient_filtered(a[0], a[1], a[2], a[3]);
}

// exact decision for a point the filter left open
__device__ __noinline__ bool inside_exact(float a00, float a01, float a02, float a10, float a11, float a12,
                                          float a20, float a21, float a22, float a30, float a31, float a32,
                                          float px, float py, float pz, int s, unsigned open_mask)
{
    const float a[4][3] = { { a00, a01, a02 }, { a10, a11, a12 }, { a20, a21, a22 }, { a30, a31, a32 } };
    const float p[3] = { px, py, pz };
    for (int k = 0; k < 4; ++k)
        if ((open_mask >> k) & 1)
            if (s * numerator_sign_exact(a, k, p) <= 0)
                return false;
    return true;
}

// One thread per tet.  Tets come from [0, total) or, when list is given,
// from list[0 .. *list_count).
// MIXED (T = float): FP32 classification and values; a tet whose summed
//   bounds exceed tau * |6V| is appended to fix_list instead and left to the
//   FP64 pass.
// !MIXED (T = double): classification and values in FP64 (FP64 mode, and
//   the fix-up pass over fix_list).
template <typename T, bool MIXED>
__global__ void __launch_bounds__(256)
k_raster(const BlockDesc* blocks, int nb, int total, const int* list, const int* list_count, const float4* pos,
         const int4* tv, const float* rho32, const double* rho64, GridDesc g, float tau, float* grid, int* owner,
         int* fix_list, int* fix_count, Status* st)
{
    unsigned long long nexact = 0, nassigned = 0, nfix = 0;
    const int n = list ? *list_count : total;
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < n; it += gridDim.x * blockDim.x)
    {
        const int t = list ? list[it] : it;
        const int b = find_blk(blocks, nb, t);
        const int4 vi = __ldg(&tv[t]);
        const int vid[4] = { vi.x, vi.y, vi.z, vi.w };
        float a[4][3];
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const float4 p4 = __ldg(&pos[vid[k]]);
            a[k][0] = p4.x; a[k][1] = p4.y; a[k][2] = p4.z;
        }
        // index box: grid positions in [lo, hi) per axis (the perturbation
        // moves points up, so a point on an upper bbox face is outside)
        int ilo[3], ihi[3];
        bool empty = false;
        float lo[3], hi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            lo[d] = fminf(fminf(a[0][d], a[1][d]), fminf(a[2][d], a[3][d]));
            hi[d] = fmaxf(fmaxf(a[0][d], a[1][d]), fmaxf(a[2][d], a[3][d]));
            const int olo = blocks[b].gmin_idx[d], ohi = blocks[b].gmax_idx[d];
            ilo[d] = first_at_or_above(lo[d], g.gmin[d], g.step[d], olo, ohi);
            ihi[d] = first_at_or_above(hi[d], g.gmin[d], g.step[d], olo, ohi + 1) - 1;
            if (ihi[d] > ohi) ihi[d] = ohi;
            if (ilo[d] > ihi[d]) empty = true;
        }
        if (empty)
            continue;

        // orientation s = sign(6V): filtered, exact when uncertain
        const float3 A0 = make_float3(a[0][0], a[0][1], a[0][2]), A1 = make_float3(a[1][0], a[1][1], a[1][2]);
        const float3 A2 = make_float3(a[2][0], a[2][1], a[2][2]), A3 = make_float3(a[3][0], a[3][1], a[3][2]);
        int s;
        T v6;
        if (MIXED)
        {
            float vb;
            const float v6f = tet_vol6_f32(A0, A1, A2, A3, vb);
            v6 = v6f;
            if (v6f > vb) s = 1;
            else if (v6f < -vb) s = -1;
            else s = tet_sign(a[0][0], a[0][1], a[0][2], a[1][0], a[1][1], a[1][2], a[2][0], a[2][1], a[2][2],
                              a[3][0], a[3][1], a[3][2]);
        }
        else
        {
            v6 = (T)tet_vol6_f64(A0, A1, A2, A3);
            s = tet_sign(a[0][0], a[0][1], a[0][2], a[1][0], a[1][1], a[1][2], a[2][0], a[2][1], a[2][2],
                         a[3][0], a[3][1], a[3][2]);
        }
        if (s == 0)
            continue;   // flat tet: no interior

        T c[4][3], Bk[4];
        numerators_setup<T>(a, lo, hi, c, Bk);
        if (MIXED && (float)(Bk[0] + Bk[1] + Bk[2] + Bk[3]) > tau * fabsf((float)v6))
        {
            fix_list[atomicAdd(fix_count, 1)] = t;
            nfix++;
            continue;
        }
        T w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            w[k] = (MIXED ? (T)__ldg(&rho32[vid[k]]) : (T)__ldg(&rho64[vid[k]])) / v6;

        const T sf = (T)s;
        const int t_local = t - blocks[b].t_off;
        for (int zi = ilo[2]; zi <= ihi[2]; ++zi)
        {
            const float pzf = zi * g.step[2] + g.gmin[2];
            for (int yi = ilo[1]; yi <= ihi[1]; ++yi)
            {
                const float pyf = yi * g.step[1] + g.gmin[1];
                // row constants and the x range that can hold inside points
                T R[4];
                T xmin = lo[0], xmax = hi[0];
                bool row_empty = false;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    const int base = k == 0 ? 1 : 0;
                    const T qy = (T)pyf - (T)a[base][1], qz = (T)pzf - (T)a[base][2];
                    R[k] = Real<T>::fma_(c[k][1], qy, c[k][2] * qz);
                    const T cx = sf * c[k][0];
                    const T rhs = -Bk[k] - sf * R[k];        // inside needs cx*qx >= rhs, up to rounding
                    if (cx > 0)
                        xmin = fmax(xmin, (T)a[base][0] + rhs / cx);
                    else if (cx < 0)
                        xmax = fmin(xmax, (T)a[base][0] + rhs / cx);
                    else if (rhs > 0)
                        row_empty = true;
                }
                const float slack = 2.0f * g.step[0];
                if (row_empty || (float)xmin > hi[0] + slack || (float)xmax < lo[0] - slack)
                    continue;
                int i0 = ilo[0], i1 = ihi[0];
                if ((float)xmin - slack > lo[0])
                    i0 = max(i0, (int)floorf(((float)xmin - slack - g.gmin[0]) / g.step[0]));
                if ((float)xmax + slack < hi[0])
                    i1 = min(i1, (int)ceilf(((float)xmax + slack - g.gmin[0]) / g.step[0]));
                const size_t row = ((size_t)zi * g.n[1] + yi) * g.n[0];
                for (int xi = i0; xi <= i1; ++xi)
                {
                    const float pxf = xi * g.step[0] + g.gmin[0];
                    const T px = pxf;
                    T N[4];
                    N[0] = Real<T>::fma_(c[0][0], px - (T)a[1][0], R[0]);
                    const T qx = px - (T)a[0][0];
                    N[1] = Real<T>::fma_(c[1][0], qx, R[1]);
                    N[2] = Real<T>::fma_(c[2][0], qx, R[2]);
                    N[3] = Real<T>::fma_(c[3][0], qx, R[3]);
                    bool in = true, out = false;
                    unsigned open = 0;
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                    {
                        const T sn = sf * N[k];
                        const bool ik = sn > Bk[k];
                        in = in && ik;
                        out = out || (sn < -Bk[k]);
                        open |= (ik ? 0u : 1u) << k;
                    }
                    if (out)
                        continue;
                    if (!in)
                    {
                        nexact++;
                        if (!inside_exact(a[0][0], a[0][1], a[0][2], a[1][0], a[1][1], a[1][2], a[2][0], a[2][1],
                                          a[2][2], a[3][0], a[3][1], a[3][2], pxf, pyf, pzf, s, open))
                            continue;
                    }
                    const T f = Real<T>::fma_(N[0], w[0], Real<T>::fma_(N[1], w[1],
                                              Real<T>::fma_(N[2], w[2], N[3] * w[3])));
                    grid[row + xi] = (float)f;
                    if (owner)
                        owner[row + xi] = t_local;
                    nassigned++;
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        nexact += __shfl_xor_sync(FULL, nexact, o);
        nassigned += __shfl_xor_sync(FULL, nassigned, o);
        nfix += __shfl_xor_sync(FULL, nfix, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        if (nexact) atomicAdd(&st->exact_tests, nexact);
        if (nassigned) atomicAdd(&st->assigned, nassigned);
        if (nfix) atomicAdd(&st->fp64_tets, nfix);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int grid_for(long long n, int block, int per_sm)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long need = (n + block - 1) / block;
    long long cap = (long long)sms * per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

void launch_star_volumes(int mode, const BlockDesc* d_blocks, int nb, int total, const float4* pos,
                         const int4* tv, double* W, float tau, Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    k_star_volumes<<<grid_for(total, 256, 8), 256, 0, s>>>(mode, d_blocks, nb, total, pos, tv, W, tau, st);
}

void launch_densities(const double* W, int n, float mass, float* rho32, double* rho64, cudaStream_t s)
{
    if (n <= 0) return;
    k_densities<<<grid_for(n, 256, 8), 256, 0, s>>>(W, n, mass, rho32, rho64);
}

void launch_raster(int mode, const BlockDesc* d_blocks, int nb, int total, const float4* pos, const int4* tv,
                   const float* rho32, const double* rho64, const GridDesc& g, float tau, float* grid, int* owner,
                   int* fix_list, int* fix_count, Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    const int nblk = grid_for(total, 256, 8);
    if (mode == TESSGPU_MODE_FP64)
        k_raster<double, false><<<nblk, 256, 0, s>>>(d_blocks, nb, total, nullptr, nullptr, pos, tv, rho32, rho64, g,
                                                      tau, grid, owner, nullptr, nullptr, st);
    else
        k_raster<float, true><<<nblk, 256, 0, s>>>(d_blocks, nb, total, nullptr, nullptr, pos, tv, rho32, rho64, g,
                                                    tau, grid, owner, fix_list, fix_count, st);
}

// the ill-conditioned tets the mixed pass listed, in FP64; the launch is sized
// for the longest possible list and reads the length on the device
void launch_raster_fix(const BlockDesc* d_blocks, int nb, int total, const float4* pos, const int4* tv,
                       const float* rho32, const double* rho64, const GridDesc& g, float* grid, int* owner,
                       const int* fix_list, const int* fix_count, Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    k_raster<double, false><<<grid_for(total / 64 + 1, 256, 2), 256, 0, s>>>(
        d_blocks, nb, total, fix_list, fix_count, pos, tv, rho32, rho64, g, 0.0f, grid, owner, nullptr, nullptr, st);
}

}  // namespace tg
