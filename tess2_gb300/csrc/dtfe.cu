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
#include "dtfe_common.cuh"
#include <float.h>
#include <limits.h>
#include <math.h>

namespace tg {

constexpr unsigned FULL = 0xffffffffu;

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
// Star volumes W_v are sums of the volumes of v's tets (accumulated as 6V,
// the orientation determinants).  Each term is rounded once to a multiple of
// 2^-scale_bits and added with 64-bit integer
// atomics: the sum is exact and independent of the order of the additions,
// so W (and rho) is bit-reproducible.  scale_bits keeps any star volume below
// 2^62 (the host derives it from the data bounds).
// rho_v = (D+1) m / W_v = 4 m / W_v, 0 for a vertex in no tet.  The sums
// hold 6x the volumes (the determinants), so rho = 24 m / sum.
__global__ void k_densities(const StarSum* W, int n, float mass, double inv_scale, float* rho32, double* rho64,
                            Status* st)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    {
        const StarSum wv = W[v];
        if (star_overflow(wv.hi, wv.lo))
            fail(st, TESSGPU_ERR_UNSUPPORTED, v);   // star volume past the fixed-point range
        const double w = star_value(wv.hi, wv.lo, inv_scale);
        const double r = w > 0.0 ? 24.0 * (double)mass / w : 0.0;
        rho32[v] = (float)r;
        rho64[v] = r;
    }
}

// ---------------------------------------------------------------------------
// rasterisation, one thread per tet
// ---------------------------------------------------------------------------
// first grid index whose position is >= x (positions are x_i = i*step + gmin in float)
__device__ __forceinline__ int first_at_or_above(float x, float gmin, float step, float inv_step, int lo, int hi)
{
    float f = (x - gmin) * inv_step;
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

// Work decomposition: a warp takes 32 tets.  Each lane sets up one tet
// (bounding box in grid indices, orientation, the four numerator planes with
// their error bounds, interpolation weights) into shared memory; then the
// warp walks the concatenated list of the 32 tets' grid rows (y, z pairs of
// their boxes), one row per lane, so a tet spanning thousands of rows is
// spread over the lanes instead of serialising one.  A row finds the x range
// its four planes allow, tests those points with the filter (exact
// arithmetic when it cannot decide) and writes the interpolated density of
// every point inside.  "x" is the tet's row axis (perm3): the axis across
// which it projects smallest, so it has the fewest rows.
//
// Instances:
//   T=float,  VAL64=false, LIST=false  mixed main pass: FP32 classification and
//       values; an ill-conditioned tet (summed bounds > tau * |6V|) is only
//       appended to fix_list
//   T=float,  VAL64=true,  LIST=true   mixed fix-up pass over fix_list: the same
//       exact classification, values from an FP64 evaluation
//   T=double, VAL64=true,  LIST=false  FP64 mode: everything in FP64
// tets with at most SLICES z slices visit only their cross-section rows (the
// launch variants with SL = 0 visit every row of the box and let the rows'
// x intervals drop the empty ones: no per-slice set-up)
constexpr int SLICES = 16;

template <typename T> struct Vec4;
template <> struct Vec4<float> { typedef float4 type; };
template <> struct Vec4<double> { typedef double4_32a type; };

template <typename T, bool VAL64, bool COMPACT, bool FLAT = false, int SL = SLICES>
struct __align__(32) RasterSmem
{
    typedef typename Vec4<T>::type T4;
    // per tet of the current batch (lane = tet slot)
    float4 A0[32], A1[32];                   // vertices 0, 1 (row-axis order); .w = bbox lo, hi along the row axis
    int    TG[32];                           // global tet index (the exact path reloads vertices 2, 3)
    int    BK[32];                           // the tet's block (its grid)
    T4     C[4][32];                         // c_k.x, c_k.y, c_k.z, B_k
    T4     W[32];                            // rho_k / 6V
    float4 XA[32], XB[32], XG[32];           // face k's x bound on row (dy, dz): XA_k + XB_k dy + XG_k dz
    int4   I0[32];                           // ix0, ix1, iy0, ny
    int4   I1[32];                           // iz0, s, local tet index, face masks | sliced flag | row axis
    int    SLC[SL > 0 ? SL : 1][32];         // per z slice: first row dy << 16 | rows
    int    pre[33];                          // prefix of the tets' row counts
    // FLAT: a round's points spread over the lanes (per row of the round)
    T      RN[4][FLAT ? 32 : 1];             // the row's R_k
    int    RJ[FLAT ? 32 : 1], RI0[FLAT ? 32 : 1], RY[FLAT ? 32 : 1], RZ[FLAT ? 32 : 1];   // tet slot, first x, y, z
    int    pp[FLAT ? 33 : 1];                // prefix of the rows' point counts
    int    Q[COMPACT ? 64 : 1];              // tets whose box holds grid points, waiting for a batch
    double C64[VAL64 && sizeof(T) == 4 ? 12 : 1][32];   // FP64 values for the fix-up pass
    double W64[VAL64 && sizeof(T) == 4 ? 4 : 1][32];
};

template <typename T> __device__ __forceinline__ T comp4(const typename Vec4<T>::type& v, int i)
{
    return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// the tet's vertices and the index box of grid points it can hold inside its
// block's grid box (positions from the block's grid; g is not read); true when
// that box is empty.  Box = the grid points whose
// float position x_i = i*step + gmin satisfies lo <= x_i < hi on every axis:
// the perturbed point x_i + (e, e^2, e^3) can only be inside the tet then.
__device__ __forceinline__ bool tet_box_in(const BlockDesc& bd, const float4* pos, const int4* tv,
                                           const GridDesc& g, int t, int* vid, float a[4][3], float* lo,
                                           float* hi, int* ilo, int* ihi)
{
    const int4 vi = __ldg(&tv[t]);
    vid[0] = vi.x; vid[1] = vi.y; vid[2] = vi.z; vid[3] = vi.w;
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const float4 p4 = __ldg(&pos[vid[k]]);
        a[k][0] = p4.x; a[k][1] = p4.y; a[k][2] = p4.z;
    }
    bool empty = false;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        lo[d] = fminf(fminf(a[0][d], a[1][d]), fminf(a[2][d], a[3][d]));
        hi[d] = fmaxf(fmaxf(a[0][d], a[1][d]), fmaxf(a[2][d], a[3][d]));
        const int olo = bd.gmin_idx[d], ohi = bd.gmax_idx[d];
        const BlockGrid& gb = bd.grid;
        ilo[d] = first_at_or_above(lo[d], gb.gmin[d], gb.step[d], gb.inv_step[d], olo, ohi);
        ihi[d] = first_at_or_above(hi[d], gb.gmin[d], gb.step[d], gb.inv_step[d], olo, ohi + 1) - 1;
        if (ihi[d] > ohi) ihi[d] = ohi;
        if (ilo[d] > ihi[d]) empty = true;
    }
    return empty;
}

__device__ __forceinline__ bool tet_box(const BlockDesc* blocks, int nb, const float4* pos, const int4* tv,
                                        const GridDesc& g, int t, int& b, int* vid, float a[4][3], float* lo,
                                        float* hi, int* ilo, int* ihi)
{
    b = find_blk(blocks, nb, t);
    return tet_box_in(blocks[b], pos, tv, g, t, vid, a, lo, hi, ilo, ihi);
}

// Each tet's rows run along the axis of its smallest projected area (fewest
// rows).  Row axis ra: the tet's coordinates are taken in the order
// (ra, b, c) = (0,1,2), (1,0,2) or (2,0,1); "x" below is the row axis, "y"
// the axis of the rows within a z slice, "z" the slice axis.  The arithmetic
// and its error bounds are the same in any order.
template <typename V>
__device__ __forceinline__ void perm3(int ra, V o0, V o1, V o2, V& n0, V& n1, V& n2)
{
    n0 = ra == 0 ? o0 : (ra == 1 ? o1 : o2);
    n1 = ra == 0 ? o1 : o0;
    n2 = ra == 2 ? o1 : o2;
}
template <typename V>
__device__ __forceinline__ void unperm3(int ra, V n0, V n1, V n2, V& x, V& y, V& z)
{
    x = ra == 0 ? n0 : n1;
    y = ra == 0 ? n1 : (ra == 1 ? n0 : n2);
    z = ra == 2 ? n0 : n2;
}

// flat index of grid point (xi, yi, zi) given in the tet's row-axis order
__device__ __forceinline__ size_t grid_index(const BlockGrid& g, int ra, int xi, int yi, int zi)
{
    int gx_, gy_, gz_;
    unperm3(ra, xi, yi, zi, gx_, gy_, gz_);
    return g.off + ((size_t)gz_ * g.n[1] + gy_) * g.n[0] + gx_;
}

// one grid point of a row: classify against the tet's four numerator planes
// (exact arithmetic when the filter cannot decide) and write the
// interpolated density when it is inside
// xi, yi, zi and pyf, pzf are in the tet's row-axis order; hx, gx the row
// axis' grid step and origin
template <typename T, bool VAL64, typename SM>
__device__ __forceinline__ void raster_point(const SM& S, int j, int xi, float pyf, float pzf, const float4& A0,
                                             const float4& A1, const int4& I1, const T* cx, const T* RN, const T* Bk,
                                             float hx, float gx, int ra, size_t gi, const int4* tv,
                                             const float4* pos, float* grid, int* owner,
                                             unsigned long long& nexact, unsigned long long& nassigned)
{
    typedef typename Vec4<T>::type T4;
    constexpr bool F32 = sizeof(T) == 4;
    const float pxf = xi * hx + gx;
    const T px = pxf;
    const int s = I1.y;
    T N[4];   // s N_k: the tables hold s c_k (see the setup)
    N[0] = Real<T>::fma_(cx[0], px - (T)A1.x, RN[0]);
    const T qx = px - (T)A0.x;
    N[1] = Real<T>::fma_(cx[1], qx, RN[1]);
    N[2] = Real<T>::fma_(cx[2], qx, RN[2]);
    N[3] = Real<T>::fma_(cx[3], qx, RN[3]);
    bool in = true, out = false;
    unsigned open = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const T sn = N[k];
        const bool ik = sn > Bk[k];
        in = in && ik;
        out = out || (sn < -Bk[k]);
        open |= (ik ? 0u : 1u) << k;
    }
    if (out)
        return;
    if (!in)
    {
        nexact++;
        const int4 vt = __ldg(&tv[S.TG[j]]);
        const float4 A2 = __ldg(&pos[vt.z]), A3 = __ldg(&pos[vt.w]);
        float a0x, a0y, a0z, a1x, a1y, a1z, qx_, qy_, qz_;
        unperm3(ra, A0.x, A0.y, A0.z, a0x, a0y, a0z);
        unperm3(ra, A1.x, A1.y, A1.z, a1x, a1y, a1z);
        unperm3(ra, pxf, pyf, pzf, qx_, qy_, qz_);
        if (!inside_exact(a0x, a0y, a0z, a1x, a1y, a1z, A2.x, A2.y, A2.z, A3.x, A3.y, A3.z, qx_, qy_, qz_, s, open))
            return;
    }
    float f;
    if (!VAL64 || !F32)
    {
        const T4 W4 = S.W[j];
        f = (float)Real<T>::fma_(N[0], W4.x, Real<T>::fma_(N[1], W4.y, Real<T>::fma_(N[2], W4.z, N[3] * W4.w)));
    }
    else
    {
        // the FP64 tables are in x, y, z order
        float a0x, a0y, a0z, a1x, a1y, a1z, qx_, qy_, qz_;
        unperm3(ra, A0.x, A0.y, A0.z, a0x, a0y, a0z);
        unperm3(ra, A1.x, A1.y, A1.z, a1x, a1y, a1z);
        unperm3(ra, pxf, pyf, pzf, qx_, qy_, qz_);
        const double q1[3] = { (double)qx_ - a1x, (double)qy_ - a1y, (double)qz_ - a1z };
        const double q0[3] = { (double)qx_ - a0x, (double)qy_ - a0y, (double)qz_ - a0z };
        double acc = 0.0;
        for (int k = 0; k < 4; ++k)
        {
            const double* qq = k == 0 ? q1 : q0;
            acc += (qq[0] * S.C64[3 * k][j] + qq[1] * S.C64[3 * k + 1][j] + qq[2] * S.C64[3 * k + 2][j]) *
                   S.W64[k][j];
        }
        f = (float)acc;
    }
    grid[gi] = f;
    if (owner)
        owner[gi] = I1.z;
    nassigned++;
}

// PB: every block has its own grid (independent sets); otherwise all blocks
// share the call's grid g
template <typename T, bool VAL64, bool LIST, int MINB, int NW, bool COMPACT, bool FLAT, bool PB, int SL = SLICES>
__global__ void __launch_bounds__(NW * 32, MINB)
k_raster(const BlockDesc* blocks, int nb, int total, const int* list, const int* list_count, const float4* pos,
         const int4* tv, const float* rho32, const double* rho64, GridDesc g, float tau, float* grid, int* owner,
         int* fix_list, int* fix_count, Status* st, int t0, int* next)
{
    typedef typename Vec4<T>::type T4;
    BlockGrid gshared;   // the shared grid (read from the kernel's parameters)
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        gshared.gmin[d] = g.gmin[d];
        gshared.step[d] = g.step[d];
        gshared.inv_step[d] = g.inv_step[d];
        gshared.n[d] = g.n[d];
    }
    gshared.off = 0;
    __shared__ RasterSmem<T, VAL64, COMPACT, FLAT, SL> smem[NW];
    constexpr bool F32 = sizeof(T) == 4;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    RasterSmem<T, VAL64, COMPACT, FLAT, SL>& S = smem[wid];
    unsigned long long nexact = 0, nassigned = 0, nfix = 0, nrows = 0, ncand = 0;
    const int n = LIST ? *list_count : total;
    const int nchunks = (n + 31) / 32;
    int qn = 0;   // queued tets (warp-uniform)
    // next: persistent warps take chunks of 32 tets in order from a counter
    // (a chunk of background tets costs far more than one of clump tets);
    // otherwise a fixed grid-stride share per warp
    int chunk = blockIdx.x * NW + wid;
    for (bool first = true;; first = false)
    {
        if (next)
        {
            int c = 0;
            if (lane == 0)
                c = atomicAdd(next, 1);
            chunk = __shfl_sync(FULL, c, 0);
        }
        else if (!first)
            chunk += gridDim.x * NW;
        const bool more = chunk < nchunks;
        if (COMPACT && more)
        {
            // ---- screen: keep the tets whose box holds grid points
            const int it = chunk * 32 + lane;
            bool keep = false;
            int t = -1;
            if (it < n)
            {
                t = LIST ? list[it] : t0 + it;
                int b, vid[4], ilo[3], ihi[3];
                float a[4][3], lo[3], hi[3];
                keep = !tet_box(blocks, nb, pos, tv, g, t, b, vid, a, lo, hi, ilo, ihi);
            }
            const unsigned m = __ballot_sync(FULL, keep);
            if (keep)
                S.Q[qn + __popc(m & ((1u << lane) - 1u))] = t;
            qn += __popc(m);
            __syncwarp();
        }
        if (!COMPACT && more)
            qn = 32;   // the chunk itself is the batch
        while (qn >= 32 || (!more && qn > 0))
        {
            // ---- a batch of up to 32 tets, one per lane
            int tq;
            if (COMPACT)
            {
                const int take = min(qn, 32);
                tq = lane < take ? S.Q[lane] : -1;
                const int rest = qn - take;
                const int carry = lane < rest ? S.Q[take + lane] : 0;
                __syncwarp();
                if (lane < rest)
                    S.Q[lane] = carry;
                qn = rest;
            }
            else
            {
                const int it = chunk * 32 + lane;
                tq = it < n ? (LIST ? list[it] : t0 + it) : -1;
                qn = 0;
            }
            int rows = 0;
            if (tq >= 0)
            {
                const int t = tq;
                int b, vid[4], ilo[3], ihi[3];
                float a[4][3], lo[3], hi[3];
                const bool empty = tet_box(blocks, nb, pos, tv, g, t, b, vid, a, lo, hi, ilo, ihi);
                int s = 0;
                T v6 = 0;
                if (!empty)
                {
                    const float3 A0 = make_float3(a[0][0], a[0][1], a[0][2]), A1 = make_float3(a[1][0], a[1][1], a[1][2]);
                    const float3 A2 = make_float3(a[2][0], a[2][1], a[2][2]), A3 = make_float3(a[3][0], a[3][1], a[3][2]);
                    if (F32)
                    {
                        float vb;
                        const float v6f = tet_vol6_f32(A0, A1, A2, A3, vb);
                        v6 = v6f;
                        if (v6f > vb) s = 1;
                        else if (v6f < -vb) s = -1;
                        else s = tet_sign(a[0][0], a[0][1], a[0][2], a[1][0], a[1][1], a[1][2], a[2][0], a[2][1],
                                          a[2][2], a[3][0], a[3][1], a[3][2]);
                    }
                    else
                    {
                        v6 = (T)tet_vol6_f64(A0, A1, A2, A3);
                        s = tet_sign(a[0][0], a[0][1], a[0][2], a[1][0], a[1][1], a[1][2], a[2][0], a[2][1], a[2][2],
                                     a[3][0], a[3][1], a[3][2]);
                    }
                }
                if (s != 0)   // s == 0: flat tet, no interior
                {
                    T c[4][3], Bk[4];
                    numerators_setup<T>(a, lo, hi, c, Bk);
                    bool keep = true;
                    if (F32 && !VAL64 && fix_list &&
                        (float)(Bk[0] + Bk[1] + Bk[2] + Bk[3]) > tau * fabsf((float)v6))
                    {
                        fix_list[atomicAdd(fix_count, 1)] = t;   // values need FP64: the fix-up pass
                        nfix++;
                        keep = false;
                    }
                    if (keep)
                    {
                        S.TG[lane] = t;
                        T4 w4;
                        const float r6 = F32 ? __frcp_rn((float)v6) : 0.0f;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                        {
                            const T sg = (T)s;
                            const T wk = sg * (F32 ? (T)(__ldg(&rho32[vid[k]]) * r6) : (T)__ldg(&rho64[vid[k]]) / v6);
                            if (k == 0) w4.x = wk;
                            else if (k == 1) w4.y = wk;
                            else if (k == 2) w4.z = wk;
                            else w4.w = wk;
                        }
                        S.W[lane] = w4;
                        if (VAL64 && F32)
                        {
                            double e[3][3], f1[3], f2[3];
                            for (int k = 0; k < 3; ++k)
                                for (int d = 0; d < 3; ++d)
                                    e[k][d] = (double)a[k + 1][d] - (double)a[0][d];
                            for (int d = 0; d < 3; ++d)
                            {
                                f1[d] = (double)a[3][d] - (double)a[1][d];
                                f2[d] = (double)a[2][d] - (double)a[1][d];
                            }
                            double cc[4][3];
                            for (int jj = 0; jj < 3; ++jj)
                            {
                                const int ja = (jj + 1) % 3, jb = (jj + 2) % 3;
                                cc[0][jj] = f1[ja] * f2[jb] - f1[jb] * f2[ja];
                                cc[1][jj] = e[1][ja] * e[2][jb] - e[1][jb] * e[2][ja];
                                cc[2][jj] = e[2][ja] * e[0][jb] - e[2][jb] * e[0][ja];
                                cc[3][jj] = e[0][ja] * e[1][jb] - e[0][jb] * e[1][ja];
                            }
                            const double v6d = e[0][0] * cc[1][0] + e[0][1] * cc[1][1] + e[0][2] * cc[1][2];
                            for (int k = 0; k < 4; ++k)
                            {
                                for (int jj = 0; jj < 3; ++jj)
                                    S.C64[3 * k + jj][lane] = cc[k][jj];
                                S.W64[k][lane] = __ldg(&rho64[vid[k]]) / v6d;
                            }
                        }
                        // the row axis: the one along which the tet's projection is smallest
                        // (the projected area across axis d is half the sum of |c_k[d]|)
                        int ra = 0;
                        {
                            float pr[3];
#pragma unroll
                            for (int d = 0; d < 3; ++d)
                                pr[d] = fabsf((float)c[0][d]) + fabsf((float)c[1][d]) + fabsf((float)c[2][d]) +
                                        fabsf((float)c[3][d]);
                            if (pr[1] < pr[0] && pr[1] <= pr[2]) ra = 1;
                            else if (pr[2] < pr[0] && pr[2] < pr[1]) ra = 2;
                        }
                        // everything below in (row axis, y, z) order
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                        {
                            perm3(ra, a[k][0], a[k][1], a[k][2], a[k][0], a[k][1], a[k][2]);
                            perm3(ra, c[k][0], c[k][1], c[k][2], c[k][0], c[k][1], c[k][2]);
                        }
                        perm3(ra, lo[0], lo[1], lo[2], lo[0], lo[1], lo[2]);
                        perm3(ra, hi[0], hi[1], hi[2], hi[0], hi[1], hi[2]);
                        perm3(ra, ilo[0], ilo[1], ilo[2], ilo[0], ilo[1], ilo[2]);
                        perm3(ra, ihi[0], ihi[1], ihi[2], ihi[0], ihi[1], ihi[2]);
                        float gst[3], gmn[3], ginv[3];
                        const BlockGrid& gb = PB ? blocks[b].grid : gshared;
                        S.BK[lane] = b;
                        perm3(ra, gb.step[0], gb.step[1], gb.step[2], gst[0], gst[1], gst[2]);
                        perm3(ra, gb.gmin[0], gb.gmin[1], gb.gmin[2], gmn[0], gmn[1], gmn[2]);
                        perm3(ra, gb.inv_step[0], gb.inv_step[1], gb.inv_step[2], ginv[0], ginv[1], ginv[2]);
                        S.A0[lane] = make_float4(a[0][0], a[0][1], a[0][2], lo[0]);
                        S.A1[lane] = make_float4(a[1][0], a[1][1], a[1][2], hi[0]);
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                        {
                            // the orientation folded in (exact: s = +-1): a point is inside
                            // when every s N_k > B_k, and s N_k times s rho_k / 6V is the
                            // same product, so the points need no sign multiply
                            const T sg = (T)s;
                            T4 ck;
                            ck.x = sg * c[k][0]; ck.y = sg * c[k][1]; ck.z = sg * c[k][2]; ck.w = Bk[k];
                            S.C[k][lane] = ck;
                        }
                        // Row-wise x bounds.  Inside needs s*N_k >= -B_k, N_k = c_kx (x - bx)
                        // + R_k(y, z); along row (dy, dz) of the box this is x >= bnd_k
                        // (s c_kx > 0) or x <= bnd_k (s c_kx < 0) with
                        //   bnd_k = bx - s B_k / c_kx - R_k / c_kx, affine in (dy, dz).
                        // E_k covers the rounding of the coefficients, of the float grid
                        // positions against the affine form, and of N_k's own evaluation,
                        // so a point outside [max lower, min upper] fails the per-point
                        // test for some face.  c_kx == 0 gives no x bound.
                        const int nyb = ihi[1] - ilo[1] + 1, nzb = ihi[2] - ilo[2] + 1;
                        int masks = 0;
                        {
                            const float h1 = gst[1], h2 = gst[2];
                            const float py0 = ilo[1] * h1 + gmn[1], pz0 = ilo[2] * h2 + gmn[2];
                            const float ymx = fmaxf(fabsf(py0), fabsf(ihi[1] * h1 + gmn[1]));
                            const float zmx = fmaxf(fabsf(pz0), fabsf(ihi[2] * h2 + gmn[2]));
                            const float xmx = fmaxf(fabsf(lo[0]), fabsf(hi[0]));
                            float xa[4], xb[4], xg[4];
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                            {
                                const int base = k == 0 ? 1 : 0;
                                const float bx = a[base][0], by = a[base][1], bz = a[base][2];
                                const float cx = (float)c[k][0], cy = (float)c[k][1], cz = (float)c[k][2];
                                const float B = (float)Bk[k];
                                if (cx == 0.0f)
                                {
                                    xa[k] = 0.0f; xb[k] = 0.0f; xg[k] = 0.0f;
                                    masks |= 1 << (4 + k);   // no x bound from this face
                                    continue;
                                }
                                const float icx = __frcp_rn(cx);
                                const float R0 = cy * (py0 - by) + cz * (pz0 - bz);
                                const float alpha = bx - (float)s * B * icx - R0 * icx;
                                const float beta = -cy * h1 * icx, gamma = -cz * h2 * icx;
                                const float E = 32.0f * EPS32 *
                                    (fabsf(bx) + xmx + fabsf(alpha) + fabsf(B * icx) + fabsf(R0 * icx) +
                                     fabsf(beta) * nyb + fabsf(gamma) * nzb +
                                     (fabsf(cy) * (ymx + fabsf(by)) + fabsf(cz) * (zmx + fabsf(bz))) * fabsf(icx)) +
                                    1e-30f;
                                const bool lo_face = (float)s * cx > 0.0f;
                                masks |= lo_face ? 1 << k : 0;
                                xa[k] = lo_face ? alpha - E : alpha + E;
                                xb[k] = beta;
                                xg[k] = gamma;
                            }
                            S.XA[lane] = make_float4(xa[0], xa[1], xa[2], xa[3]);
                            S.XB[lane] = make_float4(xb[0], xb[1], xb[2], xb[3]);
                            S.XG[lane] = make_float4(xg[0], xg[1], xg[2], xg[3]);
                        }
                        S.I0[lane] = make_int4(ilo[0], ihi[0], ilo[1], nyb);
                        if (nzb <= SL)
                        {
                            // rows of slice z: the y range of the tet's cross-section there,
                            // from the edges that cross the plane, widened by a rounding
                            // margin (an extra row is only visited, a dropped row would lose
                            // points)
                            float idz[6];
#pragma unroll
                            for (int e = 0; e < 6; ++e)
                            {
                                const int u = e < 3 ? 0 : (e < 5 ? 1 : 2);
                                const int v = e < 3 ? e + 1 : (e < 5 ? e - 1 : 3);
                                const float dz = a[v][2] - a[u][2];
                                idz[e] = dz != 0.0f ? __frcp_rn(dz) : 0.0f;
                            }
                            for (int zo = 0; zo < nzb; ++zo)
                            {
                                const float pz = (ilo[2] + zo) * gst[2] + gmn[2];
                                float ylo = FLT_MAX, yhi = -FLT_MAX;
#pragma unroll
                                for (int e = 0; e < 6; ++e)
                                {
                                    const int u = e < 3 ? 0 : (e < 5 ? 1 : 2);
                                    const int v = e < 3 ? e + 1 : (e < 5 ? e - 1 : 3);
                                    const float za = a[u][2], zb = a[v][2];
                                    if (pz < fminf(za, zb) || pz > fmaxf(za, zb))
                                        continue;
                                    float y0, y1;
                                    if (za == zb)
                                    {
                                        y0 = a[u][1];
                                        y1 = a[v][1];
                                    }
                                    else
                                    {
                                        const float tt = fminf(fmaxf((pz - za) * idz[e], 0.0f), 1.0f);
                                        y0 = y1 = fmaf(tt, a[v][1] - a[u][1], a[u][1]);
                                    }
                                    ylo = fminf(ylo, fminf(y0, y1));
                                    yhi = fmaxf(yhi, fmaxf(y0, y1));
                                }
                                int cnt = 0, d0 = 0;
                                if (ylo <= yhi)
                                {
                                    const float my = 64.0f * EPS32 * (fmaxf(fabsf(ylo), fabsf(yhi)) + hi[1] - lo[1]);
                                    const float f0 = (ylo - my - gmn[1]) * ginv[1];
                                    const float f1 = (yhi + my - gmn[1]) * ginv[1];
                                    const float mm = 1e-3f + 8.0f * EPS32 *
                                        ((fabsf(gmn[1]) + fmaxf(fabsf(ylo), fabsf(yhi))) * ginv[1] +
                                         fmaxf(fabsf(f0), fabsf(f1)));
                                    const int y0i = max(ilo[1], (int)ceilf(fmaxf(f0 - mm, (float)(ilo[1] - 1))));
                                    const int y1i = min(ihi[1], (int)floorf(fminf(f1 + mm, (float)(ihi[1] + 1))));
                                    if (y1i >= y0i)
                                    {
                                        cnt = y1i - y0i + 1;
                                        d0 = y0i - ilo[1];
                                    }
                                }
                                S.SLC[zo][lane] = (d0 << 16) | cnt;
                                rows += cnt;
                            }
                            masks |= 1 << 8;   // sliced
                        }
                        else
                            rows = nyb * nzb;
                        S.I1[lane] = make_int4(ilo[2], s, t - blocks[b].t_off, masks | (ra << 9));
                    }
                }
            }
            // exclusive prefix of the tets' row counts
            int incl = rows;
            for (int o = 1; o < 32; o <<= 1)
            {
                const int v = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += v;
            }
            S.pre[lane + 1] = incl;
            if (lane == 0) S.pre[0] = 0;
            __syncwarp();
            const int R = S.pre[32];

            // ---- rounds of 32 rows: a lane per row finds its x range, then the
            // rows' points are spread over the lanes
            int j = 0;
            for (int rbase = 0; rbase < R; rbase += 32)
            {
                const int r = rbase + lane;
                int cnt = 0;   // FLAT: this lane's row's points
                if (r < R)
                {
                    while (S.pre[j + 1] <= r) ++j;
                    const int rr = r - S.pre[j];
                    const int4 I0 = S.I0[j];
                    const int4 I1 = S.I1[j];
                    int zo, dy;
                    if ((I1.w >> 8) & 1)
                    {
                        int q = rr;
                        zo = 0;
                        int sl = S.SLC[0][j];
                        while (q >= (sl & 0xffff))
                        {
                            q -= sl & 0xffff;
                            sl = S.SLC[++zo][j];
                        }
                        dy = (sl >> 16) + q;
                    }
                    else
                    {
                        const int ny = I0.w;
                        zo = (int)(((float)rr + 0.5f) * __frcp_rn((float)ny));
                        if (zo * ny > rr) --zo;
                        else if ((zo + 1) * ny <= rr) ++zo;
                        dy = rr - zo * ny;
                    }
                    const float4 A0 = S.A0[j], A1 = S.A1[j];
                    float xmin = A0.w, xmax = A1.w;
                    {
                        const float4 XA = S.XA[j], XB = S.XB[j], XG = S.XG[j];
                        const float fdy = (float)dy, fdz = (float)zo;
                        const int m = I1.w & 0xff;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                        {
                            const float bnd = fmaf(comp4<float>(XG, k), fdz,
                                                   fmaf(comp4<float>(XB, k), fdy, comp4<float>(XA, k)));
                            if ((m >> (4 + k)) & 1) continue;
                            if ((m >> k) & 1) xmin = fmaxf(xmin, bnd);
                            else xmax = fminf(xmax, bnd);
                        }
                    }
                    nrows++;
                    if (xmin <= xmax)
                    {
                        // the tet's axes: row axis ra, then y, z (see perm3)
                        const int ra = (I1.w >> 9) & 3;
                        const BlockGrid& gb = PB ? blocks[S.BK[j]].grid : gshared;
                        float gst[3], gmn[3], ginv0;
                        perm3(ra, gb.step[0], gb.step[1], gb.step[2], gst[0], gst[1], gst[2]);
                        perm3(ra, gb.gmin[0], gb.gmin[1], gb.gmin[2], gmn[0], gmn[1], gmn[2]);
                        ginv0 = ra == 0 ? gb.inv_step[0] : (ra == 1 ? gb.inv_step[1] : gb.inv_step[2]);
                        // grid indices inside [xmin, xmax]: an index estimate widened by m
                        // grid steps, where m exceeds the rounding of the estimate and of the
                        // float grid positions (2 eps |pos| each), so no point in the range is
                        // dropped; an extra point at the edge is classified like any other
                        const float f0 = (xmin - gmn[0]) * ginv0;
                        const float f1 = (xmax - gmn[0]) * ginv0;
                        const float mg = 1e-3f + 8.0f * EPS32 * ((fabsf(gmn[0]) + fmaxf(fabsf(xmin), fabsf(xmax))) *
                                                                 ginv0 + fmaxf(fabsf(f0), fabsf(f1)));
                        const int i0 = max(I0.x, (int)ceilf(fmaxf(f0 - mg, (float)(I0.x - 1))));
                        const int i1 = min(I0.y, (int)floorf(fminf(f1 + mg, (float)(I0.y + 1))));
                        if (i0 <= i1)
                        {
                            const int yi = I0.z + dy, zi = I1.x + zo;
                            const float pyf = yi * gst[1] + gmn[1];
                            const float pzf = zi * gst[2] + gmn[2];
                            T RN[4];
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                            {
                                const T4 ck = S.C[k][j];
                                const float by = k == 0 ? A1.y : A0.y, bz = k == 0 ? A1.z : A0.z;
                                const T qy = (T)pyf - (T)by, qz = (T)pzf - (T)bz;
                                RN[k] = Real<T>::fma_(ck.y, qy, ck.z * qz);
                            }
                            ncand += i1 - i0 + 1;
                            // this lane's row, point by point
                            T cx[4], Bk[4];
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                            {
                                const T4 ck = S.C[k][j];
                                cx[k] = ck.x;
                                Bk[k] = ck.w;
                            }
                            if (FLAT)
                            {
#pragma unroll
                                for (int k = 0; k < 4; ++k)
                                    S.RN[k][lane] = RN[k];
                                S.RJ[lane] = j;
                                S.RI0[lane] = i0;
                                S.RY[lane] = yi;
                                S.RZ[lane] = zi;
                                cnt = i1 - i0 + 1;
                            }
                            else
                            {
                                // the row's grid index advances by the row axis' stride
                                const size_t stride = ra == 0 ? 1 : (ra == 1 ? (size_t)gb.n[0]
                                                                             : (size_t)gb.n[0] * gb.n[1]);
                                size_t gi = grid_index(gb, ra, i0, yi, zi);
                                for (int xi = i0; xi <= i1; ++xi, gi += stride)
                                    raster_point<T, VAL64>(S, j, xi, pyf, pzf, A0, A1, I1, cx, RN, Bk, gst[0], gmn[0],
                                                           ra, gi, tv, pos, grid, owner, nexact, nassigned);
                            }
                        }
                    }
                }
                if (FLAT)
                {
                    // prefix of the rows' point counts, then the points spread over the lanes
                    int pin = cnt;
                    for (int o = 1; o < 32; o <<= 1)
                    {
                        const int v = __shfl_up_sync(FULL, pin, o);
                        if (lane >= o) pin += v;
                    }
                    S.pp[lane + 1] = pin;
                    if (lane == 0) S.pp[0] = 0;
                    __syncwarp();
                    const int P = S.pp[32];
                    int rs = 0;
                    for (int q = lane; q < P; q += 32)
                    {
                        while (S.pp[rs + 1] <= q) ++rs;
                        const int jj = S.RJ[rs];
                        const int xi = S.RI0[rs] + (q - S.pp[rs]);
                        const int yi = S.RY[rs], zi = S.RZ[rs];
                        const float4 A0 = S.A0[jj], A1 = S.A1[jj];
                        const int4 I1 = S.I1[jj];
                        const int ra = (I1.w >> 9) & 3;
                        const BlockGrid& gb = PB ? blocks[S.BK[jj]].grid : gshared;
                        float gst[3], gmn[3];
                        perm3(ra, gb.step[0], gb.step[1], gb.step[2], gst[0], gst[1], gst[2]);
                        perm3(ra, gb.gmin[0], gb.gmin[1], gb.gmin[2], gmn[0], gmn[1], gmn[2]);
                        const float pyf = yi * gst[1] + gmn[1];
                        const float pzf = zi * gst[2] + gmn[2];
                        T cx[4], Bk[4], RN[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                        {
                            const T4 ck = S.C[k][jj];
                            cx[k] = ck.x;
                            Bk[k] = ck.w;
                            RN[k] = S.RN[k][rs];
                        }
                        raster_point<T, VAL64>(S, jj, xi, pyf, pzf, A0, A1, I1, cx, RN, Bk, gst[0], gmn[0], ra,
                                               grid_index(gb, ra, xi, yi, zi), tv, pos, grid, owner, nexact,
                                               nassigned);
                    }
                }
                __syncwarp();
            }
            __syncwarp();
        }
        if (!more)
            break;
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        nexact += __shfl_xor_sync(FULL, nexact, o);
        nassigned += __shfl_xor_sync(FULL, nassigned, o);
        nfix += __shfl_xor_sync(FULL, nfix, o);
        nrows += __shfl_xor_sync(FULL, nrows, o);
        ncand += __shfl_xor_sync(FULL, ncand, o);
    }
    if (lane == 0)
    {
        if (nrows) atomicAdd(&st->rows, nrows);
        if (ncand) atomicAdd(&st->candidates, ncand);
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

void launch_densities(const StarSum* W, int n, float mass, double inv_scale, float* rho32, double* rho64,
                      Status* st, cudaStream_t s)
{
    if (n <= 0) return;
    k_densities<<<grid_for(n, 256, 8), 256, 0, s>>>(W, n, mass, inv_scale, rho32, rho64, st);
}

// Launch variants.  Block residency per SM trades registers against latency
// hiding; COMPACT screens tets with empty boxes out before the setup; FLAT
// spreads a round's points over the lanes (it pays when a point is expensive,
// as in FP64 mode, and costs more shared-memory traffic than it saves when a
// point is cheap).  The fastest depends on the GPU, the mesh and the mode, so
// the caller times them.
//   0..2: per-lane rows, 4/5/6 blocks per SM    3: compact, 5 blocks
//   4..5: compact + flat, 4/5 blocks per SM
//   6..7: per-lane rows, 4/5 blocks per SM, every row of the box (no slices)
constexpr int N_RASTER_VARIANTS = 8;

// Blocks of a rasteriser launch: with a chunk counter, one resident wave of
// persistent blocks (the kernel's occupancy per SM); otherwise up to 16 per SM
// with a fixed share of the chunks each.
template <typename K>
static int raster_grid(K kernel, int threads, long long work, bool persistent)
{
    if (!persistent)
        return grid_for(work, threads, 16);
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
    const long long need = (work + threads - 1) / threads;
    const long long cap = (long long)sms * (per_sm > 0 ? per_sm : 1);
    return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

template <typename T, bool VAL64, bool LIST>
static void raster_variant(int variant, long long work, cudaStream_t s, const BlockDesc* d_blocks, int nb, int total,
                           const int* list, const int* list_count, const float4* pos, const int4* tv,
                           const float* rho32, const double* rho64, const GridDesc& g, float tau, float* grid,
                           int* owner, int* fix_list, int* fix_count, Status* st, int t0 = 0, bool per_block = false,
                           int* next = nullptr)
{
    // the double-precision tables need more shared memory: 3 warps per block
    constexpr int NW = (sizeof(T) == 4 && !VAL64) ? 4 : 3;
    if (per_block)
    {
        // per-block grids: one launch configuration (5 blocks per SM)
        auto kfn = k_raster<T, VAL64, LIST, 5, NW, false, false, true>;
        kfn<<<raster_grid(kfn, NW * 32, work, next != nullptr), NW * 32, 0, s>>>(
            d_blocks, nb, total, list, list_count, pos, tv, rho32, rho64, g, tau, grid, owner, fix_list, fix_count, st,
            t0, next);
        return;
    }
#define TG_RASTER(MB, C, F, SL_)                                                                                   \
    {                                                                                                              \
        auto kfn = k_raster<T, VAL64, LIST, MB, NW, C, F, false, SL_>;                                             \
        kfn<<<raster_grid(kfn, NW * 32, work, next != nullptr), NW * 32, 0, s>>>(                                  \
            d_blocks, nb, total, list, list_count, pos, tv, rho32, rho64, g, tau, grid, owner, fix_list, fix_count, \
            st, t0, next);                                                                                         \
    }
    switch (variant)
    {
    case 1: TG_RASTER(5, false, false, SLICES); break;
    case 2: TG_RASTER(6, false, false, SLICES); break;
    case 3: TG_RASTER(5, true, false, SLICES); break;
    case 4: TG_RASTER(4, true, true, SLICES); break;
    case 5: TG_RASTER(5, true, true, SLICES); break;
    case 6: TG_RASTER(4, false, false, 0); break;
    case 7: TG_RASTER(5, false, false, 0); break;
    default: TG_RASTER(4, false, false, SLICES); break;
    }
#undef TG_RASTER
}

int raster_variants() { return N_RASTER_VARIANTS; }


void launch_raster(int mode, int variant, const BlockDesc* d_blocks, int nb, int total, const float4* pos,
                   const int4* tv, const float* rho32, const double* rho64, const GridDesc& g, float tau, float* grid,
                   int* owner, int* fix_list, int* fix_count, Status* st, cudaStream_t s, const int* order,
                   const int* order_count, int t0, bool per_block, int* next)
{
    if (total <= 0) return;
    const long long work = (long long)((total + 31) / 32) * 32 * 32;
    if (order)
    {
        if (mode == TESSGPU_MODE_FP64)
            raster_variant<double, true, true>(variant, work, s, d_blocks, nb, total, order, order_count, pos, tv,
                                               rho32, rho64, g, tau, grid, owner, nullptr, nullptr, st);
        else
            raster_variant<float, false, true>(variant, work, s, d_blocks, nb, total, order, order_count, pos, tv,
                                               rho32, rho64, g, tau, grid, owner, fix_list, fix_count, st);
        return;
    }
    if (mode == TESSGPU_MODE_FP64)
        raster_variant<double, true, false>(variant, work, s, d_blocks, nb, total, nullptr, nullptr, pos, tv, rho32,
                                            rho64, g, tau, grid, owner, nullptr, nullptr, st, t0, per_block, next);
    else
        raster_variant<float, false, false>(variant, work, s, d_blocks, nb, total, nullptr, nullptr, pos, tv, rho32,
                                            rho64, g, tau, grid, owner, fix_list, fix_count, st, t0, per_block, next);
}

// ---------------------------------------------------------------------------
// spatial processing order of the tets
// ---------------------------------------------------------------------------
// The rasteriser writes each grid point once, 4 bytes at a time; tets in
// Qhull's order scatter those writes over the grid, so a 32-byte sector is
// written back to HBM several times (partial sectors cost a read-modify-write
// too).  Processing the tets brick by brick (8x8x8 grid points, bricks in
// x-fastest order, by the brick of the tet's centroid) keeps the sectors
// being written in L2.  A counting sort: key and histogram, one exclusive
// scan, scatter.  The order within a brick follows the atomics; the grid does
// not depend on it (every grid point has exactly one owner tet).
__global__ void k_order_keys(const float4* pos, const int4* tv, int total, GridDesc g, int nbx, int nby, int nbz,
                             int* key, int* hist)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        const int4 v = __ldg(&tv[t]);
        const float4 a = __ldg(&pos[v.x]), b = __ldg(&pos[v.y]), c = __ldg(&pos[v.z]), d = __ldg(&pos[v.w]);
        const float cen[3] = { 0.25f * ((a.x + b.x) + (c.x + d.x)), 0.25f * ((a.y + b.y) + (c.y + d.y)),
                               0.25f * ((a.z + b.z) + (c.z + d.z)) };
        const int nbk[3] = { nbx, nby, nbz };
        int br[3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
        {
            const float f = (cen[i] - g.gmin[i]) * g.inv_step[i];
            int gi = f > 0.0f ? (int)fminf(f, (float)(g.n[i] - 1)) : 0;
            br[i] = min(gi >> 3, nbk[i] - 1);
        }
        const int k = (br[2] * nby + br[1]) * nbx + br[0];
        key[t] = k;
        atomicAdd(&hist[k], 1);
    }
}

// exclusive prefix sum of n counts in place, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_scan_counts(int* a, int n)
{
    __shared__ long long part[1024];
    const int per = (n + 1023) / 1024;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    long long s = 0;
    for (int i = lo; i < hi; ++i)
        s += a[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1)
    {
        const long long v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = part[threadIdx.x] - s;
    for (int i = lo; i < hi; ++i)
    {
        const int c = a[i];
        a[i] = (int)run;
        run += c;
    }
}

__global__ void k_order_scatter(const int* key, int total, int* cursor, int* order)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
        order[atomicAdd(&cursor[key[t]], 1)] = t;
}

void order_bricks(const GridDesc& g, int* nbx, int* nby, int* nbz)
{
    *nbx = (g.n[0] + 7) >> 3;
    *nby = (g.n[1] + 7) >> 3;
    *nbz = (g.n[2] + 7) >> 3;
}

void launch_tet_order(const float4* pos, const int4* tv, int total, const GridDesc& g, int* key, int* hist,
                      int* order, cudaStream_t s)
{
    if (total <= 0) return;
    int nbx, nby, nbz;
    order_bricks(g, &nbx, &nby, &nbz);
    const int nk = nbx * nby * nbz;
    cudaMemsetAsync(hist, 0, sizeof(int) * nk, s);
    k_order_keys<<<grid_for(total, 256, 8), 256, 0, s>>>(pos, tv, total, g, nbx, nby, nbz, key, hist);
    k_scan_counts<<<1, 1024, 0, s>>>(hist, nk);
    k_order_scatter<<<grid_for(total, 256, 8), 256, 0, s>>>(key, total, hist, order);
}

// the tets the mixed pass listed, with FP64 values; sized for the longest
// possible list, the length is read on the device
void launch_raster_fix(const BlockDesc* d_blocks, int nb, int total, const float4* pos, const int4* tv,
                       const float* rho32, const double* rho64, const GridDesc& g, float* grid, int* owner,
                       const int* fix_list, const int* fix_count, Status* st, cudaStream_t s, bool per_block)
{
    if (total <= 0) return;
    const long long work = (long long)((total / 16 + 31) / 32) * 32 * 32;
    raster_variant<float, true, true>(0, work, s, d_blocks, nb, total, fix_list, fix_count, pos, tv, rho32, rho64, g,
                                      0.0f, grid, owner, nullptr, nullptr, st, 0, per_block);
}


// ===========================================================================
// brick rasteriser
// ===========================================================================
// Work decomposition.  The grid box of every block is cut into bricks of
// BX x BY x BZ grid points (powers of two) aligned to the global grid and
// clipped at the box's edges.  A brick's candidates are the tets whose grid
// box (tet_box_in) overlaps it, found by a counting sort of the (tet, brick)
// pairs: count, scan, scatter.  One CTA takes one brick: it rasterises the
// brick's candidates into a tile in shared memory and writes the tile out
// once, whole, in x rows of BX floats, with zeros where no tet owns a point;
// so no grid zeroing pass is needed and each grid sector is written once.
// A brick with more than BRICK_CHUNK candidates (a dense clump) is split into
// several items of that many; its region is zeroed first and each item
// writes only the points its own tets hold.
//
// Inside the CTA each warp takes 32 candidates at a time, one per lane, and
// sets them up into its shared-memory slots: grid box clipped to the brick,
// orientation, the numerator planes and error bounds of the point-in-tet
// test, interpolation weights, the x bounds of a row as affine functions of
// (y, z), the edge slopes of the z slices.  The 32 tets' work is then spread
// over the lanes level by level, so that no lane waits on another tet's long
// loop: the z slices of all 32 tets (a lane per slice: the y range of the
// tet's cross-section there), the rows of 32 slices (a lane per row: the x
// range its face bounds allow), the points of 32 rows (a lane per point: the
// filtered test, exact arithmetic when the filter cannot decide, and the
// interpolated value written to the tile).  A level finds its parent through
// an owner table the parent lanes fill.  Owners, tests and values are those
// of k_raster: the same predicates, bounds and expressions.
constexpr int BRICK_CHUNK = 2048;
constexpr unsigned BRICK_UNSET = 0xffffffffu;   // a NaN no arithmetic produces

template <typename T, int SX, int SY, int SZ>
struct __align__(32) BrickWarp
{
    typedef typename Vec4<T>::type T4;
    T4     C[4][32];                // s c_k (x, y, z) and B_k
    T4     W[32];                   // s rho_k / 6V
    double F[4][32];                // FP64 fix-up tets: rho_0 and the field's gradient
    float4 P[4][32];                // vertices; w: lo x, hi x, lo y, hi y of the tet's box
    float4 XA[32], XB[32], XG[32];  // face k's x bound on row (dy, dz): XA_k + XB_k dy + XG_k dz
    float  IDZ[6][32];              // 1 / (z_v - z_u) of the six edges (0 for an edge in a z plane)
    int4   I0[32];                  // box clipped to the brick: x0, x1, y0, y1
    int4   I1[32];                  // z0 (clipped), box's first y and z, flags
    int    TG[32];                  // tet index
    int    pre1[33];                // exclusive prefix of the tets' slice counts
    unsigned char own1[32 << SZ];   // the tet slot of every slice
};

// brick b's block (blocks' bricks are numbered in block order)
__device__ __forceinline__ int brick_block(const BlockDesc* blocks, int nb, int b)
{
    int lo = 0, hi = nb - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (blocks[mid].brick_base <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// grid points [r0, r1] of brick b of block bd
__device__ __forceinline__ void brick_region(const BlockDesc& bd, int b, int sx, int sy, int sz, int* r0, int* r1)
{
    const int l = b - bd.brick_base;
    const int bx = l % bd.brick_n[0], by = (l / bd.brick_n[0]) % bd.brick_n[1], bz = l / (bd.brick_n[0] * bd.brick_n[1]);
    const int c[3] = { bx, by, bz }, sh[3] = { sx, sy, sz };
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        const int s0 = (bd.brick_lo[d] + c[d]) << sh[d];
        r0[d] = max(s0, bd.gmin_idx[d]);
        r1[d] = min(s0 + (1 << sh[d]) - 1, bd.gmax_idx[d]);
    }
}

// the bricks tet t's grid box overlaps: brick coordinates relative to the block
__device__ __forceinline__ bool tet_bricks(const BlockDesc& bd, const float4* pos, const int4* tv, const GridDesc& g,
                                           int t, int sx, int sy, int sz, int* b0, int* b1)
{
    int vid[4], ilo[3], ihi[3];
    float a[4][3], lo[3], hi[3];
    if (tet_box_in(bd, pos, tv, g, t, vid, a, lo, hi, ilo, ihi))
        return false;
    const int sh[3] = { sx, sy, sz };
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        b0[d] = (ilo[d] >> sh[d]) - bd.brick_lo[d];
        b1[d] = (ihi[d] >> sh[d]) - bd.brick_lo[d];
    }
    return true;
}

// the term (hi, lo) added to W[key]: one or two 64-bit integer atomics.  (Merging
// the terms of the warp's lanes that share a vertex first, with match and
// reduce instructions, made the kernel five times slower on this GPU.)
__device__ __forceinline__ void add_star(StarSum* W, int key, unsigned long long hi, unsigned long long lo,
                                         bool two_words)
{
    if (two_words)
        atomicAdd(&W[key].hi, hi);
    atomicAdd(&W[key].lo, lo);
}

// Star volumes of tets [t0, t0 + nt); with BIN, also the brick rasteriser's
// pair counts of those tets (the same vertex loads serve both).
template <bool BIN>
__global__ void k_star_volumes(int mode, int t0, int nt, const float4* pos, const int4* tv, StarSum* W,
                               double scale, Status* st, const BlockDesc* blocks, int nb, GridDesc g, int sx, int sy,
                               int sz, int* cnt)
{
    const int lane = threadIdx.x & 31;
    unsigned long long nfix = 0;
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < nt;
         it += (long long)gridDim.x * blockDim.x)
    {
        const int4 vi = __ldg(&tv[t0 + it]);
        const float3 a0 = ld3(pos, vi.x), a1 = ld3(pos, vi.y), a2 = ld3(pos, vi.z), a3 = ld3(pos, vi.w);
        const double vol = tet_abs_vol6(mode == TESSGPU_MODE_FP64, a0, a1, a2, a3, &nfix);
        const bool two = mode == TESSGPU_MODE_FP64;
        unsigned long long qh, ql;
        star_term(vol, scale, two, qh, ql);
        add_star(W, vi.x, qh, ql, two);
        add_star(W, vi.y, qh, ql, two);
        add_star(W, vi.z, qh, ql, two);
        add_star(W, vi.w, qh, ql, two);
        if (BIN)
        {
            const int t = t0 + (int)it;
            const BlockDesc& bd = blocks[find_blk(blocks, nb, t)];
            int b0[3], b1[3];
            if (tet_bricks(bd, pos, tv, g, t, sx, sy, sz, b0, b1))
                for (int z = b0[2]; z <= b1[2]; ++z)
                    for (int y = b0[1]; y <= b1[1]; ++y)
                        for (int x = b0[0]; x <= b1[0]; ++x)
                            atomicAdd(&cnt[bd.brick_base + (z * bd.brick_n[1] + y) * bd.brick_n[0] + x], 1);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        nfix += __shfl_xor_sync(FULL, nfix, o);
    if (lane == 0 && nfix)
        atomicAdd(&st->fp64_tets, nfix);
}

// (tet, brick) pairs per brick
__global__ void k_bin_count(const BlockDesc* blocks, int nb, int t0, int nt, const float4* pos, const int4* tv,
                            GridDesc g, int sx, int sy, int sz, int* cnt)
{
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nt; it += gridDim.x * blockDim.x)
    {
        const int t = t0 + it;
        const BlockDesc& bd = blocks[find_blk(blocks, nb, t)];
        int b0[3], b1[3];
        if (tet_bricks(bd, pos, tv, g, t, sx, sy, sz, b0, b1))
            for (int z = b0[2]; z <= b1[2]; ++z)
                for (int y = b0[1]; y <= b1[1]; ++y)
                    for (int x = b0[0]; x <= b1[0]; ++x)
                        atomicAdd(&cnt[bd.brick_base + (z * bd.brick_n[1] + y) * bd.brick_n[0] + x], 1);
    }
}

// Bricks [bb0, bb1) of one segment (blocks whose tets are binned together):
// exclusive prefixes of the pair counts (placed in the pair list at an
// offset taken from the shared cursor) and of the items (ceil(count /
// BRICK_CHUNK), at least one per brick).  One CTA of 1024 threads.
__global__ void __launch_bounds__(1024)
k_bin_scan(int bb0, int bb1, int seg, const int* cnt, int* off, int* cur, int* item_off, int* seg_items,
           unsigned long long* pair_cursor, long long pair_cap, Status* st)
{
    __shared__ long long pc[1024], pi[1024];
    __shared__ long long s_base;
    __shared__ int s_ok;
    const int n = bb1 - bb0;
    const int per = (n + 1023) / 1024;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    long long sc = 0, si = 0;
    for (int i = lo; i < hi; ++i)
    {
        const int c = cnt[bb0 + i];
        sc += c;
        si += c > 0 ? (c + BRICK_CHUNK - 1) / BRICK_CHUNK : 1;
    }
    pc[threadIdx.x] = sc;
    pi[threadIdx.x] = si;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const long long a = threadIdx.x >= (unsigned)o ? pc[threadIdx.x - o] : 0;
        const long long b = threadIdx.x >= (unsigned)o ? pi[threadIdx.x - o] : 0;
        __syncthreads();
        pc[threadIdx.x] += a;
        pi[threadIdx.x] += b;
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        const long long tot = pc[1023];
        const unsigned long long base = atomicAdd(pair_cursor, (unsigned long long)tot);
        const bool ok = (long long)base + tot <= pair_cap;
        if (!ok)
            fail(st, TESSGPU_ERR_CAPACITY, (int)min(tot, (long long)INT_MAX));
        s_base = (long long)base;
        s_ok = ok;
        seg_items[seg] = ok ? (int)pi[1023] : 0;
    }
    __syncthreads();
    if (!s_ok)
    {
        // the list is too small: no item runs (seg_items is 0), and every
        // cursor points past the list so the scatter writes nothing
        for (int i = lo; i < hi; ++i)
        {
            off[bb0 + i] = (int)min(pair_cap, (long long)INT_MAX);
            cur[bb0 + i] = (int)min(pair_cap, (long long)INT_MAX);
            item_off[bb0 + i] = 0;
        }
        return;
    }
    long long rc = s_base + pc[threadIdx.x] - sc, ri = pi[threadIdx.x] - si;
    for (int i = lo; i < hi; ++i)
    {
        const int c = cnt[bb0 + i];
        off[bb0 + i] = (int)rc;
        cur[bb0 + i] = (int)rc;
        item_off[bb0 + i] = (int)ri;
        rc += c;
        ri += c > 0 ? (c + BRICK_CHUNK - 1) / BRICK_CHUNK : 1;
    }
}

// the pairs themselves: each brick's tets, in the order the atomics give
__global__ void k_bin_scatter(const BlockDesc* blocks, int nb, int t0, int nt, const float4* pos, const int4* tv,
                              GridDesc g, int sx, int sy, int sz, int* cur, int* pairs, long long pair_cap)
{
    for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nt; it += gridDim.x * blockDim.x)
    {
        const int t = t0 + it;
        const BlockDesc& bd = blocks[find_blk(blocks, nb, t)];
        int b0[3], b1[3];
        if (tet_bricks(bd, pos, tv, g, t, sx, sy, sz, b0, b1))
            for (int z = b0[2]; z <= b1[2]; ++z)
                for (int y = b0[1]; y <= b1[1]; ++y)
                    for (int x = b0[0]; x <= b1[0]; ++x)
                    {
                        const int q = atomicAdd(&cur[bd.brick_base + (z * bd.brick_n[1] + y) * bd.brick_n[0] + x], 1);
                        if (q >= 0 && q < pair_cap)
                            pairs[q] = t;
                    }
    }
}

// the regions of the split bricks are zeroed before their items run
__global__ void k_zero_split(const BlockDesc* blocks, int nb, int bb0, int bb1, int seg, const int* item_off,
                             const int* seg_items, int sx, int sy, int sz, GridDesc g, float* grid)
{
    for (int b = bb0 + blockIdx.x; b < bb1; b += gridDim.x)
    {
        const int i1 = b + 1 < bb1 ? item_off[b + 1] : seg_items[seg];
        if (i1 - item_off[b] <= 1)
            continue;
        const BlockDesc& bd = blocks[brick_block(blocks, nb, b)];
        int r0[3], r1[3];
        brick_region(bd, b, sx, sy, sz, r0, r1);
        const int nx = r1[0] - r0[0] + 1, ny = r1[1] - r0[1] + 1, nz = r1[2] - r0[2] + 1;
        const BlockGrid& gb = bd.grid;
        for (int i = threadIdx.x; i < nx * ny * nz; i += blockDim.x)
        {
            const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
            grid[gb.off + ((size_t)(r0[2] + z) * gb.n[1] + (r0[1] + y)) * gb.n[0] + (r0[0] + x)] = 0.0f;
        }
    }
}

// exclusive prefix of v over the warp into pre[0..32]; returns the total
__device__ __forceinline__ int warp_prefix(int v, int lane, int* pre)
{
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int u = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += u;
    }
    pre[lane + 1] = incl;
    if (lane == 0) pre[0] = 0;
    return __shfl_sync(FULL, incl, 31);
}

struct BrickCounts
{
    unsigned long long exact = 0, assigned = 0, fix = 0, rows = 0, cand = 0;
};

// one warp, up to 32 candidates [ci0, ci1) of the brick r0..r1
template <typename T, int SX, int SY, int SZ>
__device__ __forceinline__ void brick_batch(BrickWarp<T, SX, SY, SZ>& S, float* tile, const int* r0, const int* r1,
                                            int ci0, int ci1, const int* pairs, const BlockDesc& bd,
                                            const float4* pos, const int4* tv, const float* rho32,
                                            const double* rho64, const GridDesc& g0, int* owner, int fixup,
                                            BrickCounts& cn)
{
    typedef typename Vec4<T>::type T4;
    constexpr bool F32 = sizeof(T) == 4;
    const int lane = threadIdx.x & 31;
    const BlockGrid& g = bd.grid;   // the block's own grid
    int ns = 0;
    if (ci0 + lane < ci1)
    {
        const int t = __ldg(&pairs[ci0 + lane]);
        int vid[4], ilo[3], ihi[3];
        float a[4][3], lo[3], hi[3];
        const bool empty = tet_box_in(bd, pos, tv, g0, t, vid, a, lo, hi, ilo, ihi);
        const int cx0 = max(ilo[0], r0[0]), cx1 = min(ihi[0], r1[0]);
        const int cy0 = max(ilo[1], r0[1]), cy1 = min(ihi[1], r1[1]);
        const int cz0 = max(ilo[2], r0[2]), cz1 = min(ihi[2], r1[2]);
        if (!empty && cx0 <= cx1 && cy0 <= cy1 && cz0 <= cz1)
        {
            const float3 A0 = make_float3(a[0][0], a[0][1], a[0][2]), A1 = make_float3(a[1][0], a[1][1], a[1][2]);
            const float3 A2 = make_float3(a[2][0], a[2][1], a[2][2]), A3 = make_float3(a[3][0], a[3][1], a[3][2]);
            int s;
            T v6;
            if (F32)
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
            if (s != 0)   // s == 0: flat tet, no interior
            {
                T c[4][3], Bk[4];
                numerators_setup<T>(a, lo, hi, c, Bk);
                const bool fix = F32 && fixup && (float)(Bk[0] + Bk[1] + Bk[2] + Bk[3]) > DTFE_TAU * fabsf((float)v6);
                if (fix && cx0 == ilo[0] && cy0 == ilo[1] && cz0 == ilo[2])
                    cn.fix++;   // counted in the brick that holds the box's first corner
                T4 w4;
                const float r6 = F32 ? __frcp_rn((float)v6) : 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    const T wk = (T)s * (F32 ? (T)(__ldg(&rho32[vid[k]]) * r6) : (T)__ldg(&rho64[vid[k]]) / v6);
                    if (k == 0) w4.x = wk;
                    else if (k == 1) w4.y = wk;
                    else if (k == 2) w4.z = wk;
                    else w4.w = wk;
                }
                S.W[lane] = w4;
                if (fix)
                {
                    // values in FP64: rho(p) = rho_0 + (p - a0) . G with G = sum_k rho_k c_k / 6V
                    double e[3][3], f1[3], f2[3], cc[4][3];
                    for (int k = 0; k < 3; ++k)
                        for (int d = 0; d < 3; ++d)
                            e[k][d] = (double)a[k + 1][d] - (double)a[0][d];
                    for (int d = 0; d < 3; ++d)
                    {
                        f1[d] = (double)a[3][d] - (double)a[1][d];
                        f2[d] = (double)a[2][d] - (double)a[1][d];
                    }
                    for (int jj = 0; jj < 3; ++jj)
                    {
                        const int ja = (jj + 1) % 3, jb = (jj + 2) % 3;
                        cc[0][jj] = f1[ja] * f2[jb] - f1[jb] * f2[ja];
                        cc[1][jj] = e[1][ja] * e[2][jb] - e[1][jb] * e[2][ja];
                        cc[2][jj] = e[2][ja] * e[0][jb] - e[2][jb] * e[0][ja];
                        cc[3][jj] = e[0][ja] * e[1][jb] - e[0][jb] * e[1][ja];
                    }
                    const double v6d = e[0][0] * cc[1][0] + e[0][1] * cc[1][1] + e[0][2] * cc[1][2];
                    double G[3] = { 0.0, 0.0, 0.0 };
                    for (int k = 0; k < 4; ++k)
                    {
                        const double wk = __ldg(&rho64[vid[k]]) / v6d;
                        for (int d = 0; d < 3; ++d)
                            G[d] += wk * cc[k][d];
                    }
                    S.F[0][lane] = __ldg(&rho64[vid[0]]);
                    S.F[1][lane] = G[0];
                    S.F[2][lane] = G[1];
                    S.F[3][lane] = G[2];
                }
                S.P[0][lane] = make_float4(a[0][0], a[0][1], a[0][2], lo[0]);
                S.P[1][lane] = make_float4(a[1][0], a[1][1], a[1][2], hi[0]);
                S.P[2][lane] = make_float4(a[2][0], a[2][1], a[2][2], lo[1]);
                S.P[3][lane] = make_float4(a[3][0], a[3][1], a[3][2], hi[1]);
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    // the orientation folded in (s = +-1 exactly): inside when every s N_k > B_k
                    const T sg = (T)s;
                    T4 ck;
                    ck.x = sg * c[k][0]; ck.y = sg * c[k][1]; ck.z = sg * c[k][2]; ck.w = Bk[k];
                    S.C[k][lane] = ck;
                }
                // row-wise x bounds (see k_raster): bnd_k = bx - s B_k / c_kx - R_k / c_kx,
                // affine in the row's offsets (dy, dz) from the box's first row, widened by E
                int masks = 0;
                {
                    const int nyb = ihi[1] - ilo[1] + 1, nzb = ihi[2] - ilo[2] + 1;
                    const float h1 = g.step[1], h2 = g.step[2];
                    const float py0 = ilo[1] * h1 + g.gmin[1], pz0 = ilo[2] * h2 + g.gmin[2];
                    const float ymx = fmaxf(fabsf(py0), fabsf(ihi[1] * h1 + g.gmin[1]));
                    const float zmx = fmaxf(fabsf(pz0), fabsf(ihi[2] * h2 + g.gmin[2]));
                    const float xmx = fmaxf(fabsf(lo[0]), fabsf(hi[0]));
                    float xa[4], xb[4], xg[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                    {
                        const int base = k == 0 ? 1 : 0;
                        const float bx = a[base][0], by = a[base][1], bz = a[base][2];
                        const float cx = (float)c[k][0], cy = (float)c[k][1], cz = (float)c[k][2];
                        const float B = (float)Bk[k];
                        if (cx == 0.0f)
                        {
                            xa[k] = 0.0f; xb[k] = 0.0f; xg[k] = 0.0f;
                            masks |= 1 << (4 + k);   // no x bound from this face
                            continue;
                        }
                        const float icx = __frcp_rn(cx);
                        const float R0 = cy * (py0 - by) + cz * (pz0 - bz);
                        const float alpha = bx - (float)s * B * icx - R0 * icx;
                        const float beta = -cy * h1 * icx, gamma = -cz * h2 * icx;
                        const float E = 32.0f * EPS32 *
                            (fabsf(bx) + xmx + fabsf(alpha) + fabsf(B * icx) + fabsf(R0 * icx) +
                             fabsf(beta) * nyb + fabsf(gamma) * nzb +
                             (fabsf(cy) * (ymx + fabsf(by)) + fabsf(cz) * (zmx + fabsf(bz))) * fabsf(icx)) +
                            1e-30f;
                        const bool lo_face = (float)s * cx > 0.0f;
                        masks |= lo_face ? 1 << k : 0;
                        xa[k] = lo_face ? alpha - E : alpha + E;
                        xb[k] = beta;
                        xg[k] = gamma;
                    }
                    S.XA[lane] = make_float4(xa[0], xa[1], xa[2], xa[3]);
                    S.XB[lane] = make_float4(xb[0], xb[1], xb[2], xb[3]);
                    S.XG[lane] = make_float4(xg[0], xg[1], xg[2], xg[3]);
                }
#pragma unroll
                for (int e = 0; e < 6; ++e)
                {
                    const int u = e < 3 ? 0 : (e < 5 ? 1 : 2);
                    const int v = e < 3 ? e + 1 : (e < 5 ? e - 1 : 3);
                    const float dz = a[v][2] - a[u][2];
                    S.IDZ[e][lane] = dz != 0.0f ? __frcp_rn(dz) : 0.0f;
                }
                S.I0[lane] = make_int4(cx0, cx1, cy0, cy1);
                S.I1[lane] = make_int4(cz0, ilo[1], ilo[2], masks | (s > 0 ? 1 << 8 : 0) | (fix ? 1 << 9 : 0));
                S.TG[lane] = t;
                ns = cz1 - cz0 + 1;
            }
        }
    }
    // ---- the z slices of the 32 tets, a lane per slice; the lane walks the
    // slice's rows and their points itself, with the tet's tables in registers
    const int Z = warp_prefix(ns, lane, S.pre1);
    __syncwarp();
    for (int i = 0; i < ns; ++i)
        S.own1[S.pre1[lane] + i] = (unsigned char)lane;
    __syncwarp();
    for (int zb = 0; zb < Z; zb += 32)
    {
        const int it = zb + lane;
        if (it >= Z)
            continue;
        const int j = S.own1[it];
        const int4 I0 = S.I0[j], I1 = S.I1[j];
        const int zz = I1.x + (it - S.pre1[j]);
        const float4 A0 = S.P[0][j], A1 = S.P[1][j], A2 = S.P[2][j], A3 = S.P[3][j];
        const float pzf = zz * g.step[2] + g.gmin[2];
        // the y range of the tet's cross-section at z, from the edges that cross
        // the plane, widened by a rounding margin (an extra row is only visited,
        // a dropped row would lose points)
        int y0 = 0, y1 = -1;
        {
            const float a[4][3] = { { A0.x, A0.y, A0.z }, { A1.x, A1.y, A1.z }, { A2.x, A2.y, A2.z },
                                    { A3.x, A3.y, A3.z } };
            float ylo = FLT_MAX, yhi = -FLT_MAX;
#pragma unroll
            for (int e = 0; e < 6; ++e)
            {
                const int u = e < 3 ? 0 : (e < 5 ? 1 : 2);
                const int v = e < 3 ? e + 1 : (e < 5 ? e - 1 : 3);
                const float za = a[u][2], zb2 = a[v][2];
                if (pzf < fminf(za, zb2) || pzf > fmaxf(za, zb2))
                    continue;
                float y0f, y1f;
                if (za == zb2)
                {
                    y0f = a[u][1];
                    y1f = a[v][1];
                }
                else
                {
                    const float tt = fminf(fmaxf((pzf - za) * S.IDZ[e][j], 0.0f), 1.0f);
                    y0f = y1f = fmaf(tt, a[v][1] - a[u][1], a[u][1]);
                }
                ylo = fminf(ylo, fminf(y0f, y1f));
                yhi = fmaxf(yhi, fmaxf(y0f, y1f));
            }
            if (ylo <= yhi)
            {
                const float ginv = g.inv_step[1], gmn = g.gmin[1];
                const float my = 64.0f * EPS32 * (fmaxf(fabsf(ylo), fabsf(yhi)) + A3.w - A2.w);
                const float f0 = (ylo - my - gmn) * ginv;
                const float f1 = (yhi + my - gmn) * ginv;
                const float mm = 1e-3f + 8.0f * EPS32 *
                    ((fabsf(gmn) + fmaxf(fabsf(ylo), fabsf(yhi))) * ginv + fmaxf(fabsf(f0), fabsf(f1)));
                y0 = max(I0.z, (int)ceilf(fmaxf(f0 - mm, (float)(I0.z - 1))));
                y1 = min(I0.w, (int)floorf(fminf(f1 + mm, (float)(I0.w + 1))));
            }
        }
        if (y0 > y1)
            continue;
        const float4 XA = S.XA[j], XB = S.XB[j], XG = S.XG[j];
        const T4 c0 = S.C[0][j], c1 = S.C[1][j], c2 = S.C[2][j], c3 = S.C[3][j];
        const int m = I1.w & 0xff;
        const bool fix = F32 && ((I1.w >> 9) & 1);
        const float fdz = (float)(zz - I1.z);
        const float ginv0 = g.inv_step[0], gmn0 = g.gmin[0];
        for (int yy = y0; yy <= y1; ++yy)
        {
            cn.rows++;
            // the row's x range from the four faces' bounds, then the grid
            // indices inside it widened by mg grid steps (see k_raster)
            float xmin = A0.w, xmax = A1.w;
            const float fdy = (float)(yy - I1.y);
#pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                const float bnd = fmaf(comp4<float>(XG, k), fdz, fmaf(comp4<float>(XB, k), fdy, comp4<float>(XA, k)));
                if ((m >> (4 + k)) & 1) continue;
                if ((m >> k) & 1) xmin = fmaxf(xmin, bnd);
                else xmax = fminf(xmax, bnd);
            }
            if (xmin > xmax)
                continue;
            const float f0 = (xmin - gmn0) * ginv0;
            const float f1 = (xmax - gmn0) * ginv0;
            const float mg = 1e-3f + 8.0f * EPS32 * ((fabsf(gmn0) + fmaxf(fabsf(xmin), fabsf(xmax))) * ginv0 +
                                                     fmaxf(fabsf(f0), fabsf(f1)));
            const int i0 = max(I0.x, (int)ceilf(fmaxf(f0 - mg, (float)(I0.x - 1))));
            const int i1 = min(I0.y, (int)floorf(fminf(f1 + mg, (float)(I0.y + 1))));
            if (i0 > i1)
                continue;
            const float pyf = yy * g.step[1] + g.gmin[1];
            T RN[4];
            {
                const T q1y = (T)pyf - (T)A1.y, q1z = (T)pzf - (T)A1.z;
                const T q0y = (T)pyf - (T)A0.y, q0z = (T)pzf - (T)A0.z;
                RN[0] = Real<T>::fma_(c0.y, q1y, c0.z * q1z);
                RN[1] = Real<T>::fma_(c1.y, q0y, c1.z * q0z);
                RN[2] = Real<T>::fma_(c2.y, q0y, c2.z * q0z);
                RN[3] = Real<T>::fma_(c3.y, q0y, c3.z * q0z);
            }
            float* trow = tile + ((zz - r0[2]) << (SX + SY)) + ((yy - r0[1]) << SX) - r0[0];
            for (int xx = i0; xx <= i1; ++xx)
            {
                cn.cand++;
                const float pxf = xx * g.step[0] + gmn0;
                const T px = pxf;
                T N[4];
                N[0] = Real<T>::fma_(c0.x, px - (T)A1.x, RN[0]);
                const T qx = px - (T)A0.x;
                N[1] = Real<T>::fma_(c1.x, qx, RN[1]);
                N[2] = Real<T>::fma_(c2.x, qx, RN[2]);
                N[3] = Real<T>::fma_(c3.x, qx, RN[3]);
                const T Bk[4] = { c0.w, c1.w, c2.w, c3.w };
                bool in = true, out = false;
                unsigned open = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                {
                    const bool ik = N[k] > Bk[k];
                    in = in && ik;
                    out = out || (N[k] < -Bk[k]);
                    open |= (ik ? 0u : 1u) << k;
                }
                if (out)
                    continue;
                if (!in)
                {
                    cn.exact++;
                    const int sgn = (I1.w >> 8) & 1 ? 1 : -1;
                    if (!inside_exact(A0.x, A0.y, A0.z, A1.x, A1.y, A1.z, A2.x, A2.y, A2.z, A3.x, A3.y, A3.z, pxf,
                                      pyf, pzf, sgn, open))
                        continue;
                }
                float f;
                if (fix)
                    f = (float)(S.F[0][j] + ((double)pxf - (double)A0.x) * S.F[1][j] +
                                ((double)pyf - (double)A0.y) * S.F[2][j] + ((double)pzf - (double)A0.z) * S.F[3][j]);
                else
                {
                    const T4 W4 = S.W[j];
                    f = (float)Real<T>::fma_(N[0], W4.x, Real<T>::fma_(N[1], W4.y, Real<T>::fma_(N[2], W4.z, N[3] * W4.w)));
                }
                trow[xx] = f;
                if (owner)
                    owner[g.off + ((size_t)zz * g.n[1] + yy) * g.n[0] + xx] = S.TG[j] - bd.t_off;
                cn.assigned++;
            }
        }
    }
    __syncwarp();
}

template <typename T, int SX, int SY, int SZ, int NW>
__global__ void __launch_bounds__(NW * 32, 2)
k_raster_bricks(const BlockDesc* blocks, int nb, int seg, int bb0, int bb1, const int* cnt, const int* off,
                const int* item_off, const int* seg_items, int* item_counter, const int* pairs, const float4* pos,
                const int4* tv, const float* rho32, const double* rho64, GridDesc g, float* grid, int* owner,
                int fixup, Status* st)
{
    constexpr int BX = 1 << SX, BY = 1 << SY, BZ = 1 << SZ, BP = BX * BY * BZ;
    extern __shared__ __align__(32) unsigned char brick_smem[];
    float* tile = (float*)brick_smem;
    BrickWarp<T, SX, SY, SZ>* W = (BrickWarp<T, SX, SY, SZ>*)(brick_smem + BP * sizeof(float));
    __shared__ int s_item;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    BrickCounts cn;
    const int total = seg_items[seg];
    for (;;)
    {
        if (threadIdx.x == 0)
            s_item = atomicAdd(item_counter, 1);
        __syncthreads();
        const int item = s_item;
        if (item >= total)
            break;
        // the item's brick: the last b with item_off[b] <= item
        int lo = bb0, hi = bb1 - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&item_off[mid]) <= item) lo = mid; else hi = mid - 1;
        }
        const int b = lo;
        const int ib = __ldg(&item_off[b]);
        const int nitems = (b + 1 < bb1 ? __ldg(&item_off[b + 1]) : total) - ib;
        const bool split = nitems > 1;
        const int chunk = item - ib;
        const int c0 = __ldg(&off[b]) + chunk * BRICK_CHUNK;
        const int c1 = __ldg(&off[b]) + min(__ldg(&cnt[b]), (chunk + 1) * BRICK_CHUNK);
        const BlockDesc& bd = blocks[brick_block(blocks, nb, b)];
        int r0[3], r1[3];
        brick_region(bd, b, SX, SY, SZ, r0, r1);
        const float init = split ? __uint_as_float(BRICK_UNSET) : 0.0f;
        for (int i = threadIdx.x; i < BP; i += NW * 32)
            tile[i] = init;
        __syncthreads();
        for (int base = c0 + wid * 32; base < c1; base += NW * 32)
            brick_batch<T, SX, SY, SZ>(W[wid], tile, r0, r1, base, min(base + 32, c1), pairs, bd, pos, tv, rho32,
                                       rho64, g, owner, fixup, cn);
        __syncthreads();
        const int nx = r1[0] - r0[0] + 1, ny = r1[1] - r0[1] + 1, nz = r1[2] - r0[2] + 1;
        for (int i = threadIdx.x; i < BP; i += NW * 32)
        {
            const int x = i & (BX - 1), y = (i >> SX) & (BY - 1), z = i >> (SX + SY);
            if (x < nx && y < ny && z < nz)
            {
                const float v = tile[i];
                if (!split || __float_as_uint(v) != BRICK_UNSET)
                    grid[bd.grid.off + ((size_t)(r0[2] + z) * bd.grid.n[1] + (r0[1] + y)) * bd.grid.n[0] +
                         (r0[0] + x)] = v;
            }
        }
        (void)BZ;
    }
    unsigned long long v[5] = { cn.rows, cn.cand, cn.exact, cn.assigned, cn.fix };
#pragma unroll
    for (int k = 0; k < 5; ++k)
        for (int o = 16; o > 0; o >>= 1)
            v[k] += __shfl_xor_sync(FULL, v[k], o);
    if (lane == 0)
    {
        if (v[0]) atomicAdd(&st->rows, v[0]);
        if (v[1]) atomicAdd(&st->candidates, v[1]);
        if (v[2]) atomicAdd(&st->exact_tests, v[2]);
        if (v[3]) atomicAdd(&st->assigned, v[3]);
        if (v[4]) atomicAdd(&st->fp64_tets, v[4]);
    }
}

// brick shapes the autotuner tries: log2 of BX, BY, BZ, and warps per CTA
struct BrickVariant { int sx, sy, sz, nw; };
static const BrickVariant kBrickVariants[] = { { 5, 4, 4, 8 }, { 5, 3, 4, 8 }, { 5, 4, 3, 8 }, { 5, 3, 3, 8 } };
constexpr int N_BRICK_VARIANTS = sizeof(kBrickVariants) / sizeof(kBrickVariants[0]);

int brick_variants() { return N_BRICK_VARIANTS; }

void brick_shape(int variant, int* sx, int* sy, int* sz)
{
    const BrickVariant& v = kBrickVariants[variant < 0 || variant >= N_BRICK_VARIANTS ? 0 : variant];
    *sx = v.sx;
    *sy = v.sy;
    *sz = v.sz;
}

void launch_bin_reset(const BrickBins& bins, int seg, int bb0, int bb1, cudaStream_t s)
{
    if (bb1 > bb0)
        cudaMemsetAsync(bins.cnt + bb0, 0, sizeof(int) * (size_t)(bb1 - bb0), s);
    cudaMemsetAsync(bins.counters + seg, 0, sizeof(int), s);
}

void launch_bin_place(int variant, const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1, int t0, int nt,
                      const float4* pos, const int4* tv, const GridDesc& g, const BrickBins& bins, float* grid,
                      Status* st, cudaStream_t s)
{
    int sx, sy, sz;
    brick_shape(variant, &sx, &sy, &sz);
    k_bin_scan<<<1, 1024, 0, s>>>(bb0, bb1, seg, bins.cnt, bins.off, bins.cur, bins.item_off, bins.seg_items,
                                  bins.pair_cursor, bins.pair_cap, st);
    if (nt > 0 && bb1 > bb0)
    {
        k_bin_scatter<<<grid_for(nt, 256, 8), 256, 0, s>>>(d_blocks, nb, t0, nt, pos, tv, g, sx, sy, sz, bins.cur,
                                                           bins.pairs, bins.pair_cap);
        k_zero_split<<<grid_for((long long)(bb1 - bb0) * 256, 256, 4), 256, 0, s>>>(
            d_blocks, nb, bb0, bb1, seg, bins.item_off, bins.seg_items, sx, sy, sz, g, grid);
    }
}

void launch_bin_bricks(int variant, const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1, int t0, int nt,
                       const float4* pos, const int4* tv, const GridDesc& g, const BrickBins& bins, float* grid,
                       Status* st, cudaStream_t s)
{
    int sx, sy, sz;
    brick_shape(variant, &sx, &sy, &sz);
    launch_bin_reset(bins, seg, bb0, bb1, s);
    if (nt > 0 && bb1 > bb0)
        k_bin_count<<<grid_for(nt, 256, 8), 256, 0, s>>>(d_blocks, nb, t0, nt, pos, tv, g, sx, sy, sz, bins.cnt);
    launch_bin_place(variant, d_blocks, nb, seg, bb0, bb1, t0, nt, pos, tv, g, bins, grid, st, s);
}

template <typename T, int SX, int SY, int SZ, int NW>
static void raster_bricks_t(const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1, long long nbricks,
                            const BrickBins& bins, const float4* pos, const int4* tv, const float* rho32,
                            const double* rho64, const GridDesc& g, float* grid, int* owner, int fixup, Status* st,
                            cudaStream_t s)
{
    constexpr int BP = 1 << (SX + SY + SZ);
    const size_t smem = BP * sizeof(float) + NW * sizeof(BrickWarp<T, SX, SY, SZ>);
    static bool attr = false;   // per process and instance; set before the first launch
    if (!attr)
    {
        cudaFuncSetAttribute(k_raster_bricks<T, SX, SY, SZ, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        attr = true;
    }
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raster_bricks<T, SX, SY, SZ, NW>, NW * 32, smem);
    long long nblk = (long long)sms * (per_sm > 0 ? per_sm : 1);
    // items >= bricks; more CTAs than items only exit
    if (nblk > nbricks + 64) nblk = nbricks + 64;
    if (nblk < 1) nblk = 1;
    k_raster_bricks<T, SX, SY, SZ, NW><<<(int)nblk, NW * 32, smem, s>>>(
        d_blocks, nb, seg, bb0, bb1, bins.cnt, bins.off, bins.item_off, bins.seg_items, bins.counters + seg,
        bins.pairs, pos, tv, rho32, rho64, g, grid, owner, fixup, st);
}

void launch_raster_bricks(int mode, int variant, const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1,
                          const BrickBins& bins, const float4* pos, const int4* tv, const float* rho32,
                          const double* rho64, const GridDesc& g, float* grid, int* owner, Status* st,
                          cudaStream_t s)
{
    if (bb1 <= bb0) return;
    const long long nbr = bb1 - bb0;
#define TG_BRICKS(SX, SY, SZ, NW)                                                                                   \
    do {                                                                                                            \
        if (mode == TESSGPU_MODE_FP64)                                                                              \
            raster_bricks_t<double, SX, SY, SZ, NW>(d_blocks, nb, seg, bb0, bb1, nbr, bins, pos, tv, rho32, rho64, \
                                                    g, grid, owner, 0, st, s);                                     \
        else                                                                                                        \
            raster_bricks_t<float, SX, SY, SZ, NW>(d_blocks, nb, seg, bb0, bb1, nbr, bins, pos, tv, rho32, rho64,  \
                                                   g, grid, owner, 1, st, s);                                      \
    } while (0)
    switch (variant)
    {
    case 1: TG_BRICKS(5, 3, 4, 8); break;
    case 2: TG_BRICKS(5, 4, 3, 8); break;
    case 3: TG_BRICKS(5, 3, 3, 8); break;
    default: TG_BRICKS(5, 4, 4, 8); break;
    }
#undef TG_BRICKS
}

void launch_star_volumes(int mode, int total, const float4* pos, const int4* tv, StarSum* W,
                         double scale, float tau, Status* st, cudaStream_t s)
{
    (void)tau;   // DTFE_TAU
    if (total <= 0) return;
    GridDesc g0;
    k_star_volumes<false><<<grid_for(total, 256, 8), 256, 0, s>>>(mode, 0, total, pos, tv, W, scale, st, nullptr, 0,
                                                                    g0, 0, 0, 0, nullptr);
}

void launch_star_bin(int mode, int variant, const BlockDesc* d_blocks, int nb, int t0, int nt, const float4* pos,
                     const int4* tv, StarSum* W, double scale, const GridDesc& g, int* cnt, Status* st,
                     cudaStream_t s)
{
    if (nt <= 0) return;
    int sx, sy, sz;
    brick_shape(variant, &sx, &sy, &sz);
    k_star_volumes<true><<<grid_for(nt, 256, 8), 256, 0, s>>>(mode, t0, nt, pos, tv, W, scale, st, d_blocks, nb, g,
                                                               sx, sy, sz, cnt);
}

}  // namespace tg
