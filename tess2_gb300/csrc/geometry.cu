// Reference-parity geometry and density kernels.
//
// This translation unit is compiled with -fmad=false: every FP32 expression
// below is evaluated with the rounding of the reference's own operation order
// (no a*b+c contraction), which is what makes circumcenters, Voronoi volumes
// and DENSE_TESS's cell membership bit-identical to src/tet.cpp,
// src/volume.cpp and src/dense.cpp.
//
// Layout and work decomposition:
//   k_ingest        one thread per tet: tet_t -> int4 verts / int4 neighbours, global indices
//   k_vert_to_tet   one thread per tet: atomicMax (the reference keeps the last tet)
//   k_circumcenters one thread per tet, float4 out
//   k_cells<MODE>   one warp per Voronoi cell:
//                     breadth-first walk of the vertex star in the reference's order
//                     (queue and neighbour list in shared memory, membership tests
//                     spread over the lanes), one lane per Voronoi face for the
//                     ring circulation, Newell normal and face area, and for
//                     DENSE_TESS the reference's scanline walk with PtInCell
//                     evaluated by all lanes at once (a lane per face, two ballots)
//   k_cic           one thread per particle (DENSE_CIC)
#include "kernels.h"
#include <algorithm>
#include <float.h>
#include <math.h>

namespace tg {

constexpr unsigned FULL = 0xffffffffu;
constexpr int MAX_STAR = TESSGPU_MAX_STAR;
constexpr int MAX_FACES = TESSGPU_MAX_FACES;
constexpr int MAX_LINK = TESSGPU_MAX_LINK;
constexpr int ROWCAP = 128;      // scanline rows kept in shared memory per cell
constexpr int CELL_WARPS = 4;

__device__ __forceinline__ int find_block_t(const BlockDesc* b, int nb, int t)
{
    int lo = 0, hi = nb - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (b[mid].t_off <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int find_block_c(const int* c_off, int nb, int c)
{
    int lo = 0, hi = nb - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (c_off[mid] <= c) lo = mid; else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int find_block_p(const BlockDesc* b, int nb, int p)
{
    int lo = 0, hi = nb - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (b[mid].p_off <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// ingest, vert_to_tet, circumcenters
// ---------------------------------------------------------------------------
__global__ void k_ingest(const int* const* raw, const BlockDesc* blocks, int nb, int total,
                         int4* tv, int4* tn, Status* st)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        int b = find_block_t(blocks, nb, t);
        const BlockDesc& B = blocks[b];
        const int* r = raw[b] + 8 * (size_t)(t - B.t_off);
        int v[4], n[4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            v[i] = r[i];
            n[i] = r[4 + i];
            if (v[i] < 0 || v[i] >= B.np || n[i] < -1 || n[i] >= B.nt)
            {
                fail(st, TESSGPU_ERR_BAD_MESH, t);
                v[i] = 0;
                n[i] = -1;
            }
            v[i] += B.p_off;
            n[i] = n[i] >= 0 ? n[i] + B.t_off : -1;
        }
        tv[t] = make_int4(v[0], v[1], v[2], v[3]);
        tn[t] = make_int4(n[0], n[1], n[2], n[3]);
    }
}

// fill_vert_to_tet (src/tess.cpp:767-787): the last tet that names a vertex wins
__global__ void k_vert_to_tet(const int4* tv, int total, int* v2t)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        int4 v = __ldg(&tv[t]);
        atomicMax(&v2t[v.x], t);
        atomicMax(&v2t[v.y], t);
        atomicMax(&v2t[v.z], t);
        atomicMax(&v2t[v.w], t);
    }
}

// caller-provided block-local vert_to_tet -> global tet indices
__global__ void k_v2t_from_local(const int* const* raw, const BlockDesc* blocks, int nb, int total,
                                 int* v2t, Status* st)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x)
    {
        int b = find_block_p(blocks, nb, p);
        const BlockDesc& B = blocks[b];
        int t = raw[b][p - B.p_off];
        if (t >= B.nt || t < -1)
        {
            fail(st, TESSGPU_ERR_BAD_MESH, p);
            t = -1;
        }
        v2t[p] = t >= 0 ? t + B.t_off : -1;
    }
}

// circumcenter (src/tet.cpp:37-66) with norm (:122), cross (:131) and
// determinant (:139) in the reference's operation order
__device__ __forceinline__ void circumcenter_ref(float3 a, float3 b, float3 c, float3 d, float* o)
{
    float t[3] = { a.x - d.x, a.y - d.y, a.z - d.z };
    float u[3] = { b.x - d.x, b.y - d.y, b.z - d.z };
    float v[3] = { c.x - d.x, c.y - d.y, c.z - d.z };
    float nt = t[0] * t[0]; nt += t[1] * t[1]; nt += t[2] * t[2];
    float nu = u[0] * u[0]; nu += u[1] * u[1]; nu += u[2] * u[2];
    float nv = v[0] * v[0]; nv += v[1] * v[1]; nv += v[2] * v[2];
    float det = t[0] * u[1] * v[2] + u[0] * v[1] * t[2] + v[0] * t[1] * u[2] -
                v[0] * u[1] * t[2] - u[0] * t[1] * v[2] - t[0] * v[1] * u[2];
    float den = 2 * det;
    float uv[3] = { u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0] };
    float vt[3] = { v[1] * t[2] - v[2] * t[1], v[2] * t[0] - v[0] * t[2], v[0] * t[1] - v[1] * t[0] };
    float tu[3] = { t[1] * u[2] - t[2] * u[1], t[2] * u[0] - t[0] * u[2], t[0] * u[1] - t[1] * u[0] };
    float dd[3] = { d.x, d.y, d.z };
#pragma unroll
    for (int i = 0; i < 3; ++i)
        o[i] = dd[i] + (nt * uv[i] + nu * vt[i] + nv * tu[i]) / den;
}

__global__ void k_circumcenters(const float4* pos, const int4* tv, int total, float4* cc)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        int4 v = __ldg(&tv[t]);
        float o[3];
        circumcenter_ref(ld3(pos, v.x), ld3(pos, v.y), ld3(pos, v.z), ld3(pos, v.w), o);
        cc[t] = make_float4(o[0], o[1], o[2], 0.0f);
    }
}

__global__ void k_circumcenters_f64(const float4* pos, const int4* tv, int total, double* cc)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        int4 vi = __ldg(&tv[t]);
        float3 a = ld3(pos, vi.x), b = ld3(pos, vi.y), c = ld3(pos, vi.z), d = ld3(pos, vi.w);
        double tt[3] = { (double)a.x - d.x, (double)a.y - d.y, (double)a.z - d.z };
        double u[3] = { (double)b.x - d.x, (double)b.y - d.y, (double)b.z - d.z };
        double v[3] = { (double)c.x - d.x, (double)c.y - d.y, (double)c.z - d.z };
        double nt = tt[0] * tt[0] + tt[1] * tt[1] + tt[2] * tt[2];
        double nu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        double nv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        double uv[3] = { u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0] };
        double vt[3] = { v[1] * tt[2] - v[2] * tt[1], v[2] * tt[0] - v[0] * tt[2], v[0] * tt[1] - v[1] * tt[0] };
        double tu[3] = { tt[1] * u[2] - tt[2] * u[1], tt[2] * u[0] - tt[0] * u[2], tt[0] * u[1] - tt[1] * u[0] };
        double den = 2 * (tt[0] * uv[0] + tt[1] * uv[1] + tt[2] * uv[2]);
        double dd[3] = { d.x, d.y, d.z };
        for (int i = 0; i < 3; ++i)
            cc[3 * (size_t)t + i] = dd[i] + (nt * uv[i] + nu * vt[i] + nv * tu[i]) / den;
    }
}

// ---------------------------------------------------------------------------
// per-cell kernel
// ---------------------------------------------------------------------------
struct __align__(16) WarpSmem
{
    int   q[MAX_STAR];          // breadth-first queue = visited tets
    int   fu[MAX_FACES];        // neighbour vertex u of face k
    int   fut[MAX_FACES];       // first tet (in walk order) that holds u
    float fa[3 * MAX_FACES];    // DENSE_TESS: face normals; VOLUME: per-face volume terms
    float fb[3 * MAX_FACES];    // DENSE_TESS: first face vertex; VOLUME: face areas
    int2  rows[ROWCAP];         // DENSE_TESS: (zi<<16|yi, min_xi<<16|max_xi) of nonempty scan rows
};

__device__ __forceinline__ bool warp_contains(const int* a, int n, int x, int lane)
{
    bool f = false;
    for (int j = lane; j < n; j += 32)
        f |= (a[j] == x);
    return __any_sync(FULL, f);
}

// circulate_start (src/tet.cpp:164-173)
__device__ __forceinline__ int circ_start(int4 vv, int x, int y)
{
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        int v = comp(vv, i);
        if (v != x && v != y)
            return i;
    }
    return -1;
}

// circulate_next (src/tet.cpp:185-215); *bad when the mesh is inconsistent
__device__ __forceinline__ int circ_next(const int4* tv, const int4* tn, int t, int wi, int x, int y,
                                         int* next_wi, bool* bad)
{
    int4 cur = __ldg(&tv[t]);
    int nv = -1;
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        int inv = comp(cur, i);
        if (nv == -1 && i != wi && inv != x && inv != y)
            nv = inv;
    }
    int nt = comp(__ldg(&tn[t]), wi);
    *next_wi = -1;
    if (nt < 0)
        return nt;
    int4 nx = __ldg(&tv[nt]);
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (*next_wi == -1 && comp(nx, i) == nv)
            *next_wi = i;
    if (*next_wi < 0 || wi < 0)
        *bad = true;
    return nt;
}

// PtInCell (src/dense.cpp:1172-1203): lane k tests faces k, k+32, ...; the
// reference's answer is "no two decided signs differ", which two ballots give
__device__ __forceinline__ bool warp_pt_in_cell(float px, float py, float pz, const WarpSmem& S, int nf,
                                                float eps, int lane)
{
    bool pos = false, neg = false;
    for (int k = lane; k < nf; k += 32)
    {
        const float* n = &S.fa[3 * k];
        const float* v = &S.fb[3 * k];
        float dist = n[0] * (px - v[0]) + n[1] * (py - v[1]) + n[2] * (pz - v[2]);
        if (fabsf(dist) > eps)
        {
            if (dist >= 0.0f) pos = true; else neg = true;
        }
    }
    unsigned bp = __ballot_sync(FULL, pos);
    unsigned bn = __ballot_sync(FULL, neg);
    return !(bp && bn);
}

__device__ __forceinline__ void idx2phys(const int* gi, float* p, const GridDesc& g)
{
    p[0] = gi[0] * g.step[0] + g.gmin[0];
    p[1] = gi[1] * g.step[1] + g.gmin[1];
    p[2] = gi[2] * g.step[2] + g.gmin[2];
}
__device__ __forceinline__ void phys2idx(const float* p, int* gi, const GridDesc& g)
{
    gi[0] = (int)((p[0] - g.gmin[0]) / g.step[0]);
    gi[1] = (int)((p[1] - g.gmin[1]) / g.step[1]);
    gi[2] = (int)((p[2] - g.gmin[2]) / g.step[2]);
}

// deposit of one grid point: the reference adds to its own block or to the
// neighbours whose bounds contain the point; on one device there is one
// global grid, so every grid point inside the data bounds is added once
__device__ __forceinline__ bool deposit(const int* gi, float inc, const GridDesc& g, float* grid)
{
    float p[3];
    idx2phys(gi, p, g);
    if (gi[0] < 0 || gi[1] < 0 || gi[2] < 0 || gi[0] >= g.n[0] || gi[1] >= g.n[1] || gi[2] >= g.n[2])
        return false;
    if (p[0] < g.dmin[0] || p[0] > g.dmax[0] || p[1] < g.dmin[1] || p[1] > g.dmax[1] ||
        p[2] < g.dmin[2] || p[2] > g.dmax[2])
        return false;
    // projected (src/dense.cpp:1047-1090 with the x-y plane): every z of a
    // block lands in that block's 2-D array, one layer per z range of blocks
    const size_t z = g.zlayer ? (size_t)g.zlayer[gi[2]] : (size_t)gi[2];
    atomicAdd(&grid[(z * g.n[1] + gi[1]) * g.n[0] + gi[0]], inc);
    return true;
}

// DistributeScalarCIC (src/dense.cpp:1787-1872)
__device__ void distribute_cic(const float* pt, float scalar, int* idx, float* w, const GridDesc& g)
{
    int mn[3];
    phys2idx(pt, mn, g);
    float tot_weight = 0.0f, v0 = 0.0f, weights[8];
    int n = 0;
    for (int z = 0; z < 2; ++z)
        for (int y = 0; y < 2; ++y)
            for (int x = 0; x < 2; ++x)
            {
                int ijk[3] = { mn[0] + x, mn[1] + y, mn[2] + z };
                idx[3 * n] = ijk[0]; idx[3 * n + 1] = ijk[1]; idx[3 * n + 2] = ijk[2];
                float gp[3], p[3] = { pt[0], pt[1], pt[2] };
                idx2phys(ijk, gp, g);
                if (fabsf(p[0] - gp[0]) < g.eps) p[0] += 2 * g.eps;
                if (fabsf(p[1] - gp[1]) < g.eps) p[1] += 2 * g.eps;
                if (fabsf(p[2] - gp[2]) < g.eps) p[2] += 2 * g.eps;
                float vol = fabsf((gp[0] - p[0]) * (gp[1] - p[1]) * (gp[2] - p[2]));
                if (v0 == 0.0f)
                    v0 = vol;
                float v = v0 / vol;
                weights[n] = v;
                tot_weight += v;
                n++;
            }
    for (int i = 0; i < 8; ++i)
        w[i] = (weights[i] / tot_weight) * scalar;
}

// PtInCell at up to four points at once: lane group q = lane / 8 takes point q
// (coordinate `axis` = cmin_pos[axis] + (start + (k0 + q) d) step[axis], the
// other two fixed), each lane every 8th face.  The same per-face arithmetic as
// warp_pt_in_cell, so each answer is the one a single probe gives.  Bit q of
// the result is the answer at point q (q < npts).  Out of line: the walks call it from three
// places, and one copy keeps the cell kernel's code smaller (see scanline).
__device__ __noinline__ unsigned warp_pt_in_cell4(int axis, float fixed_a, float fixed_b, int start, int d, int k0,
                                                     int npts, const float* cmin_pos, const GridDesc& g,
                                                     const WarpSmem& S, int nf, float eps, int lane)
{
    const int q = lane >> 3, sub = lane & 7;
    bool pos = false, neg = false;
    if (q < npts)
    {
        const int idx = start + (k0 + q) * d;
        const float c = cmin_pos[axis] + idx * g.step[axis];
        const float px = axis == 0 ? c : fixed_a;
        const float py = axis == 0 ? fixed_a : c;
        const float pz = fixed_b;
        for (int k = sub; k < nf; k += 8)
        {
            const float* n = &S.fa[3 * k];
            const float* v = &S.fb[3 * k];
            float dist = n[0] * (px - v[0]) + n[1] * (py - v[1]) + n[2] * (pz - v[2]);
            if (fabsf(dist) > eps)
            {
                if (dist >= 0.0f) pos = true; else neg = true;
            }
        }
    }
    const unsigned bp = __ballot_sync(FULL, pos), bn = __ballot_sync(FULL, neg);
    unsigned res = 0;
#pragma unroll
    for (int h = 0; h < 4; ++h)
    {
        const unsigned m = 0xffu << (8 * h);
        if (h < npts && !((bp & m) && (bn & m)))
            res |= 1u << h;
    }
    return res;
}

// The scanline's walks: the first k in [k0, kmax) whose PtInCell answer at
// position start + k d differs from c (kmax if none), probing four positions
// per round.  The walk itself is the reference's; only its probes run ahead.
__device__ __forceinline__ int warp_walk(int axis, float fixed_a, float fixed_b, int start, int d, bool c, int k0,
                                         int kmax, const float* cmin_pos, const GridDesc& g, const WarpSmem& S,
                                         int nf, float eps, int lane)
{
    for (int k = k0; k < kmax; k += 4)
    {
        const int n = min(4, kmax - k);
        const unsigned r = warp_pt_in_cell4(axis, fixed_a, fixed_b, start, d, k, n, cmin_pos, g, S, nf, eps, lane);
        const unsigned differ = (c ? ~r : r) & ((1u << n) - 1u);
        if (differ)
            return k + __ffs(differ) - 1;
    }
    return kmax;
}

// CellInteriorGridPts (src/dense.cpp:1475-1701).  All lanes run the same
// state machine; PtInCell is evaluated cooperatively.  With rec == true the
// nonempty rows go to S.rows (overflow is flagged); with rec == false every
// row is deposited at once with per-point increment inc.
// probes: the PtInCell calls the reference's scanline makes (its walks, one
// call per position, the first position of the left walk probed twice)
struct ScanOut { int tot; int nrows; bool overflow; int deposited; int probes; };

// out of line, like warp_pt_in_cell4: called twice per cell (count, then deposit), and one copy
// keeps the cell kernel's code small enough for the instruction cache (the two: 118 -> 91 ms at
// 2M -> 512^3)
__device__ __noinline__ ScanOut scanline(const int* cgp, const int* cmin_idx, const float* cmin_pos, WarpSmem& S, int nf,
                            const GridDesc& g, int lane, bool rec, float inc, float* grid)
{
    ScanOut o = { 0, 0, false, 0, 0 };
    float gp[3];
    int x_left = cgp[0] / 2, x_right = cgp[0] / 2, y_start = 0, first_x = 0;
    const float eps = g.eps;
    for (int zi = 0; zi < cgp[2]; zi++)
    {
        gp[2] = cmin_pos[2] + zi * g.step[2];
        bool border_found = false, z_step_done = false;
        for (int yi = y_start; yi < cgp[1]; yi++)
        {
            gp[1] = cmin_pos[1] + yi * g.step[1];
            gp[0] = cmin_pos[0] + x_left * g.step[0];
            gp[2] = cmin_pos[2] + zi * g.step[2];
            bool x_in_left = warp_pt_in_cell(gp[0], gp[1], gp[2], S, nf, eps, lane);
            bool x_in_right = x_in_left;
            int min_xi = cgp[0] - 1, max_xi = 0;
            // left walk: from x_left, leftwards while inside (x_in_left) or
            // rightwards while outside; x_left moves to the first point that
            // answers otherwise.  Position 0 is x_left, already probed.
            {
                const bool c = x_in_left;
                const int d = c ? -1 : 1;
                const int kmax = d < 0 ? x_left + 1 : cgp[0] - x_left;
                const int ks = warp_walk(0, gp[1], gp[2], x_left, d, c, 1, kmax, cmin_pos, g, S, nf, eps, lane);
                o.probes += 1 + (ks < kmax ? ks + 1 : ks);
                if (c && ks > 0)
                {
                    min_xi = min(min_xi, x_left - (ks - 1));
                    max_xi = max(max_xi, x_left);
                }
                if (ks < kmax)
                {
                    const int xs = x_left + ks * d;
                    if (!c)
                    {
                        min_xi = min(min_xi, xs);
                        max_xi = max(max_xi, xs);
                    }
                    x_left = xs;
                }
            }
            // right walk, mirrored, from x_right
            {
                const bool c = x_in_right;
                const int d = c ? 1 : -1;
                const int kmax = d > 0 ? cgp[0] - x_right : x_right + 1;
                const int ks = warp_walk(0, gp[1], gp[2], x_right, d, c, 0, kmax, cmin_pos, g, S, nf, eps, lane);
                o.probes += ks < kmax ? ks + 1 : ks;
                if (c && ks > 0)
                {
                    min_xi = min(min_xi, x_right);
                    max_xi = max(max_xi, x_right + (ks - 1));
                }
                if (ks < kmax)
                {
                    const int xs = x_right + ks * d;
                    if (!c)
                    {
                        min_xi = min(min_xi, xs);
                        max_xi = max(max_xi, xs);
                    }
                    x_right = xs;
                }
            }
            if (min_xi <= max_xi)
            {
                o.tot += max_xi - min_xi + 1;
                if (yi == y_start)
                    first_x = (min_xi + max_xi) / 2;
                if (rec)
                {
                    if (o.nrows < ROWCAP)
                    {
                        if (lane == 0)
                            S.rows[o.nrows] = make_int2((zi << 16) | yi, (min_xi << 16) | max_xi);
                        o.nrows++;
                    }
                    else
                        o.overflow = true;
                }
                else
                {
                    for (int xi = min_xi + lane; xi <= max_xi; xi += 32)
                    {
                        int gi[3] = { cmin_idx[0] + xi, cmin_idx[1] + yi, cmin_idx[2] + zi };
                        o.deposited += deposit(gi, inc, g, grid) ? 1 : 0;
                    }
                }
            }
            int first_y = y_start;
            if (min_xi <= max_xi && !border_found)
            {
                first_y = yi;
                border_found = true;
            }
            if (min_xi > max_xi && border_found)
                z_step_done = true;
            if ((yi == cgp[1] - 1 || z_step_done) && zi + 1 < cgp[2])
            {
                gp[2] = cmin_pos[2] + (zi + 1) * g.step[2];
                gp[0] = cmin_pos[0] + first_x * g.step[0];
                // from first_y down while inside, never below 1: y_start is the first
                // row that answers outside, or 0
                const int ks = warp_walk(1, gp[0], gp[2], first_y, -1, true, 0, first_y, cmin_pos, g, S, nf, eps, lane);
                o.probes += ks < first_y ? ks + 1 : ks;
                y_start = first_y - ks;
            }
            if (z_step_done)
                break;
        }
    }
    __syncwarp();
    return o;
}

template <int MODE>
__global__ void __launch_bounds__(CELL_WARPS * 32, 7)   // 7 blocks per SM: shared memory allows 7 as well
k_cells(const BlockDesc* blocks, const int* c_off, int nb, int total_cells, const float4* pos,
        const int4* tv, const int4* tn, const int* v2t, const float4* cc, const double* cc64, GridDesc g,
        float* grid, int* out_i, float* out_f, float* out_area, double* out_d, int* cell_counts, Status* st)
{
    __shared__ WarpSmem smem[CELL_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    WarpSmem& S = smem[w];
    double acc_mass = 0.0;
    unsigned long long acc_cells = 0, acc_probes = 0, acc_faces = 0;

    // persistent warps take cells in order from a counter: cells differ in
    // cost by orders of magnitude (a background cell's scanline against a
    // clump cell's CIC fallback), and a fixed share per warp left SMs idle
    // while the last blocks ran
    for (;;)
    {
        int c = 0;
        if (lane == 0)
            c = atomicAdd(&st->cell_next, 1);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= total_cells)
            break;
        const int b = find_block_c(c_off, nb, c);
        const int p_off = blocks[b].p_off;
        const int v = p_off + (c - c_off[b]);
        const int t0 = v2t[v];
        if (t0 < 0)
        {
            if (lane == 0)
            {
                if (MODE == CELL_COMPLETE) out_i[c] = -1;
                if (MODE == CELL_VOLUME) { out_f[c] = -1.0f; if (out_area) out_area[c] = -1.0f; }
                if (MODE == CELL_VOLUME_F64) out_d[c] = -1.0;
                if (MODE == CELL_DENSE_TESS && cell_counts) cell_counts[c] = -1;
            }
            continue;
        }

        // ---- star walk (neighbor_edges, src/tet.cpp:228-270; complete :337-378)
        int qn = 1, head = 0, nf = 0, err = 0;
        bool finite = true;
        if (lane == 0)
            S.q[0] = t0;
        __syncwarp();
        while (head < qn)
        {
            const int tt = S.q[head++];
            const int4 vv = __ldg(&tv[tt]);
            const int4 nn = __ldg(&tn[tt]);
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                const int u = comp(vv, i);
                if (u == v)
                    continue;
                if (MODE != CELL_COMPLETE)
                {
                    if (!warp_contains(S.fu, nf, u, lane))
                    {
                        if (nf >= MAX_FACES) { err = TESSGPU_ERR_FACE_OVERFLOW; break; }
                        if (lane == 0) { S.fu[nf] = u; S.fut[nf] = tt; }
                        __syncwarp();
                        nf++;
                    }
                }
                const int nx = comp(nn, i);
                if (nx == -1) { finite = false; break; }
                if (!warp_contains(S.q, qn, nx, lane))
                {
                    if (qn >= MAX_STAR) { err = TESSGPU_ERR_STAR_OVERFLOW; break; }
                    if (lane == 0) S.q[qn] = nx;
                    __syncwarp();
                    qn++;
                }
            }
            if (!finite || err)
                break;
        }
        __syncwarp();
        if (err)
        {
            if (lane == 0)
            {
                fail(st, err, c);
                if (MODE == CELL_COMPLETE) out_i[c] = -2;
                if (MODE == CELL_VOLUME) out_f[c] = -2.0f;
                if (MODE == CELL_VOLUME_F64) out_d[c] = -2.0;
                if (MODE == CELL_DENSE_TESS && cell_counts) cell_counts[c] = -2;
            }
            continue;
        }
        if (MODE == CELL_COMPLETE)
        {
            if (lane == 0) out_i[c] = finite ? 1 : 0;
            continue;
        }
        if (!finite)
        {
            if (lane == 0)
            {
                if (MODE == CELL_VOLUME) { out_f[c] = -1.0f; if (out_area) out_area[c] = -1.0f; }
                if (MODE == CELL_VOLUME_F64) out_d[c] = -1.0;
                if (MODE == CELL_DENSE_TESS && cell_counts) cell_counts[c] = -1;
            }
            continue;
        }

        const float3 site = ld3(pos, v);
        float bmin[3] = { FLT_MAX, FLT_MAX, FLT_MAX }, bmax[3] = { -FLT_MAX, -FLT_MAX, -FLT_MAX };
        bool bad = false, longring = false;
        double vol64_terms = 0.0;  // unused by FP32 modes

        // ---- one lane per face: ring around edge (v, u) starting at ut (fill_edge_link)
        for (int k = lane; k < nf; k += 32)
        {
            const int u = S.fu[k], ut = S.fut[k];
            int wi = circ_start(__ldg(&tv[ut]), v, u);
            int t = ut, len = 0;
            float area = 0.0f;
            double area64 = 0.0;
            float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
            float f0[3] = { 0, 0, 0 }, pr[3] = { 0, 0, 0 };
            double a64[3] = { 0, 0, 0 }, p64[3] = { 0, 0, 0 };
            while (true)
            {
                if (MODE == CELL_VOLUME_F64)
                {
                    double c3[3] = { cc64[3 * (size_t)t], cc64[3 * (size_t)t + 1], cc64[3 * (size_t)t + 2] };
                    if (len == 0) { a64[0] = c3[0]; a64[1] = c3[1]; a64[2] = c3[2]; }
                    else if (len >= 2)
                    {
                        double ab[3] = { p64[0] - a64[0], p64[1] - a64[1], p64[2] - a64[2] };
                        double ac[3] = { c3[0] - a64[0], c3[1] - a64[1], c3[2] - a64[2] };
                        double cp[3] = { ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2],
                                         ab[0] * ac[1] - ab[1] * ac[0] };
                        area64 += sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]) / 2;
                    }
                    p64[0] = c3[0]; p64[1] = c3[1]; p64[2] = c3[2];
                }
                else
                {
                    const float4 c4 = __ldg(&cc[t]);
                    const float c3[3] = { c4.x, c4.y, c4.z };
                    if (MODE == CELL_VOLUME)
                    {
                        // volume() fan, src/volume.cpp:25-47: a = ring[0]; (a, ring[i], ring[i+1])
                        if (len == 0) { f0[0] = c3[0]; f0[1] = c3[1]; f0[2] = c3[2]; }
                        else if (len >= 2)
                        {
                            float ab[3] = { pr[0] - f0[0], pr[1] - f0[1], pr[2] - f0[2] };
                            float ac[3] = { c3[0] - f0[0], c3[1] - f0[1], c3[2] - f0[2] };
                            float cp[3] = { ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2],
                                            ab[0] * ac[1] - ab[1] * ac[0] };
                            float nrm = cp[0] * cp[0];
                            nrm += cp[1] * cp[1];
                            nrm += cp[2] * cp[2];
                            area = (float)((double)area + sqrt((double)nrm) / 2);
                        }
                    }
                    else
                    {
                        // CellBounds (src/dense.cpp:690-718): bbox and Newell normal in ring order
                        if (len == 0) { f0[0] = c3[0]; f0[1] = c3[1]; f0[2] = c3[2]; }
                        else
                        {
                            n0 += (pr[1] - c3[1]) * (pr[2] + c3[2]);
                            n1 += (pr[2] - c3[2]) * (pr[0] + c3[0]);
                            n2 += (pr[0] - c3[0]) * (pr[1] + c3[1]);
                        }
#pragma unroll
                        for (int d = 0; d < 3; ++d)
                        {
                            bmin[d] = fminf(bmin[d], c3[d]);
                            bmax[d] = fmaxf(bmax[d], c3[d]);
                        }
                    }
                    pr[0] = c3[0]; pr[1] = c3[1]; pr[2] = c3[2];
                }
                len++;
                if (len > MAX_LINK) { longring = true; break; }
                int nwi;
                const int nt = circ_next(tv, tn, t, wi, v, u, &nwi, &bad);
                if (nt == ut || nt == -1)
                    break;
                if (bad)
                    break;
                t = nt;
                wi = nwi;
            }
            if (MODE == CELL_VOLUME)
            {
                const float3 pu = ld3(pos, u);
                float dn = (pu.x - site.x) * (pu.x - site.x);
                dn += (pu.y - site.y) * (pu.y - site.y);
                dn += (pu.z - site.z) * (pu.z - site.z);
                const float dist = sqrtf(dn);
                S.fa[k] = area * dist / 6;
                S.fb[k] = area;
            }
            else if (MODE == CELL_VOLUME_F64)
            {
                const float3 pu = ld3(pos, u);
                double e0 = (double)pu.x - site.x, e1 = (double)pu.y - site.y, e2 = (double)pu.z - site.z;
                const double term = area64 * sqrt(e0 * e0 + e1 * e1 + e2 * e2) / 6;
                reinterpret_cast<double*>(S.fa)[k] = term;   // MAX_FACES doubles fit in fa
            }
            else
            {
                // closing Newell term (last, first), NewellNormal src/dense.cpp:1139-1161
                n0 += (pr[1] - f0[1]) * (pr[2] + f0[2]);
                n1 += (pr[2] - f0[2]) * (pr[0] + f0[0]);
                n2 += (pr[0] - f0[0]) * (pr[1] + f0[1]);
                const float mag = sqrtf(n0 * n0 + n1 * n1 + n2 * n2);
                n0 /= mag; n1 /= mag; n2 /= mag;
                n0 = -n0; n1 = -n1; n2 = -n2;
                const float wv[3] = { f0[0] - site.x, f0[1] - site.y, f0[2] - site.z };
                if (wv[0] * n0 + wv[1] * n1 + wv[2] * n2 < 0.0f)
                {
                    n0 = -n0; n1 = -n1; n2 = -n2;
                }
                S.fa[3 * k] = n0; S.fa[3 * k + 1] = n1; S.fa[3 * k + 2] = n2;
                S.fb[3 * k] = f0[0]; S.fb[3 * k + 1] = f0[1]; S.fb[3 * k + 2] = f0[2];
            }
        }
        (void)vol64_terms;
        const bool any_bad = __any_sync(FULL, bad);
        const bool any_long = __any_sync(FULL, longring);
        __syncwarp();
        if (any_bad || any_long)
        {
            if (lane == 0)
            {
                fail(st, any_long ? TESSGPU_ERR_LINK_OVERFLOW : TESSGPU_ERR_BAD_MESH, c);
                if (MODE == CELL_VOLUME) out_f[c] = -2.0f;
                if (MODE == CELL_VOLUME_F64) out_d[c] = -2.0;
                if (MODE == CELL_DENSE_TESS && cell_counts) cell_counts[c] = -2;
            }
            continue;
        }

        if (MODE == CELL_VOLUME)
        {
            if (lane == 0)
            {
                float vol = 0.0f, ar = 0.0f;
                for (int k = 0; k < nf; ++k)
                {
                    vol += S.fa[k];
                    ar += S.fb[k];
                }
                out_f[c] = vol;
                if (out_area) out_area[c] = ar;
            }
            __syncwarp();
            continue;
        }
        if (MODE == CELL_VOLUME_F64)
        {
            if (lane == 0)
            {
                double vol = 0.0;
                for (int k = 0; k < nf; ++k)
                    vol += reinterpret_cast<const double*>(S.fa)[k];
                out_d[c] = vol;
            }
            __syncwarp();
            continue;
        }

        // ---- DENSE_TESS: cell bounds, CellGridPts (src/dense.cpp:1363-1458)
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
            for (int o = 16; o > 0; o >>= 1)
            {
                bmin[d] = fminf(bmin[d], __shfl_xor_sync(FULL, bmin[d], o));
                bmax[d] = fmaxf(bmax[d], __shfl_xor_sync(FULL, bmax[d], o));
            }
        }
        float epsv[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
            epsv[d] = (g.dmax[d] - g.dmin[d]) * 2.0f * FLT_EPSILON;
        if (bmin[0] < g.dmin[0] - epsv[0] || bmin[1] < g.dmin[1] - epsv[1] || bmin[2] < g.dmin[2] - epsv[2] ||
            bmax[0] > g.dmax[0] + epsv[0] || bmax[1] > g.dmax[1] + epsv[1] || bmax[2] > g.dmax[2] + epsv[2])
        {
            if (lane == 0 && cell_counts) cell_counts[c] = 0;
            continue;
        }
        int cmin_idx[3], cmax_idx[3], cgp[3];
        float cmin_pos[3];
        phys2idx(bmin, cmin_idx, g);
        phys2idx(bmax, cmax_idx, g);
        idx2phys(cmin_idx, cmin_pos, g);
        for (int d = 0; d < 3; ++d)
            cgp[d] = cmax_idx[d] - cmin_idx[d] + 1;

        ScanOut so = scanline(cgp, cmin_idx, cmin_pos, S, nf, g, lane, true, 0.0f, grid);
        acc_probes += (unsigned)so.probes;
        acc_faces += (unsigned long long)so.probes * nf;
        int ndep = 0, npts;
        double cell_mass = 0.0;
        if (so.tot > 0)
        {
            npts = so.tot;
            const double m = (double)(g.mass / (float)so.tot);   // src/dense.cpp:1692
            const float inc = (float)(m / (double)g.div);           // src/dense.cpp:290
            if (!so.overflow)
            {
                for (int r = 0; r < so.nrows; ++r)
                {
                    const int2 row = S.rows[r];
                    const int zi = row.x >> 16, yi = row.x & 0xffff;
                    const int lo = row.y >> 16, hi = row.y & 0xffff;
                    for (int xi = lo + lane; xi <= hi; xi += 32)
                    {
                        int gi[3] = { cmin_idx[0] + xi, cmin_idx[1] + yi, cmin_idx[2] + zi };
                        ndep += deposit(gi, inc, g, grid) ? 1 : 0;
                    }
                }
            }
            else
            {
                ScanOut s2 = scanline(cgp, cmin_idx, cmin_pos, S, nf, g, lane, false, inc, grid);
                ndep = s2.deposited;
            }
            for (int o = 16; o > 0; o >>= 1)
                ndep += __shfl_xor_sync(FULL, ndep, o);
            cell_mass = m * ndep;
        }
        else
        {
            // no interior grid point: CIC weights at the site (src/dense.cpp:1437-1455)
            npts = 8;
            int idx[24];
            float wgt[8];
            const float site3[3] = { site.x, site.y, site.z };
            distribute_cic(site3, g.mass, idx, wgt, g);
            if (lane < 8)
            {
                const float inc = (float)((double)wgt[lane] / (double)g.div);
                if (deposit(&idx[3 * lane], inc, g, grid))
                    cell_mass = (double)wgt[lane];
            }
            for (int o = 16; o > 0; o >>= 1)
                cell_mass += __shfl_xor_sync(FULL, cell_mass, o);
        }
        if (lane == 0)
        {
            if (cell_counts) cell_counts[c] = npts;
            acc_mass += cell_mass;
            acc_cells++;
        }
        __syncwarp();
    }
    if (MODE == CELL_DENSE_TESS && lane == 0 && acc_cells)
    {
        atomicAdd(&st->tot_mass, acc_mass);
        atomicAdd(&st->check_mass, acc_cells);
        atomicAdd(&st->probes, acc_probes);
        atomicAdd(&st->face_tests, acc_faces);
    }
}

// IterateCellsCic (src/dense.cpp:486-562): one thread per particle
__global__ void k_cic(const BlockDesc* blocks, const int* c_off, int nb, int total, const float4* pos,
                      GridDesc g, float* grid, Status* st)
{
    double acc = 0.0;
    unsigned long long cells = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x)
    {
        const int b = find_block_c(c_off, nb, c);
        const BlockDesc& B = blocks[b];
        const int v = B.p_off + (c - c_off[b]);
        const float3 p = ld3(pos, v);
        const float pt[3] = { p.x, p.y, p.z };
        int idx[24];
        float w[8];
        distribute_cic(pt, g.mass, idx, w, g);
        cells++;
        for (int i = 0; i < 8; ++i)
        {
            float gp[3];
            idx2phys(&idx[3 * i], gp, g);
            const bool own = gp[0] >= B.bmin[0] && gp[0] <= B.bmax[0] && gp[1] >= B.bmin[1] &&
                             gp[1] <= B.bmax[1] && gp[2] >= B.bmin[2] && gp[2] <= B.bmax[2];
            // own block: float quotient (src/dense.cpp:539); neighbour: double (src/dense.cpp:193)
            const float inc = own ? w[i] / g.div : (float)((double)w[i] / (double)g.div);
            if (deposit(&idx[3 * i], inc, g, grid))
                acc += (double)w[i];
        }
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        acc += __shfl_xor_sync(FULL, acc, o);
        cells += __shfl_xor_sync(FULL, cells, o);
    }
    if ((threadIdx.x & 31) == 0 && cells)
    {
        atomicAdd(&st->tot_mass, acc);
        atomicAdd(&st->check_mass, cells);
    }
}

// reorder_neighbors (src/tess-qhull.c:161-225): for vertex v = 0..3 in turn,
// the first still-unused neighbour (in the given order) that does not hold
// verts[v] becomes tets[v]; -1 when none does (a hull face).  Each tet only
// reads the other tets' vertices, which never change, so tets are independent.
__global__ void k_reorder_neighbors(int* tets, int total, Status* st)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        int* r = tets + 8 * (size_t)t;
        const int4 rv = reinterpret_cast<const int4*>(r)[0], rn = reinterpret_cast<const int4*>(r)[1];
        int v[4] = { rv.x, rv.y, rv.z, rv.w }, nb[4] = { rn.x, rn.y, rn.z, rn.w }, out[4];
        for (int i = 0; i < 4; ++i)
        {
            if (nb[i] >= total || nb[i] < -1)
            {
                fail(st, TESSGPU_ERR_BAD_MESH, t);
                nb[i] = -1;
            }
        }
        // the neighbours' vertices (never written here), all four loads in flight at once
        int4 cv[4];
#pragma unroll
        for (int n = 0; n < 4; ++n)
            cv[n] = nb[n] >= 0 ? __ldg(reinterpret_cast<const int4*>(tets + 8 * (size_t)nb[n]))
                               : make_int4(-1, -1, -1, -1);
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            out[i] = -1;
#pragma unroll
            for (int n = 0; n < 4; ++n)
            {
                if (out[i] >= 0 || nb[n] < 0)   // found already; -1 (hull) or -2 (taken)
                    continue;
                if (cv[n].x != v[i] && cv[n].y != v[i] && cv[n].z != v[i] && cv[n].w != v[i])
                {
                    out[i] = nb[n];
                    nb[n] = -2;
                }
            }
        }
        reinterpret_cast<int4*>(r)[1] = make_int4(out[0], out[1], out[2], out[3]);
    }
}

// ---------------------------------------------------------------------------
// incomplete_cells (src/tess.cpp:492-628)
// ---------------------------------------------------------------------------
// side_of_plane (src/tet.cpp:70-119): whether the box reaches the far side of
// the plane of the face opposite vertex j, as seen from vertex j; a degenerate
// face counts as reaching it.  dot (src/tet.cpp:22) and cross (:131) in the
// reference's order.
__device__ __forceinline__ bool side_of_plane_ref(const float* box, const float3* P, int j)
{
    int idx[4] = { 0, 1, 2, 3 };
    idx[j] = 3;
    idx[3] = j;
    const float3 x = P[idx[0]], y = P[idx[1]], z = P[idx[2]], p = P[idx[3]];
    const float u[3] = { y.x - x.x, y.y - x.y, y.z - x.z };
    const float v[3] = { z.x - x.x, z.y - x.y, z.z - x.z };
    const float n[3] = { u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0] };
    const float xx[3] = { x.x, x.y, x.z };
    const float pp[3] = { p.x, p.y, p.z };
    float res = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        res += n[i] * (pp[i] - xx[i]);
    const int sign = res > 0.0f ? 1 : (res < 0.0f ? -1 : 0);
    if (sign == 0)
        return true;
    res = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        if ((sign > 0) != (n[i] < 0.0f))
            res += n[i] * (box[i] - xx[i]);
        else
            res += n[i] * (box[3 + i] - xx[i]);
    }
    return (sign > 0) != (res > 0.0f);
}

// Euclidean distance from a point to a box (0 inside), as DIY's
// distance(bounds, point) computes it: per axis the excess beyond the box,
// squared and summed in float, then the square root
__device__ __forceinline__ float box_distance(const float* box, const float* c)
{
    float res = 0.0f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float diff = 0.0f, d;
        d = box[i] - c[i];
        if (d > diff) diff = d;
        d = c[i] - box[3 + i];
        if (d > diff) diff = d;
        res += diff * diff;
    }
    return sqrtf(res);
}

// One thread per tet.  Bit i of masks[c_off + p] is set when original particle
// p must go to link i of its block (the reference's to_send[p] sets):
//  - for a hull face opposite vertex j with a local vertex, every link whose
//    (wrapped) box reaches past the face gets the face's local vertices;
//  - unless the circumsphere lies deeper in the block than its radius on
//    every axis, every link whose box is within the radius of the
//    circumcenter gets the tet's local vertices.
// links6: wrapped link boxes (min xyz, max xyz), block b's at link_off[b]..link_off[b+1)
__global__ void k_incomplete_cells(const BlockDesc* blocks, int nb, int total, const float4* pos, const int4* tv,
                                   const int4* tn, const float* links6, const int* link_off, const int* first_link,
                                   unsigned long long* masks)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
    {
        const int b = find_block_t(blocks, nb, t);
        const BlockDesc& B = blocks[b];
        const int4 v4 = __ldg(&tv[t]);
        const int4 n4 = __ldg(&tn[t]);
        const int vl[4] = { v4.x - B.p_off, v4.y - B.p_off, v4.z - B.p_off, v4.w - B.p_off };
        const int nbr[4] = { n4.x, n4.y, n4.z, n4.w };
        bool local[4];
        bool any = false;
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            local[k] = vl[k] >= 0 && vl[k] < B.norig;
            any |= local[k];
        }
        if (!any)
            continue;
        const float3 P[4] = { ld3(pos, v4.x), ld3(pos, v4.y), ld3(pos, v4.z), ld3(pos, v4.w) };
        float c[3];
        circumcenter_ref(P[0], P[1], P[2], P[3], c);
        // distance (src/tet.cpp:146-153) from the circumcenter to vertex 0
        const float p0[3] = { P[0].x, P[0].y, P[0].z };
        float n2 = 0.0f;
#pragma unroll
        for (int i = 0; i < 3; ++i)
            n2 += (c[i] - p0[i]) * (c[i] - p0[i]);
        const float rad = sqrtf(n2);

        const int l0 = link_off[b] + first_link[b], l1 = link_off[b + 1];
        unsigned long long m[4] = { 0ull, 0ull, 0ull, 0ull };
        for (int j = 0; j < 4; ++j)
        {
            if (nbr[j] != -1)
                continue;
            bool face_local = false;
            for (int k = 0; k < 4; ++k)
                if (k != j && local[k]) face_local = true;
            if (!face_local)
                continue;
            for (int i = l0; i < l1; ++i)
                if (side_of_plane_ref(&links6[6 * i], P, j))
                {
                    const unsigned long long bit = 1ull << (i - link_off[b]);
                    for (int k = 0; k < 4; ++k)
                        if (k != j) m[k] |= bit;
                }
        }
        int j;
        for (j = 0; j < 3; ++j)
        {
            if (c[j] - B.bmin[j] <= rad) break;
            if (B.bmax[j] - c[j] <= rad) break;
        }
        if (j < 3)
            for (int i = l0; i < l1; ++i)
                if (box_distance(&links6[6 * i], c) <= rad)
                {
                    const unsigned long long bit = 1ull << (i - link_off[b]);
                    for (int k = 0; k < 4; ++k) m[k] |= bit;
                }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (local[k] && m[k])
                atomicOr(&masks[B.c_off + vl[k]], m[k]);
    }
}

// blocks without tets send every original particle to every link
// (src/tess.cpp:587-603); fill: per block, the mask of its links from first_link
__global__ void k_fill_masks(const BlockDesc* blocks, const int* c_off, int nb, int total_cells,
                             const unsigned long long* fill, unsigned long long* masks)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total_cells; c += gridDim.x * blockDim.x)
    {
        const int b = find_block_c(c_off, nb, c);
        if (blocks[b].nt == 0)
            masks[c] = fill[b];
    }
}

// enqueued (the reference's return value) per block: set bits of its masks
__global__ void k_count_sends(const int* c_off, int nb, int total_cells, const unsigned long long* masks,
                              unsigned long long* counts)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total_cells; c += gridDim.x * blockDim.x)
    {
        const int n = __popcll(masks[c]);
        if (n) atomicAdd(&counts[find_block_c(c_off, nb, c)], (unsigned long long)n);
    }
}

// z-projection of a 3-D grid into layers: layer l at (x, y) accumulates
// value * dz over its z indices [zs[l], zs[l+1]) in ascending z.  One thread
// per column (scalar) or per four columns (x extent a multiple of 4: 16-byte
// loads); consecutive threads read consecutive x, so every z step is
// coalesced, and the inner loop has no store, so its loads overlap.
__global__ void k_project_layers(const float* __restrict__ grid, long long area, const int* __restrict__ zs,
                                 int num_layers, float dz, float* __restrict__ layers)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < area;
         c += (long long)gridDim.x * blockDim.x)
        for (int l = 0; l < num_layers; ++l)
        {
            float acc = 0.0f;
            const int z1 = zs[l + 1];
#pragma unroll 16
            for (int z = zs[l]; z < z1; ++z)
                acc += __ldcs(&grid[z * area + c]) * dz;
            layers[l * area + c] = acc;
        }
}

__global__ void k_project_layers4(const float4* __restrict__ grid, long long area4, const int* __restrict__ zs,
                                  int num_layers, float dz, float4* __restrict__ layers)
{
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < area4;
         c += (long long)gridDim.x * blockDim.x)
        for (int l = 0; l < num_layers; ++l)
        {
            float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            const int z1 = zs[l + 1];
#pragma unroll 8
            for (int z = zs[l]; z < z1; ++z)
            {
                const float4 v = __ldcs(&grid[z * area4 + c]);
                acc.x += v.x * dz;
                acc.y += v.y * dz;
                acc.z += v.z * dz;
                acc.w += v.w * dz;
            }
            layers[l * area4 + c] = acc;
        }
}

// ProjectGrid (src/dense.cpp:881-1023): the z=0 block of each column adds the
// other blocks of the column in block order; here layer 0 adds layers 1.. in order
__global__ void k_sum_layers(const float* layers, int num_layers, long long area, float* out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < area;
         i += (long long)gridDim.x * blockDim.x)
    {
        float acc = layers[i];
        for (int l = 1; l < num_layers; ++l)
            acc += layers[l * area + i];
        out[i] = acc;
    }
}

__global__ void k_grid_max(const float* grid, long long n, float* out)
{
    float m = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, grid[i]);
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(FULL, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(reinterpret_cast<int*>(out), __float_as_int(m));   // non-negative floats order as ints
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int grid1d(long long n, int block, int sm_mult = 8)
{
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long need = (n + block - 1) / block;
    long long cap = (long long)sms * sm_mult;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

void launch_ingest(const int* const* d_raw, const BlockDesc* d_blocks, int nb, int total, int4* tv, int4* tn,
                   Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    k_ingest<<<grid1d(total, 256), 256, 0, s>>>(d_raw, d_blocks, nb, total, tv, tn, st);
}
void launch_vert_to_tet(const int4* tv, int total, int* v2t, cudaStream_t s)
{
    if (total <= 0) return;
    k_vert_to_tet<<<grid1d(total, 256), 256, 0, s>>>(tv, total, v2t);
}
void launch_v2t_from_local(const int* const* d_raw, const BlockDesc* d_blocks, int nb, int total, int* v2t,
                           Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    k_v2t_from_local<<<grid1d(total, 256), 256, 0, s>>>(d_raw, d_blocks, nb, total, v2t, st);
}
void launch_circumcenters(const float4* pos, const int4* tv, int total, float4* cc, cudaStream_t s)
{
    if (total <= 0) return;
    k_circumcenters<<<grid1d(total, 256), 256, 0, s>>>(pos, tv, total, cc);
}
void launch_circumcenters_f64(const float4* pos, const int4* tv, int total, double* cc, cudaStream_t s)
{
    if (total <= 0) return;
    k_circumcenters_f64<<<grid1d(total, 256), 256, 0, s>>>(pos, tv, total, cc);
}
void launch_cells(int mode, const BlockDesc* d_blocks, const int* d_c_off, int nb, int total, const float4* pos,
                  const int4* tv, const int4* tn, const int* v2t, const float4* cc, const double* cc64,
                  const GridDesc& g, float* grid, int* out_i, float* out_f, float* out_area, double* out_d,
                  int* cell_counts, Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    // one resident wave of persistent blocks (the kernel's occupancy per SM)
    int dev = 0, sms = 152, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int nt = CELL_WARPS * 32;
    switch (mode)
    {
    case CELL_COMPLETE: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cells<CELL_COMPLETE>, nt, 0); break;
    case CELL_VOLUME: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cells<CELL_VOLUME>, nt, 0); break;
    case CELL_VOLUME_F64:
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cells<CELL_VOLUME_F64>, nt, 0);
        break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cells<CELL_DENSE_TESS>, nt, 0); break;
    }
    const long long need = ((long long)total + CELL_WARPS - 1) / CELL_WARPS;
    const int nblk = (int)std::min<long long>(need, (long long)sms * std::max(per_sm, 1));
    cudaMemsetAsync(&st->cell_next, 0, sizeof(int), s);
    switch (mode)
    {
    case CELL_COMPLETE:
        k_cells<CELL_COMPLETE><<<nblk, nt, 0, s>>>(d_blocks, d_c_off, nb, total, pos, tv, tn, v2t, cc, cc64, g,
                                                   grid, out_i, out_f, out_area, out_d, cell_counts, st);
        break;
    case CELL_VOLUME:
        k_cells<CELL_VOLUME><<<nblk, nt, 0, s>>>(d_blocks, d_c_off, nb, total, pos, tv, tn, v2t, cc, cc64, g,
                                                 grid, out_i, out_f, out_area, out_d, cell_counts, st);
        break;
    case CELL_VOLUME_F64:
        k_cells<CELL_VOLUME_F64><<<nblk, nt, 0, s>>>(d_blocks, d_c_off, nb, total, pos, tv, tn, v2t, cc, cc64, g,
                                                     grid, out_i, out_f, out_area, out_d, cell_counts, st);
        break;
    default:
        k_cells<CELL_DENSE_TESS><<<nblk, nt, 0, s>>>(d_blocks, d_c_off, nb, total, pos, tv, tn, v2t, cc, cc64, g,
                                                     grid, out_i, out_f, out_area, out_d, cell_counts, st);
        break;
    }
}

void launch_cic(const BlockDesc* d_blocks, const int* d_c_off, int nb, int total, const float4* pos,
                const GridDesc& g, float* grid, Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    k_cic<<<grid1d(total, 256), 256, 0, s>>>(d_blocks, d_c_off, nb, total, pos, g, grid, st);
}

void launch_project_layers(const float* grid, int nx, int ny, const int* zs, int num_layers, float dz,
                           float* layers, cudaStream_t s)
{
    const long long area = (long long)nx * ny;
    if (area <= 0 || num_layers <= 0) return;
    if (nx % 4 == 0 && ((uintptr_t)grid & 15) == 0 && ((uintptr_t)layers & 15) == 0)
        k_project_layers4<<<grid1d(area / 4, 256, 16), 256, 0, s>>>((const float4*)grid, area / 4, zs, num_layers,
                                                                    dz, (float4*)layers);
    else
        k_project_layers<<<grid1d(area, 256, 16), 256, 0, s>>>(grid, area, zs, num_layers, dz, layers);
}

void launch_sum_layers(const float* layers, int num_layers, long long area, float* out, cudaStream_t s)
{
    if (area <= 0 || num_layers <= 0) return;
    k_sum_layers<<<grid1d(area, 256), 256, 0, s>>>(layers, num_layers, area, out);
}

void launch_incomplete_cells(const BlockDesc* blocks, const int* c_off, int nb, int total_tets, int total_cells,
                             const float4* pos, const int4* tv, const int4* tn, const float* links6,
                             const int* link_off, const int* first_link, const unsigned long long* fill,
                             unsigned long long* masks, unsigned long long* counts, cudaStream_t s)
{
    if (total_cells > 0)
        k_fill_masks<<<grid1d(total_cells, 256), 256, 0, s>>>(blocks, c_off, nb, total_cells, fill, masks);
    if (total_tets > 0)
        k_incomplete_cells<<<grid1d(total_tets, 256), 256, 0, s>>>(blocks, nb, total_tets, pos, tv, tn, links6,
                                                                   link_off, first_link, masks);
    if (total_cells > 0)
        k_count_sends<<<grid1d(total_cells, 256), 256, 0, s>>>(c_off, nb, total_cells, masks, counts);
}

void launch_reorder_neighbors(int* d_tets, int total, Status* st, cudaStream_t s)
{
    if (total <= 0) return;
    k_reorder_neighbors<<<grid1d(total, 256, 32), 256, 0, s>>>(d_tets, total, st);
}

void launch_grid_max(const float* grid, long long n, float* d_max, cudaStream_t s)
{
    if (n <= 0) return;
    k_grid_max<<<grid1d(n, 256, 4), 256, 0, s>>>(grid, n, d_max);
}
}  // namespace tg
