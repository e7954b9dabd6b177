/*
 * CPU oracle for the tess2 post-Delaunay geometry + density path.
 * TEST INFRASTRUCTURE ONLY (see tess_oracle.h); build with -ffp-contract=off.
 *
 * Part 1 restates, operation for operation, the reference's FP32 code:
 *   src/tet.cpp      circumcenter :37-66, norm :122, cross :131, determinant :139,
 *                    distance :146, circulate_start/next :164-215,
 *                    neighbor_edges :228-270, complete :337-378, fill_edge_link :389-409
 *   src/volume.cpp   fill_circumcenters :6-11, volume :13-54
 *   src/tess.cpp     fill_vert_to_tet :767-787
 *   src/dense.cpp    dense :30-103, init_dense :106, est_dense :130, recvd_pts :166,
 *                    IterateCells :220-313, IterateCellsCic :486-562,
 *                    BlockGridParams :575-648, CellBounds :657-736, index :1047,
 *                    idx2phys :1098, phys2idx :1117, NewellNormal :1131, PtInCell :1172,
 *                    Global2LocalIdx :1210, DataBounds :1221, CellGridPts :1363,
 *                    CellInteriorGridPts :1475, GridStepParams :1712,
 *                    DistributeScalarCIC :1787
 * Mixed float/double expressions keep the reference's promotions (for
 * example the double sqrt in volume()'s face-area sum, src/volume.cpp:34,
 * where <cmath>'s global sqrt takes a double).
 *
 * Part 2 holds the FP64 references for the stages the reference does not have.
 */
#include "tess_oracle.h"
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>

/* ------------------------------------------------------------------ */
/* small growable arrays                                              */
/* ------------------------------------------------------------------ */
typedef struct { int* a; int n, cap; } ivec;

static void iv_push(ivec* v, int x)
{
    if (v->n == v->cap)
    {
        v->cap = v->cap ? 2 * v->cap : 64;
        v->a = (int*)realloc(v->a, sizeof(int) * (size_t)v->cap);
    }
    v->a[v->n++] = x;
}
static int iv_has(const ivec* v, int x)
{
    for (int i = 0; i < v->n; ++i)
        if (v->a[i] == x)
            return 1;
    return 0;
}
static void iv_free(ivec* v) { free(v->a); v->a = NULL; v->n = v->cap = 0; }

/* ------------------------------------------------------------------ */
/* part 1: reference-order FP32 geometry                              */
/* ------------------------------------------------------------------ */

/* src/tess.cpp:767-787: the last tet that names a vertex wins */
void orc_fill_vert_to_tet(int num_particles, const orc_tet* tets, int num_tets, int* vert_to_tet)
{
    for (int p = 0; p < num_particles; ++p)
        vert_to_tet[p] = -1;
    for (int t = 0; t < num_tets; ++t)
        for (int v = 0; v < 4; ++v)
            vert_to_tet[tets[t].verts[v]] = t;
}

static float norm3(const float* x)          /* |x|^2, src/tet.cpp:122 */
{
    float r = 0;
    for (int i = 0; i < 3; ++i)
        r += x[i] * x[i];
    return r;
}
static void cross3(float* r, const float* u, const float* v)   /* src/tet.cpp:131 */
{
    r[0] = u[1] * v[2] - u[2] * v[1];
    r[1] = u[2] * v[0] - u[0] * v[2];
    r[2] = u[0] * v[1] - u[1] * v[0];
}
static float det3f(const float* t, const float* u, const float* v)   /* src/tet.cpp:139 */
{
    return t[0] * u[1] * v[2] + u[0] * v[1] * t[2] + v[0] * t[1] * u[2] -
           v[0] * u[1] * t[2] - u[0] * t[1] * v[2] - t[0] * v[1] * u[2];
}
static float dist3(const float* u, const float* v)   /* src/tet.cpp:146 */
{
    float n = 0;
    for (int i = 0; i < 3; ++i)
        n += (u[i] - v[i]) * (u[i] - v[i]);
    return (float)sqrt((double)n);
}

/* src/tet.cpp:37-66 */
void orc_circumcenter(float* c, const orc_tet* tet, const float* particles)
{
    const float* a = &particles[3 * tet->verts[0]];
    const float* b = &particles[3 * tet->verts[1]];
    const float* cc = &particles[3 * tet->verts[2]];
    const float* d = &particles[3 * tet->verts[3]];
    float t[3], u[3], v[3];
    for (int i = 0; i < 3; ++i)
    {
        t[i] = a[i] - d[i];
        u[i] = b[i] - d[i];
        v[i] = cc[i] - d[i];
    }
    float norm_t = norm3(t), norm_u = norm3(u), norm_v = norm3(v);
    float den = 2 * det3f(t, u, v);
    float uv[3], vt[3], tu[3];
    cross3(uv, u, v);
    cross3(vt, v, t);
    cross3(tu, t, u);
    for (int i = 0; i < 3; ++i)
        c[i] = d[i] + (norm_t * uv[i] + norm_u * vt[i] + norm_v * tu[i]) / den;
}

void orc_fill_circumcenters(const float* particles, const orc_tet* tets, int num_tets, float* out)
{
    for (int i = 0; i < num_tets; ++i)
        orc_circumcenter(&out[3 * i], &tets[i], particles);
}

/* src/tet.cpp:337-378.  Breadth-first over the star of v across faces that
   contain v; 0 as soon as such a face is on the hull. */
int orc_complete(int v, const orc_tet* tets, int num_tets, int t)
{
    (void)num_tets;
    ivec q = {0};
    iv_push(&q, t);
    int head = 0, result = 1;
    while (head < q.n && result)
    {
        int tt = q.a[head++];
        for (int i = 0; i < 4; ++i)
        {
            if (tets[tt].verts[i] == v)
                continue;
            int next = tets[tt].tets[i];
            if (next == -1) { result = 0; break; }
            if (!iv_has(&q, next))
                iv_push(&q, next);
        }
    }
    iv_free(&q);
    return result;
}

void orc_complete_all(const orc_tet* tets, int num_tets, const int* vert_to_tet, int n, int* out)
{
    for (int v = 0; v < n; ++v)
        out[v] = vert_to_tet[v] < 0 ? -1 : orc_complete(v, tets, num_tets, vert_to_tet[v]);
}

/* src/tet.cpp:228-270.  The reference pushes every neighbour and skips
   visited tets when it pops them; marking tets when they are first queued
   visits them in the same order, so the (u, ut) list is identical. */
static int neighbor_edges_iv(int v, const orc_tet* tets, int t, ivec* pairs, int* finite)
{
    ivec q = {0}, seen_u = {0};
    *finite = 1;
    pairs->n = 0;
    iv_push(&q, t);
    int head = 0;
    while (head < q.n)
    {
        int tt = q.a[head++];
        for (int i = 0; i < 4; ++i)
        {
            int u = tets[tt].verts[i];
            if (u == v)
                continue;
            if (!iv_has(&seen_u, u))
            {
                iv_push(&seen_u, u);
                iv_push(pairs, u);
                iv_push(pairs, tt);
            }
            int next = tets[tt].tets[i];
            if (next == -1)
                *finite = 0;
            else if (!iv_has(&q, next))
                iv_push(&q, next);
        }
    }
    iv_free(&q);
    iv_free(&seen_u);
    return pairs->n / 2;
}

int orc_neighbor_edges(int v, const orc_tet* tets, int t, int* pairs, int cap, int* finite)
{
    ivec p = {0};
    int n = neighbor_edges_iv(v, tets, t, &p, finite);
    if (n <= cap)
        memcpy(pairs, p.a, sizeof(int) * 2 * (size_t)n);
    iv_free(&p);
    return n <= cap ? n : -n - 1;
}

/* src/tet.cpp:164-173 */
static int circulate_start(const orc_tet* tets, int t, int x, int y)
{
    for (int i = 0; i < 4; ++i)
    {
        int v = tets[t].verts[i];
        if (v != x && v != y)
            return i;
    }
    return -1;
}

/* src/tet.cpp:185-215 */
static void circulate_next(int* next_t, int* next_v, const orc_tet* tets, int t, int v, int x, int y)
{
    const orc_tet* cur = tets + t;
    int nv = -1;
    for (int i = 0; i < 4; ++i)
    {
        int inv = cur->verts[i];
        if (i != v && inv != x && inv != y) { nv = inv; break; }
    }
    *next_t = cur->tets[v];
    *next_v = -1;
    if (*next_t < 0)
        return;
    const orc_tet* next = tets + *next_t;
    for (int i = 0; i < 4; ++i)
        if (next->verts[i] == nv) { *next_v = i; return; }
}

/* src/tet.cpp:389-409 */
static void fill_edge_link_iv(int v, int u, int ut, const orc_tet* tets, ivec* link)
{
    link->n = 0;
    int wi = circulate_start(tets, ut, v, u);
    int t = ut;
    for (;;)
    {
        iv_push(link, t);
        int next_t, next_wi;
        circulate_next(&next_t, &next_wi, tets, t, wi, v, u);
        if (next_t == ut || next_t == -1)
            break;
        t = next_t;
        wi = next_wi;
    }
}

int orc_fill_edge_link(int v, int u, int ut, const orc_tet* tets, int* link, int cap)
{
    ivec l = {0};
    fill_edge_link_iv(v, u, ut, tets, &l);
    int n = l.n;
    if (n <= cap)
        memcpy(link, l.a, sizeof(int) * (size_t)n);
    iv_free(&l);
    return n <= cap ? n : -n - 1;
}

/* src/volume.cpp:13-54; *area_out (may be NULL) receives the sum of the
   cell's face areas in face order, in float (the quantity volume() weights
   by the edge lengths; tess2 itself does not return it) */
static float volume_area(int v, const int* vert_to_tet, const orc_tet* tets, const float* particles,
                         const float* cc, float* area_out)
{
    int vt = vert_to_tet[v];
    ivec nbrs = {0}, link = {0};
    int finite;
    int nf = neighbor_edges_iv(v, tets, vt, &nbrs, &finite);
    float vol = 0, area_sum = 0;
    if (area_out)
        *area_out = -1;
    if (!finite)
    {
        iv_free(&nbrs);
        return -1;
    }
    for (int k = 0; k < nf; ++k)
    {
        int u = nbrs.a[2 * k], ut = nbrs.a[2 * k + 1];
        fill_edge_link_iv(v, u, ut, tets, &link);
        float area = 0;
        int a = link.a[0];
        for (int i = 1; i < link.n - 1; ++i)
        {
            int b = link.a[i], c = link.a[i + 1];
            float ab[3], ac[3], cp[3];
            for (int j = 0; j < 3; ++j)
            {
                ab[j] = cc[3 * b + j] - cc[3 * a + j];
                ac[j] = cc[3 * c + j] - cc[3 * a + j];
            }
            cross3(cp, ab, ac);
            area = (float)((double)area + sqrt((double)norm3(cp)) / 2);
        }
        float dist = dist3(&particles[3 * u], &particles[3 * v]);
        vol += area * dist / 6;
        area_sum += area;
    }
    iv_free(&nbrs);
    iv_free(&link);
    if (area_out)
        *area_out = area_sum;
    return vol;
}

float orc_volume(int v, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                 const float* particles, const float* cc)
{
    (void)num_tets;
    return volume_area(v, vert_to_tet, tets, particles, cc, NULL);
}

void orc_volumes(int n, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                 const float* particles, float* out)
{
    float* cc = (float*)malloc(sizeof(float) * 3 * (size_t)(num_tets ? num_tets : 1));
    orc_fill_circumcenters(particles, tets, num_tets, cc);
    for (int v = 0; v < n; ++v)
        out[v] = vert_to_tet[v] < 0 ? -1.0f : orc_volume(v, vert_to_tet, tets, num_tets, particles, cc);
    free(cc);
}

/* volumes and total face areas of cells [0, n) (-1 for both where the cell
   is infinite or the vertex is in no tet) */
void orc_volume_areas(int n, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                      const float* particles, float* vol, float* area)
{
    float* cc = (float*)malloc(sizeof(float) * 3 * (size_t)(num_tets ? num_tets : 1));
    orc_fill_circumcenters(particles, tets, num_tets, cc);
    for (int v = 0; v < n; ++v)
    {
        if (vert_to_tet[v] < 0)
        {
            vol[v] = -1.0f;
            area[v] = -1.0f;
        }
        else
            vol[v] = volume_area(v, vert_to_tet, tets, particles, cc, &area[v]);
    }
    free(cc);
}

/* ------------------------------------------------------------------ */
/* part 1: density grid helpers                                       */
/* ------------------------------------------------------------------ */

/* src/dense.cpp:1098-1106 */
static void idx2phys(const int* gi, float* pos, const float* step, const float* gmin)
{
    pos[0] = gi[0] * step[0] + gmin[0];
    pos[1] = gi[1] * step[1] + gmin[1];
    pos[2] = gi[2] * step[2] + gmin[2];
}
/* src/dense.cpp:1117-1125 (float quotient truncated toward zero) */
static void phys2idx(const float* pos, int* gi, const float* step, const float* gmin)
{
    gi[0] = (int)((pos[0] - gmin[0]) / step[0]);
    gi[1] = (int)((pos[1] - gmin[1]) / step[1]);
    gi[2] = (int)((pos[2] - gmin[2]) / step[2]);
}

/* src/dense.cpp:1712-1767 */
void orc_grid_step_params(int num_given_bounds, const float* given_mins, const float* given_maxs,
                          const float* data_mins, const float* data_maxs,
                          float* grid_phys_mins, float* grid_phys_maxs, float* grid_step_size,
                          const int* glo_num_idx)
{
    float max_data_size = data_maxs[0] - data_mins[0];
    if (data_maxs[1] - data_mins[1] > max_data_size)
        max_data_size = data_maxs[1] - data_mins[1];
    if (data_maxs[2] - data_mins[2] > max_data_size)
        max_data_size = data_maxs[2] - data_mins[2];
    for (int i = 0; i < 3; ++i)
    {
        grid_phys_mins[i] = data_mins[i] - (max_data_size - (data_maxs[i] - data_mins[i])) / 2.0;
        grid_phys_maxs[i] = data_maxs[i] + (max_data_size - (data_maxs[i] - data_mins[i])) / 2.0;
    }
    for (int i = 0; i < 3 && i < num_given_bounds; ++i)
    {
        grid_phys_mins[i] = given_mins[i];
        grid_phys_maxs[i] = given_maxs[i];
    }
    for (int i = 0; i < 3; ++i)
        grid_step_size[i] = (grid_phys_maxs[i] - grid_phys_mins[i]) / (glo_num_idx[i] - 1);
}

/* src/dense.cpp:1221-1275 (single process: the all-reduce is the identity) */
void orc_data_bounds(int nblocks, const orc_block* blocks, float* data_mins, float* data_maxs)
{
    for (int i = 0; i < nblocks; ++i)
        for (int d = 0; d < 3; ++d)
        {
            if (i == 0 || blocks[i].bounds_min[d] < data_mins[d])
                data_mins[d] = blocks[i].bounds_min[d];
            if (i == 0 || blocks[i].bounds_max[d] > data_maxs[d])
                data_maxs[d] = blocks[i].bounds_max[d];
        }
}

/* src/dense.cpp:575-648 */
void orc_block_grid_params(const orc_block* b, const float* gmin, const float* step,
                           float eps, const float* data_mins, const float* data_maxs,
                           const int* glo_num_idx, int* min_idx, int* max_idx, int* num_idx)
{
    float pos[3];
    phys2idx(b->bounds_min, min_idx, step, gmin);
    idx2phys(min_idx, pos, step, gmin);
    for (int i = 0; i < 3; ++i)
        if (pos[i] < b->bounds_min[i])
            min_idx[i]++;
    phys2idx(b->bounds_max, max_idx, step, gmin);
    idx2phys(max_idx, pos, step, gmin);
    for (int i = 0; i < 3; ++i)
        if (pos[i] + step[i] <= b->bounds_max[i])
            max_idx[i]++;
    for (int i = 0; i < 3; ++i)
        if (fabs(data_mins[i] + max_idx[i] * step[i] - b->bounds_max[i]) < eps &&
            fabs(b->bounds_max[i] - data_maxs[i]) > step[i])
            max_idx[i]--;
    for (int i = 0; i < 3; ++i)
        if (fabs(b->bounds_min[i] - data_mins[i]) < step[i])
            min_idx[i] = 0;
    for (int i = 0; i < 3; ++i)
        if (fabs(b->bounds_max[i] - data_maxs[i]) < step[i])
            max_idx[i] = glo_num_idx[i] - 1;
    for (int i = 0; i < 3; ++i)
        num_idx[i] = max_idx[i] - min_idx[i] + 1;
}

/* src/dense.cpp:1131-1162 */
static void newell_normal(const float* verts, int nv, float* normal)
{
    normal[0] = 0.0f; normal[1] = 0.0f; normal[2] = 0.0f;
    for (int i = 0; i < nv; ++i)
    {
        int cur = i, next = (i + 1) % nv;
        normal[0] += (verts[3 * cur + 1] - verts[3 * next + 1]) * (verts[3 * cur + 2] + verts[3 * next + 2]);
        normal[1] += (verts[3 * cur + 2] - verts[3 * next + 2]) * (verts[3 * cur + 0] + verts[3 * next + 0]);
        normal[2] += (verts[3 * cur + 0] - verts[3 * next + 0]) * (verts[3 * cur + 1] + verts[3 * next + 1]);
    }
    float mag = (float)sqrt((double)(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]));
    normal[0] /= mag; normal[1] /= mag; normal[2] /= mag;
    normal[0] = -normal[0]; normal[1] = -normal[1]; normal[2] = -normal[2];
}

/* a cell polyhedron: per face its unit normal and its first vertex */
typedef struct
{
    int    nf;
    float* normals;    /* 3 * nf */
    float* v0;         /* 3 * nf, face_verts[k][0..2] */
    int    cap;
} cell_faces;

/* src/dense.cpp:1172-1203 */
static int pt_in_cell(const float* pt, const cell_faces* f, float eps)
{
    int old_sign = 0;
    for (int k = 0; k < f->nf; ++k)
    {
        const float* n = &f->normals[3 * k];
        const float* v = &f->v0[3 * k];
        float dist = n[0] * (pt[0] - v[0]) + n[1] * (pt[1] - v[1]) + n[2] * (pt[2] - v[2]);
        if (fabsf(dist) > eps)
        {
            int sign = (dist >= 0.0 ? 1 : -1);
            if (old_sign == 0)
                old_sign = sign;
            if (old_sign != sign)
                return 0;
        }
    }
    return 1;
}

/* src/dense.cpp:657-736.  The cell's circumcenters come from cc (the same
   function the reference recomputes per face vertex, so the same bits). */
static void cell_bounds(const orc_block* b, int cell, const float* cc, float* cmin, float* cmax,
                        cell_faces* f, ivec* nbrs, ivec* link, float** fv, int* fv_cap)
{
    int finite;
    int nf = neighbor_edges_iv(cell, b->tets, b->vert_to_tet[cell], nbrs, &finite);
    if (nf > f->cap)
    {
        f->cap = nf;
        f->normals = (float*)realloc(f->normals, sizeof(float) * 3 * (size_t)nf);
        f->v0 = (float*)realloc(f->v0, sizeof(float) * 3 * (size_t)nf);
    }
    f->nf = nf;
    const float* site = &b->particles[3 * cell];
    for (int k = 0; k < nf; ++k)
    {
        int u = nbrs->a[2 * k], ut = nbrs->a[2 * k + 1];
        fill_edge_link_iv(cell, u, ut, b->tets, link);
        if (3 * link->n > *fv_cap)
        {
            *fv_cap = 3 * link->n;
            *fv = (float*)realloc(*fv, sizeof(float) * (size_t)*fv_cap);
        }
        for (int l = 0; l < link->n; ++l)
        {
            const float* vv = &cc[3 * link->a[l]];
            (*fv)[3 * l] = vv[0]; (*fv)[3 * l + 1] = vv[1]; (*fv)[3 * l + 2] = vv[2];
            for (int d = 0; d < 3; ++d)
            {
                if ((k == 0 && l == 0) || vv[d] < cmin[d]) cmin[d] = vv[d];
                if ((k == 0 && l == 0) || vv[d] > cmax[d]) cmax[d] = vv[d];
            }
        }
        float n[3];
        newell_normal(*fv, link->n, n);
        float v[3];
        v[0] = (*fv)[0] - site[0];
        v[1] = (*fv)[1] - site[1];
        v[2] = (*fv)[2] - site[2];
        if (v[0] * n[0] + v[1] * n[1] + v[2] * n[2] < 0.0)
        {
            n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2];
        }
        for (int d = 0; d < 3; ++d)
        {
            f->normals[3 * k + d] = n[d];
            f->v0[3 * k + d] = (*fv)[d];
        }
    }
}

/* src/dense.cpp:1787-1872.  idx: 24 ints, w: 8 float masses */
static void distribute_cic(const float* pt, float scalar, int* idx, float* w,
                           const float* step, const float* gmin, float eps)
{
    int mn[3], mx[3];
    phys2idx(pt, mn, step, gmin);
    mx[0] = mn[0] + 1; mx[1] = mn[1] + 1; mx[2] = mn[2] + 1;
    float tot_weight = 0.0f, v0 = 0.0f, weights[8];
    int ijk[3], n = 0;
    for (ijk[2] = mn[2]; ijk[2] <= mx[2]; ijk[2]++)
        for (ijk[1] = mn[1]; ijk[1] <= mx[1]; ijk[1]++)
            for (ijk[0] = mn[0]; ijk[0] <= mx[0]; ijk[0]++)
            {
                idx[3 * n] = ijk[0]; idx[3 * n + 1] = ijk[1]; idx[3 * n + 2] = ijk[2];
                float gp[3], p[3] = { pt[0], pt[1], pt[2] };
                idx2phys(ijk, gp, step, gmin);
                if (fabsf(p[0] - gp[0]) < eps) p[0] += 2 * eps;
                if (fabsf(p[1] - gp[1]) < eps) p[1] += 2 * eps;
                if (fabsf(p[2] - gp[2]) < eps) p[2] += 2 * eps;
                float vol = fabsf((gp[0] - p[0]) * (gp[1] - p[1]) * (gp[2] - p[2]));
                if (v0 == 0.0)
                    v0 = vol;
                float v = v0 / vol;
                weights[n] = v;
                tot_weight += v;
                n++;
            }
    for (int i = 0; i < 8; ++i)
    {
        weights[i] /= tot_weight;
        w[i] = weights[i] * scalar;
    }
}

/* per-cell scratch reused across cells, like the reference's grid_pts/border */
typedef struct
{
    int*    gidx;     /* 3 per point */
    double* gmass;
    int*    border;
    int     alloc;    /* points allocated */
    cell_faces f;
    ivec    nbrs, link;
    float*  fv;
    int     fv_cap;
} cell_ws;

static void ws_free(cell_ws* w)
{
    free(w->gidx); free(w->gmass); free(w->border);
    free(w->f.normals); free(w->f.v0);
    iv_free(&w->nbrs); iv_free(&w->link);
    free(w->fv);
    memset(w, 0, sizeof(*w));
}

/* src/dense.cpp:1475-1701 */
static int cell_interior_grid_pts(const int* cgp, const int* cmin_idx, const float* cmin_pos,
                                  cell_ws* w, const float* step, float eps, float mass)
{
    int num_grid_pts = 0, tot_num_grid_pts = 0;
    float gp[3];
    int x_left = cgp[0] / 2, x_right = cgp[0] / 2, y_start = 0;
    int x_in_left, x_in_right, min_xi, max_xi, border_found, z_step_done;
    int xi, yi, zi, yj, first_x = 0;
    int* border = w->border;
    const cell_faces* f = &w->f;

    for (zi = 0; zi < cgp[2]; zi++)
    {
        gp[2] = cmin_pos[2] + zi * step[2];
        border_found = 0;
        z_step_done = 0;
        for (yj = 0; yj < y_start; yj++)
        {
            border[2 * (zi * cgp[1] + yj)] = 1;
            border[2 * (zi * cgp[1] + yj) + 1] = 0;
        }
        for (yi = y_start; yi < cgp[1]; yi++)
        {
            gp[1] = cmin_pos[1] + yi * step[1];
            gp[0] = cmin_pos[0] + x_left * step[0];
            gp[1] = cmin_pos[1] + yi * step[1];
            gp[2] = cmin_pos[2] + zi * step[2];
            x_in_left = x_in_right = pt_in_cell(gp, f, eps);
            min_xi = cgp[0] - 1;
            max_xi = 0;

            for (xi = x_left; xi >= 0 && xi < cgp[0];)
            {
                gp[0] = cmin_pos[0] + xi * step[0];
                if (pt_in_cell(gp, f, eps))
                {
                    if (xi < min_xi) min_xi = xi;
                    if (xi > max_xi) max_xi = xi;
                    if (x_in_left)
                        xi--;
                    else
                    {
                        x_left = xi;
                        break;
                    }
                }
                else
                {
                    if (!x_in_left)
                        xi++;
                    else
                    {
                        x_left = xi;
                        break;
                    }
                }
            }
            for (xi = x_right; xi >= 0 && xi < cgp[0];)
            {
                gp[0] = cmin_pos[0] + xi * step[0];
                if (pt_in_cell(gp, f, eps))
                {
                    if (xi < min_xi) min_xi = xi;
                    if (xi > max_xi) max_xi = xi;
                    if (x_in_right)
                        xi++;
                    else
                    {
                        x_right = xi;
                        break;
                    }
                }
                else
                {
                    if (!x_in_right)
                        xi--;
                    else
                    {
                        x_right = xi;
                        break;
                    }
                }
            }
            border[2 * (zi * cgp[1] + yi)] = min_xi;
            border[2 * (zi * cgp[1] + yi) + 1] = max_xi;

            if (min_xi <= max_xi)
            {
                tot_num_grid_pts += (max_xi - min_xi + 1);
                if (yi == y_start)
                    first_x = (min_xi + max_xi) / 2;
            }
            int first_y = y_start;
            if (min_xi <= max_xi && !border_found)
            {
                first_y = yi;
                border_found = 1;
            }
            if (min_xi > max_xi && border_found)
                z_step_done = 1;
            if ((yi == cgp[1] - 1 || z_step_done) && zi + 1 < cgp[2])
            {
                gp[2] = cmin_pos[2] + (zi + 1) * step[2];
                gp[0] = cmin_pos[0] + first_x * step[0];
                for (yj = first_y; yj > 0; yj--)
                {
                    gp[1] = cmin_pos[1] + yj * step[1];
                    if (!pt_in_cell(gp, f, eps))
                        break;
                }
                y_start = yj;
            }
            if (z_step_done)
            {
                for (yj = yi + 1; yj < cgp[1]; yj++)
                {
                    border[2 * (zi * cgp[1] + yj)] = 1;
                    border[2 * (zi * cgp[1] + yj) + 1] = 0;
                }
                break;
            }
        }
    }

    num_grid_pts = 0;
    for (zi = 0; zi < cgp[2]; zi++)
        for (yi = 0; yi < cgp[1]; yi++)
        {
            min_xi = border[2 * (zi * cgp[1] + yi)];
            max_xi = border[2 * (zi * cgp[1] + yi) + 1];
            for (xi = min_xi; xi <= max_xi; xi++)
            {
                w->gidx[3 * num_grid_pts] = cmin_idx[0] + xi;
                w->gidx[3 * num_grid_pts + 1] = cmin_idx[1] + yi;
                w->gidx[3 * num_grid_pts + 2] = cmin_idx[2] + zi;
                w->gmass[num_grid_pts] = (double)(mass / (float)tot_num_grid_pts);
                num_grid_pts++;
            }
        }
    return num_grid_pts;
}

/* src/dense.cpp:1363-1458 */
static int cell_grid_pts(const float* cmins, const float* cmaxs, cell_ws* w,
                         const float* data_mins, const float* data_maxs,
                         const float* gmin, const float* step, float mass, float eps, const float* site)
{
    float epsilon[3];
    for (int i = 0; i < 3; ++i)
        epsilon[i] = (data_maxs[i] - data_mins[i]) * 2.0f * FLT_EPSILON;
    if (cmins[0] < data_mins[0] - epsilon[0] || cmins[1] < data_mins[1] - epsilon[1] ||
        cmins[2] < data_mins[2] - epsilon[2] || cmaxs[0] > data_maxs[0] + epsilon[0] ||
        cmaxs[1] > data_maxs[1] + epsilon[1] || cmaxs[2] > data_maxs[2] + epsilon[2])
        return 0;

    int cmin_idx[3], cmax_idx[3], cgp[3];
    float cmin_pos[3];
    phys2idx(cmins, cmin_idx, step, gmin);
    phys2idx(cmaxs, cmax_idx, step, gmin);
    idx2phys(cmin_idx, cmin_pos, step, gmin);
    for (int i = 0; i < 3; ++i)
        cgp[i] = cmax_idx[i] - cmin_idx[i] + 1;
    int npts = cgp[0] * cgp[1] * cgp[2];
    if (npts < 8)
        npts = 8;
    if (npts > w->alloc)
    {
        w->gidx = (int*)realloc(w->gidx, sizeof(int) * 3 * (size_t)npts);
        w->gmass = (double*)realloc(w->gmass, sizeof(double) * (size_t)npts);
        w->border = (int*)realloc(w->border, sizeof(int) * 2 * (size_t)npts);
        w->alloc = npts;
    }
    int n = cell_interior_grid_pts(cgp, cmin_idx, cmin_pos, w, step, eps, mass);
    if (!n)
    {
        float wm[8];
        distribute_cic(site, mass, w->gidx, wm, step, gmin, eps);
        for (int i = 0; i < 8; ++i)
            w->gmass[i] = (double)wm[i];
        n = 8;
    }
    return n;
}

/* one cell of IterateCells: -1 skipped, 0 outside, else #points in w */
static int iterate_cell(const orc_block* b, int cell, const float* cc, cell_ws* w,
                        const float* data_mins, const float* data_maxs,
                        const float* gmin, const float* step, float mass, float eps, float* cb6)
{
    if (b->vert_to_tet[cell] == -1 || !orc_complete(cell, b->tets, b->num_tets, b->vert_to_tet[cell]))
        return -1;
    float cmin[3], cmax[3];
    cell_bounds(b, cell, cc, cmin, cmax, &w->f, &w->nbrs, &w->link, &w->fv, &w->fv_cap);
    if (cb6)
        for (int i = 0; i < 3; ++i) { cb6[i] = cmin[i]; cb6[3 + i] = cmax[i]; }
    return cell_grid_pts(cmin, cmax, w, data_mins, data_maxs, gmin, step, mass, eps,
                         &b->particles[3 * cell]);
}

int orc_cell_grid_pts(const orc_block* b, int cell, const float* data_mins, const float* data_maxs,
                      const float* gmin, const float* step, float mass, float eps,
                      int* idx, double* pmass, int cap, float* cb6)
{
    float* cc = (float*)malloc(sizeof(float) * 3 * (size_t)(b->num_tets ? b->num_tets : 1));
    orc_fill_circumcenters(b->particles, b->tets, b->num_tets, cc);
    cell_ws w;
    memset(&w, 0, sizeof(w));
    int n = iterate_cell(b, cell, cc, &w, data_mins, data_maxs, gmin, step, mass, eps, cb6);
    for (int i = 0; i < n && i < cap; ++i)
    {
        idx[3 * i] = w.gidx[3 * i]; idx[3 * i + 1] = w.gidx[3 * i + 1]; idx[3 * i + 2] = w.gidx[3 * i + 2];
        pmass[i] = w.gmass[i];
    }
    ws_free(&w);
    free(cc);
    return n;
}

/* DENSE_TESS's per-cell work (IterateCells, src/dense.cpp:220-313: CellBounds,
   CellGridPts, the deposits) for a list of one block's cells, with the block's
   circumcenters cc computed beforehand; the deposits go into grid (the global
   grid, x fastest; may be NULL) and each cell's CellGridPts result into
   counts (may be NULL: -1 skipped cell, else the grid points it deposited
   to).  Returns the cells that deposited.  For timing the reference estimator
   on samples of cells and checking samples of a large run. */
long orc_dense_tess_cells(const orc_block* b, const float* cc, const int* cells, int ncells, const float* data6,
                          const int* glo_num_idx, float mass, float eps, float* grid, int* counts)
{
    float gmin[3], gmax[3], step[3];
    orc_grid_step_params(0, NULL, NULL, data6, data6 + 3, gmin, gmax, step, glo_num_idx);
    const float div = step[0] * step[1] * step[2];
    cell_ws w;
    memset(&w, 0, sizeof(w));
    long done = 0;
    for (int k = 0; k < ncells; ++k)
    {
        const int n = iterate_cell(b, cells[k], cc, &w, data6, data6 + 3, gmin, step, mass, eps, NULL);
        if (counts)
            counts[k] = n;
        if (n <= 0)
            continue;
        done++;
        for (int i = 0; i < n && grid; ++i)
        {
            const int* gi = &w.gidx[3 * i];
            if (gi[0] < 0 || gi[1] < 0 || gi[2] < 0 || gi[0] >= glo_num_idx[0] || gi[1] >= glo_num_idx[1] ||
                gi[2] >= glo_num_idx[2])
                continue;
            float* d = &grid[((size_t)gi[2] * glo_num_idx[1] + gi[1]) * glo_num_idx[0] + gi[0]];
            *d = (float)((double)*d + w.gmass[i] / div);
        }
    }
    ws_free(&w);
    return done;
}

/* ------------------------------------------------------------------ */
/* part 1: dense() over blocks                                        */
/* ------------------------------------------------------------------ */
typedef struct { int idx[3]; double mass; } sent_pt;
typedef struct { sent_pt* a; long n, cap; } svec;
static void sv_push(svec* v, const int* idx, double m)
{
    if (v->n == v->cap)
    {
        v->cap = v->cap ? 2 * v->cap : 256;
        v->a = (sent_pt*)realloc(v->a, sizeof(sent_pt) * (size_t)v->cap);
    }
    v->a[v->n].idx[0] = idx[0]; v->a[v->n].idx[1] = idx[1]; v->a[v->n].idx[2] = idx[2];
    v->a[v->n].mass = m;
    v->n++;
}

typedef struct
{
    int    min_idx[3], max_idx[3], num_idx[3];
    float* density;
} block_grid;

static int inside_bounds(const float* p, const float* mn, const float* mx)
{
    return p[0] >= mn[0] && p[0] <= mx[0] && p[1] >= mn[1] && p[1] <= mx[1] &&
           p[2] >= mn[2] && p[2] <= mx[2];
}

/* local array slot of a global grid index (Global2LocalIdx + index,
   src/dense.cpp:1047-1090, 1210-1218), -1 past the block array; projected
   onto the x-y plane every z maps to the block's 2-D array */
static long local_index(const block_grid* g, const int* gi, int project)
{
    int l[3];
    for (int d = 0; d < 3; ++d)
    {
        l[d] = gi[d] - g->min_idx[d];
        if (l[d] < 0 || l[d] >= g->num_idx[d])
            return -1;
    }
    if (project)
        return (long)l[1] * g->num_idx[0] + l[0];
    return ((long)l[2] * g->num_idx[1] + l[1]) * g->num_idx[0] + l[0];
}

long orc_dense(int alg, int nblocks, const orc_block* blocks,
               int num_given_bounds, const float* given_mins, const float* given_maxs,
               float mass, float eps, const int* glo_num_idx,
               float* global_grid, float* grid_out6, float* data_out6, double* stats3,
               int* cell_counts)
{
    return orc_dense_bounds(alg, nblocks, blocks, NULL, num_given_bounds, given_mins, given_maxs, mass, eps,
                            glo_num_idx, global_grid, grid_out6, data_out6, stats3, cell_counts);
}

long orc_dense_bounds(int alg, int nblocks, const orc_block* blocks, const float* data6,
                      int num_given_bounds, const float* given_mins, const float* given_maxs,
                      float mass, float eps, const int* glo_num_idx,
                      float* global_grid, float* grid_out6, float* data_out6, double* stats3,
                      int* cell_counts)
{
    return orc_dense_ex(alg, nblocks, blocks, data6, 0, num_given_bounds, given_mins, given_maxs, mass, eps,
                        glo_num_idx, global_grid, NULL, grid_out6, data_out6, stats3, cell_counts);
}

long orc_dense_ex(int alg, int nblocks, const orc_block* blocks, const float* data6, int project,
                  int num_given_bounds, const float* given_mins, const float* given_maxs,
                  float mass, float eps, const int* glo_num_idx,
                  float* global_grid, float* block_out, float* grid_out6, float* data_out6, double* stats3,
                  int* cell_counts)
{
    float data_mins[3], data_maxs[3], gmin[3], gmax[3], step[3];
    orc_data_bounds(nblocks, blocks, data_mins, data_maxs);
    if (data6)
        for (int i = 0; i < 3; ++i) { data_mins[i] = data6[i]; data_maxs[i] = data6[3 + i]; }
    orc_grid_step_params(num_given_bounds, given_mins, given_maxs, data_mins, data_maxs,
                         gmin, gmax, step, glo_num_idx);
    float max_dense = 0.0f, check_mass = 0.0f;
    double tot_mass = 0.0;
    long lost = 0;

    block_grid* bg = (block_grid*)calloc((size_t)nblocks, sizeof(block_grid));
    for (int i = 0; i < nblocks; ++i)
    {
        orc_block_grid_params(&blocks[i], gmin, step, eps, data_mins, data_maxs, glo_num_idx,
                              bg[i].min_idx, bg[i].max_idx, bg[i].num_idx);
        /* init_dense, src/dense.cpp:117-121 */
        long npts = (long)bg[i].num_idx[0] * bg[i].num_idx[1] * (project ? 1 : bg[i].num_idx[2]);
        bg[i].density = (float*)calloc((size_t)(npts > 0 ? npts : 1), sizeof(float));
    }
    /* src/dense.cpp:241-242 */
    float div = project ? step[0] * step[1] : step[0] * step[1] * step[2];

    /* queues[dest * nblocks + src] */
    svec* queues = (svec*)calloc((size_t)nblocks * nblocks, sizeof(svec));
    cell_ws w;
    memset(&w, 0, sizeof(w));
    long cell_base = 0;

    for (int bi = 0; bi < nblocks; ++bi)
    {
        const orc_block* b = &blocks[bi];
        float* cc = NULL;
        if (alg == 0)
        {
            cc = (float*)malloc(sizeof(float) * 3 * (size_t)(b->num_tets ? b->num_tets : 1));
            orc_fill_circumcenters(b->particles, b->tets, b->num_tets, cc);
        }
        for (int cell = 0; cell < b->num_orig_particles; ++cell)
        {
            int n;
            int cic_idx[24];
            float cic_w[8];
            if (alg == 0)
            {
                n = iterate_cell(b, cell, cc, &w, data_mins, data_maxs, gmin, step, mass, eps, NULL);
                if (cell_counts)
                    cell_counts[cell_base + cell] = n;
                if (n <= 0)
                    continue;
            }
            else
            {
                distribute_cic(&b->particles[3 * cell], mass, cic_idx, cic_w, step, gmin, eps);
                n = 8;
                if (cell_counts)
                    cell_counts[cell_base + cell] = 8;
            }
            check_mass++;
            for (int i = 0; i < n; ++i)
            {
                const int* gi = alg == 0 ? &w.gidx[3 * i] : &cic_idx[3 * i];
                double m = alg == 0 ? w.gmass[i] : (double)cic_w[i];
                float gp[3];
                idx2phys(gi, gp, step, gmin);
                if (inside_bounds(gp, b->bounds_min, b->bounds_max))
                {
                    long li = local_index(&bg[bi], gi, project);
                    if (li < 0) { lost++; continue; }
                    float* d = &bg[bi].density[li];
                    if (alg == 0)
                        *d = (float)((double)*d + m / div);     /* src/dense.cpp:290 */
                    else
                        *d += cic_w[i] / div;                    /* src/dense.cpp:539 */
                    tot_mass += m;
                    if (*d > max_dense)
                        max_dense = *d;
                }
                else
                {
                    int sent = 0;
                    for (int nb = 0; nb < nblocks; ++nb)
                        if (nb != bi && inside_bounds(gp, blocks[nb].bounds_min, blocks[nb].bounds_max))
                        {
                            sv_push(&queues[(size_t)nb * nblocks + bi], gi, m);
                            sent = 1;
                        }
                    if (!sent)
                        lost++;
                }
            }
        }
        cell_base += b->num_orig_particles;
        free(cc);
    }

    /* recvd_pts, src/dense.cpp:166-202: sources in ascending gid order */
    for (int bi = 0; bi < nblocks; ++bi)
    {
        int order[1024];
        int ns = 0;
        for (int s = 0; s < nblocks && ns < 1024; ++s)
            if (queues[(size_t)bi * nblocks + s].n)
                order[ns++] = s;
        for (int i = 1; i < ns; ++i)
            for (int j = i; j > 0 && blocks[order[j]].gid < blocks[order[j - 1]].gid; --j)
            {
                int t = order[j]; order[j] = order[j - 1]; order[j - 1] = t;
            }
        for (int k = 0; k < ns; ++k)
        {
            svec* q = &queues[(size_t)bi * nblocks + order[k]];
            for (long j = 0; j < q->n; ++j)
            {
                long li = local_index(&bg[bi], q->a[j].idx, project);
                if (li < 0) { lost++; continue; }
                float* d = &bg[bi].density[li];
                *d = (float)((double)*d + q->a[j].mass / div);
                tot_mass += q->a[j].mass;
                if (*d > max_dense)
                    max_dense = *d;
            }
        }
    }

    size_t nx = glo_num_idx[0], ny = glo_num_idx[1];
    if (block_out)
    {
        size_t off = 0;
        for (int i = 0; i < nblocks; ++i)
        {
            size_t n = (size_t)bg[i].num_idx[0] * bg[i].num_idx[1] * (project ? 1 : bg[i].num_idx[2]);
            memcpy(block_out + off, bg[i].density, sizeof(float) * n);
            off += n;
        }
    }
    if (project)
    {
        /* ProjectGrid (src/dense.cpp:881-1023) with every block in this
           process: the root of a column is the block with the same x-y grid
           origin and min_idx[2] == 0 (the last such block by gid order); the
           other blocks, in block order, add their first num_idx[0]*num_idx[1]
           values into it */
        for (int i = 0; i < nblocks; ++i)
        {
            if (!bg[i].min_idx[2])
                continue;
            int root = -1;
            for (int j = 0; j < nblocks; ++j)
                if (bg[j].min_idx[0] == bg[i].min_idx[0] && bg[j].min_idx[1] == bg[i].min_idx[1] &&
                    !bg[j].min_idx[2] && (root < 0 || blocks[j].gid > blocks[root].gid))
                    root = j;
            if (root < 0)
                continue;
            long n = (long)bg[i].num_idx[0] * bg[i].num_idx[1];
            for (long k = 0; k < n; ++k)
                bg[root].density[k] += bg[i].density[k];
        }
        /* WriteGrid (src/dense.cpp:812-828): root blocks write their 2-D
           arrays at (min_idx[1], min_idx[0]) of the glo_num_idx[1] x [0] array */
        memset(global_grid, 0, sizeof(float) * nx * ny);
        for (int i = 0; i < nblocks; ++i)
        {
            if (bg[i].min_idx[2])
                continue;
            for (int y = 0; y < bg[i].num_idx[1]; ++y)
                for (int x = 0; x < bg[i].num_idx[0]; ++x)
                    global_grid[(size_t)(bg[i].min_idx[1] + y) * nx + (bg[i].min_idx[0] + x)] =
                        bg[i].density[(size_t)y * bg[i].num_idx[0] + x];
        }
        for (int i = 0; i < nblocks; ++i)
            free(bg[i].density);
    }
    else
        memset(global_grid, 0, sizeof(float) * nx * ny * (size_t)glo_num_idx[2]);
    for (int i = 0; i < nblocks && !project; ++i)
    {
        for (int z = 0; z < bg[i].num_idx[2]; ++z)
            for (int y = 0; y < bg[i].num_idx[1]; ++y)
                for (int x = 0; x < bg[i].num_idx[0]; ++x)
                    global_grid[((size_t)(bg[i].min_idx[2] + z) * ny + (bg[i].min_idx[1] + y)) * nx +
                                (bg[i].min_idx[0] + x)] =
                        bg[i].density[((size_t)z * bg[i].num_idx[1] + y) * bg[i].num_idx[0] + x];
        free(bg[i].density);
    }
    for (size_t i = 0; i < (size_t)nblocks * nblocks; ++i)
        free(queues[i].a);
    free(queues);
    free(bg);
    ws_free(&w);

    if (grid_out6)
        for (int i = 0; i < 3; ++i) { grid_out6[i] = gmin[i]; grid_out6[3 + i] = step[i]; }
    if (data_out6)
        for (int i = 0; i < 3; ++i) { data_out6[i] = data_mins[i]; data_out6[3 + i] = data_maxs[i]; }
    if (stats3)
    {
        stats3[0] = max_dense;
        stats3[1] = tot_mass;
        stats3[2] = check_mass;
    }
    return lost;
}

/* ------------------------------------------------------------------ */
/* part 1: incomplete_cells (src/tess.cpp:492-628)                    */
/* ------------------------------------------------------------------ */
/* src/tet.cpp:70-119; dot, src/tet.cpp:22-28 */
int orc_side_of_plane(const float* box6, const orc_tet* tet, const float* particles, int j)
{
    int idx[4] = { 0, 1, 2, 3 };
    int tmp = idx[j]; idx[j] = idx[3]; idx[3] = tmp;
    const float* x = &particles[3 * tet->verts[idx[0]]];
    const float* y = &particles[3 * tet->verts[idx[1]]];
    const float* z = &particles[3 * tet->verts[idx[2]]];
    const float* p = &particles[3 * tet->verts[idx[3]]];
    float u[3], v[3], n[3];
    for (int i = 0; i < 3; ++i)
    {
        u[i] = y[i] - x[i];
        v[i] = z[i] - x[i];
    }
    cross3(n, u, v);
    float res = 0;
    for (int i = 0; i < 3; ++i)
        res += n[i] * (p[i] - x[i]);
    int sign = res > 0 ? 1 : (res < 0 ? -1 : 0);
    if (sign == 0)
        return 1;
    res = 0;
    for (int i = 0; i < 3; ++i)
    {
        if ((sign > 0) != (n[i] < 0))
            res += n[i] * (box6[i] - x[i]);
        else
            res += n[i] * (box6[3 + i] - x[i]);
    }
    return (sign > 0) != (res > 0);
}

float orc_distance(const float* u, const float* v) { return dist3(u, v); }

/* DIY's distance(bounds, point) (github.com/diatomic/diy, not vendored by
   the reference): per axis the excess of the point beyond the box, squared
   and summed in float; the square root of the sum */
float orc_box_distance(const float* box6, const float* c)
{
    float res = 0;
    for (int i = 0; i < 3; ++i)
    {
        float diff = 0, d;
        d = box6[i] - c[i];
        if (d > diff) diff = d;
        d = c[i] - box6[3 + i];
        if (d > diff) diff = d;
        res += diff * diff;
    }
    return (float)sqrt((double)res);
}

long orc_incomplete_cells(const orc_block* b, int num_links, const float* links6, const int* wrap3,
                          int last_neighbor, unsigned long long* masks)
{
    int norig = b->num_orig_particles;
    for (int p = 0; p < norig; ++p)
        masks[p] = 0;
    /* wrap_bounds (DIY): bounds += wrap * (data max - data min) */
    float* nb6 = (float*)malloc(sizeof(float) * 6 * (size_t)(num_links > 0 ? num_links : 1));
    for (int i = 0; i < num_links; ++i)
        for (int d = 0; d < 3; ++d)
        {
            float ext = b->data_max[d] - b->data_min[d];
            int w = wrap3 ? wrap3[3 * i + d] : 0;
            nb6[6 * i + d] = links6[6 * i + d] + w * ext;
            nb6[6 * i + 3 + d] = links6[6 * i + 3 + d] + w * ext;
        }
    for (int t = 0; t < b->num_tets; ++t)
    {
        const orc_tet* tt = &b->tets[t];
        int j;
        for (j = 0; j < 4; ++j)
            if (tt->verts[j] < norig)
                break;
        if (j == 4)
            continue;
        float center[3];
        orc_circumcenter(center, tt, b->particles);
        float rad = dist3(center, &b->particles[3 * tt->verts[0]]);
        for (j = 0; j < 4; ++j)
        {
            if (tt->tets[j] != -1)
                continue;
            int k;
            for (k = 0; k < 4; ++k)
            {
                if (k == j) continue;
                if (tt->verts[k] < norig) break;
            }
            if (k == 4)
                continue;
            for (int i = last_neighbor; i < num_links; ++i)
            {
                if (!orc_side_of_plane(&nb6[6 * i], tt, b->particles, j))
                    continue;
                for (int v = 0; v < 4; ++v)
                {
                    if (v == j) continue;
                    int p = tt->verts[v];
                    if (p >= norig) continue;
                    masks[p] |= 1ull << i;
                }
            }
        }
        for (j = 0; j < 3; ++j)
        {
            if (center[j] - b->bounds_min[j] <= rad) break;
            if (b->bounds_max[j] - center[j] <= rad) break;
        }
        if (j == 3)
            continue;
        for (int i = last_neighbor; i < num_links; ++i)
        {
            if (orc_box_distance(&nb6[6 * i], center) <= rad)
                for (int v = 0; v < 4; ++v)
                {
                    int p = tt->verts[v];
                    if (p >= norig) continue;
                    masks[p] |= 1ull << i;
                }
        }
    }
    /* src/tess.cpp:587-603 (release build: no assert) */
    if (b->num_tets == 0)
        for (int p = 0; p < norig; ++p)
            for (int i = last_neighbor; i < num_links; ++i)
                masks[p] |= 1ull << i;
    long enqueued = 0;
    for (int p = 0; p < norig; ++p)
        for (int i = 0; i < 64; ++i)
            enqueued += (long)((masks[p] >> i) & 1ull);
    free(nb6);
    return enqueued;
}

/* src/tess-qhull.c:161-225: for vertex v in order, the first neighbour not yet
   taken that does not hold verts[v]; -1 when none does */
void orc_reorder_neighbors(orc_tet* tets, int num_tets)
{
    for (int t = 0; t < num_tets; ++t)
    {
        int nb[4], out[4];
        for (int n = 0; n < 4; ++n)
            nb[n] = tets[t].tets[n];
        for (int v = 0; v < 4; ++v)
        {
            out[v] = -1;
            for (int n = 0; n < 4; ++n)
            {
                int c = nb[n];
                if (c < 0)
                    continue;
                int has = 0;
                for (int k = 0; k < 4; ++k)
                    if (tets[c].verts[k] == tets[t].verts[v])
                        has = 1;
                if (!has)
                {
                    out[v] = c;
                    nb[n] = -2;
                    break;
                }
            }
        }
        for (int n = 0; n < 4; ++n)
            tets[t].tets[n] = out[n];
    }
}

/* ------------------------------------------------------------------ */
/* part 2: FP64 references                                                */
/* ------------------------------------------------------------------ */

void orc_fill_circumcenters_f64(const float* particles, const orc_tet* tets, int num_tets, double* out)
{
    for (int k = 0; k < num_tets; ++k)
    {
        const float* a = &particles[3 * tets[k].verts[0]];
        const float* b = &particles[3 * tets[k].verts[1]];
        const float* c = &particles[3 * tets[k].verts[2]];
        const float* d = &particles[3 * tets[k].verts[3]];
        double t[3], u[3], v[3];
        for (int i = 0; i < 3; ++i)
        {
            t[i] = (double)a[i] - d[i];
            u[i] = (double)b[i] - d[i];
            v[i] = (double)c[i] - d[i];
        }
        double nt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
        double nu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        double nv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        double uv[3] = { u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0] };
        double vt[3] = { v[1] * t[2] - v[2] * t[1], v[2] * t[0] - v[0] * t[2], v[0] * t[1] - v[1] * t[0] };
        double tu[3] = { t[1] * u[2] - t[2] * u[1], t[2] * u[0] - t[0] * u[2], t[0] * u[1] - t[1] * u[0] };
        double den = 2 * (t[0] * uv[0] + t[1] * uv[1] + t[2] * uv[2]);
        for (int i = 0; i < 3; ++i)
            out[3 * k + i] = d[i] + (nt * uv[i] + nu * vt[i] + nv * tu[i]) / den;
    }
}

/* volume() (src/volume.cpp:13-54) with every quantity in double */
void orc_volumes_f64(int n, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                     const float* particles, double* out)
{
    double* cc = (double*)malloc(sizeof(double) * 3 * (size_t)(num_tets ? num_tets : 1));
    orc_fill_circumcenters_f64(particles, tets, num_tets, cc);
    ivec nbrs = {0}, link = {0};
    for (int v = 0; v < n; ++v)
    {
        if (vert_to_tet[v] < 0) { out[v] = -1; continue; }
        int finite;
        int nf = neighbor_edges_iv(v, tets, vert_to_tet[v], &nbrs, &finite);
        if (!finite) { out[v] = -1; continue; }
        double vol = 0;
        for (int k = 0; k < nf; ++k)
        {
            int u = nbrs.a[2 * k], ut = nbrs.a[2 * k + 1];
            fill_edge_link_iv(v, u, ut, tets, &link);
            double area = 0;
            int a = link.a[0];
            for (int i = 1; i < link.n - 1; ++i)
            {
                int b = link.a[i], c = link.a[i + 1];
                double ab[3], ac[3];
                for (int j = 0; j < 3; ++j)
                {
                    ab[j] = cc[3 * b + j] - cc[3 * a + j];
                    ac[j] = cc[3 * c + j] - cc[3 * a + j];
                }
                double cp[3] = { ab[1] * ac[2] - ab[2] * ac[1], ab[2] * ac[0] - ab[0] * ac[2],
                                 ab[0] * ac[1] - ab[1] * ac[0] };
                area += sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]) / 2;
            }
            double dd = 0;
            for (int j = 0; j < 3; ++j)
            {
                double e = (double)particles[3 * u + j] - particles[3 * v + j];
                dd += e * e;
            }
            vol += area * sqrt(dd) / 6;
        }
        out[v] = vol;
    }
    iv_free(&nbrs);
    iv_free(&link);
    free(cc);
}

/* ---- exact predicates for float32 inputs ---------------------------
   Every monomial of the orientation determinant is a product of three
   float32 numbers.  x*y is exact in double (48 significant bits); the
   product with z is split into hi + lo with one FMA (Dekker/Knuth
   two-product).  The signed sum of the resulting doubles is evaluated
   exactly by Shewchuk's grow-expansion (J. R. Shewchuk, "Adaptive
   Precision Floating-Point Arithmetic and Fast Robust Geometric
   Predicates", 1997), whose largest component carries the sign. */
static void two_sum(double a, double b, double* s, double* e)
{
    double x = a + b, bv = x - a, av = x - bv;
    *e = (a - av) + (b - bv);
    *s = x;
}

static int exact_sign(const double* t, int n)
{
    double e[64];
    int m = 0;
    for (int i = 0; i < n; ++i)
    {
        double q = t[i];
        int k = 0;
        for (int j = 0; j < m; ++j)
        {
            double hi, lo;
            two_sum(q, e[j], &hi, &lo);
            if (lo != 0.0)
                e[k++] = lo;
            q = hi;
        }
        if (q != 0.0)
            e[k++] = q;
        m = k;
    }
    return m == 0 ? 0 : (e[m - 1] > 0 ? 1 : -1);
}

static int add_triple(double* t, int n, double s, float x, float y, float z)
{
    double xy = (double)x * (double)y;
    double hi = xy * (double)z;
    double lo = fma(xy, (double)z, -hi);
    t[n] = s * hi;
    t[n + 1] = s * lo;
    return n + 2;
}

/* det3(u, v, w) = u . (v x w) as 6 signed monomials */
static int add_det3(double* t, int n, double s, const float* u, const float* v, const float* w)
{
    n = add_triple(t, n, s, u[0], v[1], w[2]);
    n = add_triple(t, n, -s, u[0], v[2], w[1]);
    n = add_triple(t, n, s, u[1], v[2], w[0]);
    n = add_triple(t, n, -s, u[1], v[0], w[2]);
    n = add_triple(t, n, s, u[2], v[0], w[1]);
    n = add_triple(t, n, -s, u[2], v[1], w[0]);
    return n;
}

/* O(x,y,z,p) = det[y-x; z-x; p-x] = det3(y,z,p) - det3(x,z,p) + det3(x,y,p) - det3(x,y,z) */
static int orient_exact(const float* x, const float* y, const float* z, const float* p)
{
    double t[48];
    int n = 0;
    n = add_det3(t, n, 1.0, y, z, p);
    n = add_det3(t, n, -1.0, x, z, p);
    n = add_det3(t, n, 1.0, x, y, p);
    n = add_det3(t, n, -1.0, x, y, z);
    return exact_sign(t, n);
}

/* the same determinant in double with Shewchuk's orient3d error bound;
   returns the certain sign or falls back to the exact evaluation */
static int orient_filtered(const float* x, const float* y, const float* z, const float* p)
{
    /* det[x-p; y-p; z-p] = -O(x,y,z,p) */
    double adx = (double)x[0] - p[0], ady = (double)x[1] - p[1], adz = (double)x[2] - p[2];
    double bdx = (double)y[0] - p[0], bdy = (double)y[1] - p[1], bdz = (double)y[2] - p[2];
    double cdx = (double)z[0] - p[0], cdy = (double)z[1] - p[1], cdz = (double)z[2] - p[2];
    double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    double cdxady = cdx * ady, adxcdy = adx * cdy;
    double adxbdy = adx * bdy, bdxady = bdx * ady;
    double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    double perm = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) + (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz) +
                  (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    const double eps = 1.1102230246251565e-16;   /* 2^-53 */
    double bound = (7.0 + 56.0 * eps) * eps * perm;
    if (det > bound) return -1;
    if (-det > bound) return 1;
    return orient_exact(x, y, z, p);
}

int orc_orient3d_exact(const float* a, const float* b, const float* c, const float* d)
{
    return orient_exact(a, b, c, d);
}

/* exact sign of component j of (y-x) x (z-x): six products of two floats */
static int face_normal_sign(const float* x, const float* y, const float* z, int j)
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

/* F_i (face opposite vertex i) and the sign relating D_i(p) = O(a0..p..a3)
   to O(F_i, p) */
static const int face_of[4][3] = { {1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2} };
static const int face_sigma[4] = { -1, 1, -1, 1 };

int orc_tet_contains(const float* particles, const orc_tet* t, const float* p)
{
    const float* a[4];
    for (int i = 0; i < 4; ++i)
        a[i] = &particles[3 * t->verts[i]];
    int s = orient_exact(a[0], a[1], a[2], a[3]);
    if (s == 0)
        return 0;
    for (int i = 0; i < 4; ++i)
    {
        const float* x = a[face_of[i][0]];
        const float* y = a[face_of[i][1]];
        const float* z = a[face_of[i][2]];
        int o = orient_filtered(x, y, z, p);
        if (o == 0)
            for (int j = 0; j < 3 && o == 0; ++j)
                o = face_normal_sign(x, y, z, j);
        if (s * face_sigma[i] * o <= 0)
            return 0;
    }
    return 1;
}

long orc_dtfe_f64(int nblocks, const orc_block* blocks,
                  int num_given_bounds, const float* given_mins, const float* given_maxs,
                  float mass, float eps, const int* glo_num_idx,
                  float* global_grid, double* rho_out, int* owner_out, float* grid_out6)
{
    return orc_dtfe_f64_sample(nblocks, blocks, NULL, num_given_bounds, given_mins, given_maxs, mass, eps,
                               glo_num_idx, 1, global_grid, rho_out, owner_out, grid_out6);
}

long orc_dtfe_f64_sample(int nblocks, const orc_block* blocks, const float* data6,
                         int num_given_bounds, const float* given_mins, const float* given_maxs,
                         float mass, float eps, const int* glo_num_idx, int raster_stride,
                         float* global_grid, double* rho_out, int* owner_out, float* grid_out6)
{
    float data_mins[3], data_maxs[3], gmin[3], gmax[3], step[3];
    orc_data_bounds(nblocks, blocks, data_mins, data_maxs);
    if (data6)
        for (int i = 0; i < 3; ++i) { data_mins[i] = data6[i]; data_maxs[i] = data6[3 + i]; }
    if (raster_stride < 1)
        raster_stride = 1;
    orc_grid_step_params(num_given_bounds, given_mins, given_maxs, data_mins, data_maxs,
                         gmin, gmax, step, glo_num_idx);
    size_t nx = glo_num_idx[0], ny = glo_num_idx[1], nz = glo_num_idx[2];
    memset(global_grid, 0, sizeof(float) * nx * ny * nz);
    if (owner_out)
        for (size_t i = 0; i < nx * ny * nz; ++i)
            owner_out[i] = -1;
    long assigned = 0;
    long rho_base = 0;

    for (int bi = 0; bi < nblocks; ++bi)
    {
        const orc_block* b = &blocks[bi];
        int mn[3], mx[3], num[3];
        orc_block_grid_params(b, gmin, step, eps, data_mins, data_maxs, glo_num_idx, mn, mx, num);
        double* W = (double*)calloc((size_t)(b->num_particles ? b->num_particles : 1), sizeof(double));
        double* rho = (double*)calloc((size_t)(b->num_particles ? b->num_particles : 1), sizeof(double));
        for (int t = 0; t < b->num_tets; ++t)
        {
            const float* a = &b->particles[3 * b->tets[t].verts[0]];
            double e[3][3];
            for (int k = 0; k < 3; ++k)
            {
                const float* q = &b->particles[3 * b->tets[t].verts[k + 1]];
                for (int d = 0; d < 3; ++d)
                    e[k][d] = (double)q[d] - a[d];
            }
            double det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) +
                         e[0][1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
                         e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
            double vol = fabs(det) / 6.0;
            for (int k = 0; k < 4; ++k)
                W[b->tets[t].verts[k]] += vol;
        }
        for (int v = 0; v < b->num_particles; ++v)
            rho[v] = W[v] > 0 ? 4.0 * (double)mass / W[v] : 0.0;

        for (int t = 0; t < b->num_tets; t += raster_stride)
        {
            const orc_tet* tt = &b->tets[t];
            const float* a[4];
            float lo[3], hi[3];
            for (int k = 0; k < 4; ++k)
                a[k] = &b->particles[3 * tt->verts[k]];
            for (int d = 0; d < 3; ++d)
            {
                lo[d] = hi[d] = a[0][d];
                for (int k = 1; k < 4; ++k)
                {
                    if (a[k][d] < lo[d]) lo[d] = a[k][d];
                    if (a[k][d] > hi[d]) hi[d] = a[k][d];
                }
            }
            int ilo[3], ihi[3];
            int skip = 0;
            for (int d = 0; d < 3; ++d)
            {
                /* candidate range, widened by one: the exact test decides */
                ilo[d] = (int)floor(((double)lo[d] - gmin[d]) / step[d]) - 1;
                ihi[d] = (int)floor(((double)hi[d] - gmin[d]) / step[d]) + 1;
                if (ilo[d] < mn[d]) ilo[d] = mn[d];
                if (ihi[d] > mx[d]) ihi[d] = mx[d];
                if (ilo[d] > ihi[d]) skip = 1;
            }
            if (skip)
                continue;
            if (orient_exact(a[0], a[1], a[2], a[3]) == 0)
                continue;
            double e[3][3];
            for (int k = 0; k < 3; ++k)
                for (int d = 0; d < 3; ++d)
                    e[k][d] = (double)a[k + 1][d] - a[0][d];
            double V = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) +
                       e[0][1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
                       e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
            double r[4];
            for (int k = 0; k < 4; ++k)
                r[k] = rho[tt->verts[k]];
            int gi[3];
            for (gi[2] = ilo[2]; gi[2] <= ihi[2]; gi[2]++)
                for (gi[1] = ilo[1]; gi[1] <= ihi[1]; gi[1]++)
                    for (gi[0] = ilo[0]; gi[0] <= ihi[0]; gi[0]++)
                    {
                        float p[3];
                        idx2phys(gi, p, step, gmin);
                        if (!orc_tet_contains(b->particles, tt, p))
                            continue;
                        double q[3] = { (double)p[0] - a[0][0], (double)p[1] - a[0][1], (double)p[2] - a[0][2] };
                        double l1 = (q[0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) +
                                     q[1] * (e[1][2] * e[2][0] - e[1][0] * e[2][2]) +
                                     q[2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0])) / V;
                        double l2 = (e[0][0] * (q[1] * e[2][2] - q[2] * e[2][1]) +
                                     e[0][1] * (q[2] * e[2][0] - q[0] * e[2][2]) +
                                     e[0][2] * (q[0] * e[2][1] - q[1] * e[2][0])) / V;
                        double l3 = (e[0][0] * (e[1][1] * q[2] - e[1][2] * q[1]) +
                                     e[0][1] * (e[1][2] * q[0] - e[1][0] * q[2]) +
                                     e[0][2] * (e[1][0] * q[1] - e[1][1] * q[0])) / V;
                        double l0 = 1.0 - l1 - l2 - l3;
                        double f = l0 * r[0] + l1 * r[1] + l2 * r[2] + l3 * r[3];
                        size_t g = ((size_t)gi[2] * ny + gi[1]) * nx + gi[0];
                        global_grid[g] = (float)f;
                        if (owner_out)
                            owner_out[g] = t;
                        assigned++;
                    }
        }
        if (rho_out)
            for (int v = 0; v < b->num_particles; ++v)
                rho_out[rho_base + v] = rho[v];
        rho_base += b->num_particles;
        free(W);
        free(rho);
    }
    if (grid_out6)
        for (int i = 0; i < 3; ++i) { grid_out6[i] = gmin[i]; grid_out6[3 + i] = step[i]; }
    return assigned;
}
