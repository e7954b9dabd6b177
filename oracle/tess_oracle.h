/*
 * CPU oracle for the tess2 post-Delaunay geometry + density path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only as the checker
 * or the timed CPU baseline; the product never calls it.
 *
 * Two parts:
 *  1. A plain-C restatement of the reference's FP32 algorithms, operation for
 *     operation (no FMA contraction: build with -ffp-contract=off), so that
 *     its outputs are bit-identical to the reference's own build
 *     (oracle/_ref/libtess_ref.so).  It is pinned against golden vectors
 *     produced by that build (tests/golden/).
 *  2. FP64 references for the new, non-reference stages (Voronoi volumes in FP64,
 *     DTFE vertex densities and tet-linear grid interpolation).  The DTFE
 *     point-to-tet assignment uses exact orientation signs for float32
 *     inputs with a symbolic perturbation of the grid point, so it is a
 *     partition of the triangulated region that any exact implementation
 *     reproduces bit for bit.
 */
#ifndef TESS_ORACLE_H
#define TESS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* include/tess/tet.h:4-7 */
typedef struct orc_tet { int verts[4]; int tets[4]; } orc_tet;

/* One DIY block (include/tess/delaunay.h:38-63 plus DBlock bounds,
   include/tess/delaunay.hpp:18-23) as plain arrays. */
typedef struct orc_block
{
    int          gid;
    float        bounds_min[3], bounds_max[3];
    float        data_min[3], data_max[3];
    int          num_orig_particles;
    int          num_particles;
    const float* particles;     /* 3 * num_particles */
    int          num_tets;
    const orc_tet* tets;
    const int*   vert_to_tet;   /* num_particles */
} orc_block;

/* ---- part 1: reference-order FP32 restatement ---- */
void  orc_fill_vert_to_tet(int num_particles, const orc_tet* tets, int num_tets, int* vert_to_tet);
void  orc_circumcenter(float* c, const orc_tet* tet, const float* particles);
void  orc_fill_circumcenters(const float* particles, const orc_tet* tets, int num_tets, float* out);
int   orc_complete(int v, const orc_tet* tets, int num_tets, int t);
void  orc_complete_all(const orc_tet* tets, int num_tets, const int* vert_to_tet, int n, int* out);
int   orc_neighbor_edges(int v, const orc_tet* tets, int t, int* pairs, int cap, int* finite);
int   orc_fill_edge_link(int v, int u, int ut, const orc_tet* tets, int* link, int cap);
float orc_volume(int v, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                 const float* particles, const float* circumcenters);
void  orc_volumes(int n, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                  const float* particles, float* out);
long  orc_dense_tess_cells(const orc_block* b, const float* cc, const int* cells, int ncells, const float* data6,
                           const int* glo_num_idx, float mass, float eps, float* grid, int* counts);
void  orc_volume_areas(int n, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                       const float* particles, float* vol, float* area);

void  orc_grid_step_params(int num_given_bounds, const float* given_mins, const float* given_maxs,
                           const float* data_mins, const float* data_maxs,
                           float* grid_phys_mins, float* grid_phys_maxs, float* grid_step_size,
                           const int* glo_num_idx);
void  orc_data_bounds(int nblocks, const orc_block* blocks, float* data_mins, float* data_maxs);
void  orc_block_grid_params(const orc_block* b, const float* grid_phys_mins, const float* grid_step_size,
                            float eps, const float* data_mins, const float* data_maxs,
                            const int* glo_num_idx, int* min_idx, int* max_idx, int* num_idx);

/* One cell of IterateCells: -1 skipped (incomplete), 0 outside data bounds,
   else the number of grid points (idx: 3 ints each, mass: double each, up to cap). */
int   orc_cell_grid_pts(const orc_block* b, int cell, const float* data_mins, const float* data_maxs,
                        const float* grid_phys_mins, const float* grid_step_size, float mass, float eps,
                        int* idx, double* pmass, int cap, float* cell_bounds6);

/* dense() over all blocks (alg 0 = DENSE_TESS, 1 = DENSE_CIC) into a global
   grid (x fastest).  cell_counts (optional, per block concatenated over
   num_orig_particles) receives orc_cell_grid_pts' return value per cell
   (DENSE_TESS) or 8 (DENSE_CIC).  stats3: max_dense, tot_mass, check_mass
   for this call.  Returns the number of deposits that fell outside every
   block array (0 for well-formed inputs). */
long  orc_dense(int alg, int nblocks, const orc_block* blocks,
                int num_given_bounds, const float* given_mins, const float* given_maxs,
                float mass, float eps, const int* glo_num_idx,
                float* global_grid, float* grid_out6, float* data_out6, double* stats3,
                int* cell_counts);
/* orc_dense with the data bounds given (data6: mins[3], maxs[3]), as every
   rank sees them after DataBounds' all-reduce when one process holds one
   block of a larger decomposition. */
long  orc_dense_bounds(int alg, int nblocks, const orc_block* blocks, const float* data6,
                       int num_given_bounds, const float* given_mins, const float* given_maxs,
                       float mass, float eps, const int* glo_num_idx,
                       float* global_grid, float* grid_out6, float* data_out6, double* stats3,
                       int* cell_counts);

/* orc_dense_bounds with dense()'s project flag (x-y plane): block arrays of
   num_idx[0]*num_idx[1] floats holding mass per area summed over the block's
   z range; global_grid then receives ProjectGrid's column sums as WriteGrid
   writes them (glo_num_idx[1] x [0] floats), block_out (optional) every
   block's array as dense() leaves it, concatenated in block order. */
long  orc_dense_ex(int alg, int nblocks, const orc_block* blocks, const float* data6, int project,
                   int num_given_bounds, const float* given_mins, const float* given_maxs,
                   float mass, float eps, const int* glo_num_idx,
                   float* global_grid, float* block_out, float* grid_out6, float* data_out6, double* stats3,
                   int* cell_counts);

/* incomplete_cells (src/tess.cpp:492-628) for one block: links6 holds the
   num_links (<= 64) neighbour core boxes (min xyz, max xyz), wrap3 (may be
   NULL) their wrap directions; masks[p] for each original particle gets bit i
   when the reference's to_send[p] holds link i.  Returns the number of
   (particle, link) pairs (the reference's return value). */
long  orc_incomplete_cells(const orc_block* b, int num_links, const float* links6, const int* wrap3,
                           int last_neighbor, unsigned long long* masks);
/* side_of_plane (src/tet.cpp:70-119) */
int   orc_side_of_plane(const float* box6, const orc_tet* tet, const float* particles, int j);
/* distance (src/tet.cpp:146-153) */
float orc_distance(const float* u, const float* v);
/* DIY's distance(bounds, point) */
float orc_box_distance(const float* box6, const float* c);

/* src/tess-qhull.c:161-225, in place */
void  orc_reorder_neighbors(orc_tet* tets, int num_tets);

/* ---- part 2: FP64 references ---- */
void  orc_fill_circumcenters_f64(const float* particles, const orc_tet* tets, int num_tets, double* out);
void  orc_volumes_f64(int n, const int* vert_to_tet, const orc_tet* tets, int num_tets,
                      const float* particles, double* out);

/* exact sign of det[b-a; c-a; d-a] for float32 inputs */
int   orc_orient3d_exact(const float* a, const float* b, const float* c, const float* d);
/* 1 if the symbolically perturbed point p + (e, e^2, e^3) lies inside tet t */
int   orc_tet_contains(const float* particles, const orc_tet* t, const float* p);

/* DTFE in FP64: per-vertex density rho = 4 m / (sum of |tet volume| over the
   vertex's tets), then for every grid point a block owns (BlockGridParams)
   the barycentric interpolation of rho in the tet that contains it (0 outside
   every tet).  rho_out: per block concatenated over num_particles (optional);
   owner_out: containing tet (block-local index) per global grid point, -1 if
   none (optional).  Grid parameters follow dense() (GridStepParams over the
   union of block bounds).  Returns the number of grid points assigned. */
long  orc_dtfe_f64(int nblocks, const orc_block* blocks,
                   int num_given_bounds, const float* given_mins, const float* given_maxs,
                   float mass, float eps, const int* glo_num_idx,
                   float* global_grid, double* rho_out, int* owner_out, float* grid_out6);
/* orc_dtfe_f64 with explicit data bounds (may be NULL) that rasterises only
   every raster_stride-th tet (a bounded sample for CPU timing). */
long  orc_dtfe_f64_sample(int nblocks, const orc_block* blocks, const float* data6,
                          int num_given_bounds, const float* given_mins, const float* given_maxs,
                          float mass, float eps, const int* glo_num_idx, int raster_stride,
                          float* global_grid, double* rho_out, int* owner_out, float* grid_out6);

#ifdef __cplusplus
}
#endif
#endif
