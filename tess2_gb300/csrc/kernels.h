// Host-side launchers of the tess2_gb300 kernels (one .cu per family).
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"
#include "dtfe_common.cuh"

namespace tg {

// geometry.cu  (reference-order FP32, built with -fmad=false)
void launch_ingest(const int* const* d_raw_tets, const BlockDesc* d_blocks, int nb, int total_tets,
                   int4* tv, int4* tn, Status* st, cudaStream_t s);
void launch_vert_to_tet(const int4* tv, int total_tets, int* v2t, cudaStream_t s);
void launch_v2t_from_local(const int* const* d_raw_v2t, const BlockDesc* d_blocks, int nb, int total_particles,
                           int* v2t, Status* st, cudaStream_t s);
void launch_circumcenters(const float4* pos, const int4* tv, int total_tets, float4* cc, cudaStream_t s);
void launch_circumcenters_f64(const float4* pos, const int4* tv, int total_tets, double* cc3, cudaStream_t s);

enum CellMode { CELL_COMPLETE = 0, CELL_VOLUME = 1, CELL_DENSE_TESS = 2, CELL_VOLUME_F64 = 3 };
// one warp per cell (the original particles of every block)
void launch_cells(int mode, const BlockDesc* d_blocks, const int* d_cell_off, int nb, int total_cells,
                  const float4* pos, const int4* tv, const int4* tn, const int* v2t, const float4* cc,
                  const double* cc64, const GridDesc& g, float* grid, int* out_i, float* out_f, float* out_area,
                  double* out_d, int* cell_counts, Status* st, cudaStream_t s);
void launch_cic(const BlockDesc* d_blocks, const int* d_cell_off, int nb, int total_cells, const float4* pos,
                const GridDesc& g, float* grid, Status* st, cudaStream_t s);
void launch_grid_max(const float* grid, long long n, float* d_max, cudaStream_t s);
void launch_reorder_neighbors(int* d_tets, int total_tets, Status* st, cudaStream_t s);
void launch_incomplete_cells(const BlockDesc* blocks, const int* c_off, int nb, int total_tets, int total_cells,
                             const float4* pos, const int4* tv, const int4* tn, const float* links6,
                             const int* link_off, const int* first_link, const unsigned long long* fill,
                             unsigned long long* masks, unsigned long long* counts, cudaStream_t s);
void launch_project_layers(const float* grid, int nx, int ny, const int* zs, int num_layers, float dz,
                           float* layers, cudaStream_t s);
void launch_sum_layers(const float* layers, int num_layers, long long area, float* out, cudaStream_t s);

// dtfe.cu  (built with -fmad=false; FMAs only where written)
void launch_star_volumes(int mode, int total_tets, const float4* pos, const int4* tv, StarSum* W,
                         double scale, float tau, Status* st, cudaStream_t s);
void launch_densities(const StarSum* W, int total_particles, float mass, double inv_scale, float* rho32,
                      double* rho64, Status* st, cudaStream_t s);
void launch_raster(int mode, int variant, const BlockDesc* d_blocks, int nb, int total_tets, const float4* pos,
                   const int4* tv, const float* rho32, const double* rho64, const GridDesc& g, float tau, float* grid,
                   int* owner, int* fix_list, int* fix_count, Status* st, cudaStream_t s,
                   const int* order = nullptr, const int* order_count = nullptr, int t0 = 0,
                   bool per_block = false, int* next = nullptr);   // next: zeroed chunk counter (persistent)
int  raster_variants();
void order_bricks(const GridDesc& g, int* nbx, int* nby, int* nbz);
void launch_tet_order(const float4* pos, const int4* tv, int total, const GridDesc& g, int* key, int* hist,
                      int* order, cudaStream_t s);
// brick rasteriser: bins of (tet, brick) pairs per segment of blocks, then
// one CTA per brick (dtfe.cu)
struct BrickBins
{
    int* cnt;                        // per brick: pairs
    int* off;                        // per brick: first pair in the pair list
    int* cur;                        // per brick: scatter cursor
    int* item_off;                   // per brick: first item within its segment
    int* seg_items;                  // per segment: items
    int* counters;                   // per segment: items taken by the rasteriser's CTAs
    int* pairs;                      // tet indices, brick by brick
    long long pair_cap;
    unsigned long long* pair_cursor; // pairs placed so far (all segments of a call)
};
int  brick_variants();
void brick_shape(int variant, int* sx, int* sy, int* sz);
void launch_bin_reset(const BrickBins& bins, int seg, int bb0, int bb1, cudaStream_t s);
// star volumes of tets [t0, t0 + nt) fused with their pair counts
void launch_star_bin(int mode, int variant, const BlockDesc* d_blocks, int nb, int t0, int nt, const float4* pos,
                     const int4* tv, StarSum* W, double scale, const GridDesc& g, int* cnt, Status* st,
                     cudaStream_t s);
// scan (pair and item offsets), scatter, zeroing of split bricks' regions
void launch_bin_place(int variant, const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1, int t0, int nt,
                      const float4* pos, const int4* tv, const GridDesc& g, const BrickBins& bins, float* grid,
                      Status* st, cudaStream_t s);
void launch_bin_bricks(int variant, const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1, int t0, int nt,
                       const float4* pos, const int4* tv, const GridDesc& g, const BrickBins& bins, float* grid,
                       Status* st, cudaStream_t s);
void launch_raster_bricks(int mode, int variant, const BlockDesc* d_blocks, int nb, int seg, int bb0, int bb1,
                          const BrickBins& bins, const float4* pos, const int4* tv, const float* rho32,
                          const double* rho64, const GridDesc& g, float* grid, int* owner, Status* st,
                          cudaStream_t s);
void launch_raster_fix(const BlockDesc* d_blocks, int nb, int total_tets, const float4* pos, const int4* tv,
                       const float* rho32, const double* rho64, const GridDesc& g, float* grid, int* owner,
                       const int* fix_list, const int* fix_count, Status* st, cudaStream_t s,
                       bool per_block = false);

}
