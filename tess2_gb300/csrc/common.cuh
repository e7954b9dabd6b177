// Shared device-side definitions of the tess2_gb300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/tess2_gb300.h"

namespace tg {

// Device layout of a batch of blocks (all blocks concatenated):
//   pos  float4[N]  particle x,y,z (w unused), blocks back to back
//   tv   int4[T]    tet vertices, global particle indices
//   tn   int4[T]    tet neighbours (tn.i opposite tv.i), global tet indices, -1 on the hull
//   v2t  int[N]     a tet containing each particle (the highest-numbered), -1 if none
//   cc   float4[T]  circumcenters (DENSE_TESS / volume only)
// the grid a block's DTFE rasteriser writes: grid positions x_i = i * step +
// gmin per axis, n points per axis, x fastest, starting at float offset off of
// the output (every block of a dense() call shares one grid; a batch of
// independent particle sets gives each set its own)
struct BlockGrid
{
    float     gmin[3], step[3], inv_step[3];
    int       n[3];
    long long off;
};

struct BlockDesc
{
    int   gid;
    float bmin[3], bmax[3];      // DBlock::bounds
    int   p_off, np, norig;      // first particle, particles, original particles
    int   t_off, nt;             // first tet, tets
    int   c_off;                 // first cell in the batch's cell numbering (original particles)
    int   gmin_idx[3], gmax_idx[3], gnum_idx[3];   // BlockGridParams of the current grid
    // DTFE brick rasteriser: the bricks covering the grid box, brick_n[0] x
    // brick_n[1] x brick_n[2] of them from brick coordinates brick_lo, numbered
    // from brick_base in the batch's brick numbering (x fastest)
    int   brick_base, brick_lo[3], brick_n[3];
    BlockGrid grid;
};

struct GridDesc
{
    float gmin[3];               // grid_phys_mins
    float step[3];               // grid_step_size
    float dmin[3], dmax[3];      // data bounds
    int   n[3];                  // glo_num_idx
    float eps, mass, div;        // eps, particle mass, step0*step1*step2
    float inv_step[3];           // 1 / step (index estimates only; exact checks follow)
    const int* zlayer;           // projected grid: layer of each z index (nullptr: 3-D grid)
};

// first failure wins; detail records the offending item
struct Status
{
    int code;
    int detail;
    unsigned long long fp64_tets;
    unsigned long long exact_tests;
    unsigned long long assigned;
    double tot_mass;
    unsigned long long check_mass;
    unsigned long long rows;        // DTFE: grid rows visited
    unsigned long long candidates;  // DTFE: grid points tested
    unsigned long long probes;      // DENSE_TESS: PtInCell calls of the scanline
    unsigned long long face_tests;  // DENSE_TESS: probes x faces of the cell
    int cell_next;                  // k_cells: the next cell a warp takes (zeroed per launch)
};

__device__ __forceinline__ void fail(Status* st, int code, int detail)
{
    if (atomicCAS(&st->code, 0, code) == 0)
        st->detail = detail;
}

// index of the block that holds item i given ascending offsets off[0..nb)
__device__ __forceinline__ int find_block(const int* off, int nb, int i)
{
    int lo = 0, hi = nb - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float3 ld3(const float4* pos, int i)
{
    float4 p = __ldg(&pos[i]);
    return make_float3(p.x, p.y, p.z);
}

__device__ __forceinline__ int4 ldtv(const int4* tv, int t) { return __ldg(&tv[t]); }
__device__ __forceinline__ int comp(const int4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

}  // namespace tg

// host-side launchers (one translation unit per kernel family)
namespace tg {
struct Batch;
struct Ctx;
}
