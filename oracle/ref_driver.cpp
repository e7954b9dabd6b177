// Test-only driver around the reference's own geometry and density code.
//
// oracle/Makefile compiles this file together with the reference's unmodified
// src/tet.cpp, src/volume.cpp and src/dense.cpp (against the single-rank
// MPI/DIY stand-ins in oracle/ref_shim/) into oracle/_ref/libtess_ref.so.
// The entry points below only marshal plain arrays into the reference's data
// model (dblock_t/DBlock, include/tess/delaunay.h:38-63, delaunay.hpp:18-23)
// and call the reference functions; every number they return is computed by
// the reference.  Nothing in the product links this library: it exists to
// generate golden vectors and to pin the restated oracle (tess_oracle.c).
#include <vector>
#include <cstdlib>
#include <cstring>
#include "tess/dense.hpp"
#include "tess/volume.h"

struct tess_shim_reduce_log tess_shim_reduce_record;

// same layout as tess_oracle.h's orc_block
struct ref_block
{
    int          gid;
    float        bounds_min[3], bounds_max[3];
    float        data_min[3], data_max[3];
    int          num_orig_particles;
    int          num_particles;
    const float* particles;     // 3 * num_particles
    int          num_tets;
    const int*   tets;          // 8 * num_tets: verts[4], tets[4] (tet_t)
    const int*   vert_to_tet;   // num_particles
};

static DBlock* make_dblock(const ref_block& rb)
{
    DBlock* b = new DBlock;
    std::memset(static_cast<dblock_t*>(b), 0, sizeof(dblock_t));
    b->gid = rb.gid;
    for (int i = 0; i < 3; ++i)
    {
        b->bounds.min[i] = rb.bounds_min[i];
        b->bounds.max[i] = rb.bounds_max[i];
        b->data_bounds.min[i] = rb.data_min[i];
        b->data_bounds.max[i] = rb.data_max[i];
    }
    b->num_orig_particles = rb.num_orig_particles;
    b->num_particles = rb.num_particles;
    b->particles = (float*)std::malloc(sizeof(float) * 3 * (rb.num_particles ? rb.num_particles : 1));
    std::memcpy(b->particles, rb.particles, sizeof(float) * 3 * rb.num_particles);
    b->num_tets = rb.num_tets;
    b->tets = (tet_t*)std::malloc(sizeof(tet_t) * (rb.num_tets ? rb.num_tets : 1));
    std::memcpy(b->tets, rb.tets, sizeof(tet_t) * rb.num_tets);
    b->vert_to_tet = (int*)std::malloc(sizeof(int) * (rb.num_particles ? rb.num_particles : 1));
    std::memcpy(b->vert_to_tet, rb.vert_to_tet, sizeof(int) * rb.num_particles);
    b->density = NULL;
    return b;
}

static void free_dblock(DBlock* b)
{
    std::free(b->particles);
    std::free(b->tets);
    std::free(b->vert_to_tet);
    delete[] b->density;
    delete b;
}

extern "C" {

// src/volume.cpp:6-11
void ref_fill_circumcenters(const float* particles, const int* tets, int num_tets, float* out)
{
    std::vector<float> cc;
    fill_circumcenters(cc, (tet_t*)tets, num_tets, (float*)particles);
    std::memcpy(out, cc.data(), sizeof(float) * 3 * (size_t)num_tets);
}

// src/tet.cpp:337-378 for every vertex; -1 where vert_to_tet is -1
void ref_complete_all(const int* tets, int num_tets, const int* vert_to_tet, int n, int* out)
{
    for (int v = 0; v < n; ++v)
        out[v] = vert_to_tet[v] < 0 ? -1 : complete(v, (tet_t*)tets, num_tets, vert_to_tet[v]);
}

// src/volume.cpp:13-54 for every vertex (the reference returns -1 for infinite cells)
void ref_volumes(int n, const int* vert_to_tet, const int* tets, int num_tets,
                 const float* particles, float* out)
{
    std::vector<float> cc;
    fill_circumcenters(cc, (tet_t*)tets, num_tets, (float*)particles);
    for (int v = 0; v < n; ++v)
        out[v] = vert_to_tet[v] < 0 ? -1.0f
               : volume(v, (int*)vert_to_tet, (tet_t*)tets, num_tets, (float*)particles, cc);
}

// src/tet.cpp:228-270; writes (u, ut) pairs, returns their count (or -count-1 past cap)
int ref_neighbor_edges(int v, const int* tets, int t, int* out_pairs, int cap, int* finite)
{
    std::vector< std::pair<int,int> > nbrs;
    *finite = neighbor_edges(nbrs, v, (tet_t*)tets, t) ? 1 : 0;
    int n = (int)nbrs.size();
    if (n > cap)
        return -n - 1;
    for (int i = 0; i < n; ++i)
    {
        out_pairs[2 * i] = nbrs[i].first;
        out_pairs[2 * i + 1] = nbrs[i].second;
    }
    return n;
}

// One cell of IterateCells (src/dense.cpp:245-268): complete test, CellBounds,
// CellGridPts.  Returns -1 for a skipped (incomplete) cell, 0 for a cell
// outside the data bounds, else the number of grid points, whose global
// indices and masses are written to idx (3 per point) and mass, up to cap.
int ref_cell_grid_pts(const ref_block* rb, int cell, const float* data_mins, const float* data_maxs,
                      const float* grid_phys_mins, const float* grid_step_size, float mass, float eps,
                      int* idx, double* pmass, int cap, float* cell_bounds6)
{
    DBlock* b = make_dblock(*rb);
    int result;
    if (b->vert_to_tet[cell] == -1 || !complete(cell, b->tets, b->num_tets, b->vert_to_tet[cell]))
        result = -1;
    else
    {
        float cell_min[3], cell_max[3];
        std::vector<float> normals;
        std::vector< std::vector<float> > face_verts;
        CellBounds(b, cell, cell_min, cell_max, normals, face_verts);
        if (cell_bounds6)
            for (int i = 0; i < 3; ++i) { cell_bounds6[i] = cell_min[i]; cell_bounds6[3 + i] = cell_max[i]; }
        grid_pt_t* grid_pts = NULL;
        int* border = NULL;
        int alloc = 0;
        result = CellGridPts(cell_min, cell_max, grid_pts, border, alloc, normals, face_verts,
                             (float*)data_mins, (float*)data_maxs, (float*)grid_phys_mins,
                             (float*)grid_step_size, mass, eps, &b->particles[3 * cell]);
        for (int i = 0; i < result && i < cap; ++i)
        {
            idx[3 * i] = grid_pts[i].idx[0];
            idx[3 * i + 1] = grid_pts[i].idx[1];
            idx[3 * i + 2] = grid_pts[i].idx[2];
            pmass[i] = grid_pts[i].mass;
        }
        std::free(grid_pts);
        std::free(border);
    }
    free_dblock(b);
    return result;
}

// The reference's dense() (src/dense.cpp:30-103) over nblocks blocks held in
// one process; every block links to every other block.  The per-block
// densities are placed at their BlockGridParams offsets in global_grid
// (x fastest, glo_num_idx[0]*glo_num_idx[1]*glo_num_idx[2] floats, zeroed
// here), which is the layout WriteGrid writes (src/dense.cpp:831-850).
// grid_out6 receives grid_phys_mins[3], grid_step_size[3]; data_out6 the data
// bounds; stats3 the values dense_stats() reduces: max_dense, tot_mass,
// check_mass (accumulated over all calls in this process, as in the reference).
static void add_blocks(diy::Master& master, std::vector<DBlock*>& dbs, int nblocks, const ref_block* blocks)
{
    for (int i = 0; i < nblocks; ++i)
    {
        DBlock* b = make_dblock(blocks[i]);
        RCLink* l = new RCLink;
        for (int j = 0; j < nblocks; ++j)
        {
            if (j == i) continue;
            diy::BlockID id { blocks[j].gid, 0 };
            l->neighbors.push_back(id);
            diy::ContinuousBounds cb(3);
            for (int d = 0; d < 3; ++d) { cb.min[d] = blocks[j].bounds_min[d]; cb.max[d] = blocks[j].bounds_max[d]; }
            l->cores.push_back(cb);
        }
        master.add(blocks[i].gid, b, l);
        dbs.push_back(b);
    }
}

void ref_dense(int alg_type, int nblocks, const ref_block* blocks,
               int num_given_bounds, const float* given_mins, const float* given_maxs,
               float mass, float eps, const int* glo_num_idx,
               float* global_grid, float* grid_out6, float* data_out6, double* stats3)
{
    diy::Master master;
    std::vector<DBlock*> dbs;
    add_blocks(master, dbs, nblocks, blocks);

    float gmins[3] = {0, 0, 0}, gmaxs[3] = {0, 0, 0};
    if (given_mins) for (int i = 0; i < 3; ++i) gmins[i] = given_mins[i];
    if (given_maxs) for (int i = 0; i < 3; ++i) gmaxs[i] = given_maxs[i];
    float proj_plane[3] = {0, 0, 1};
    float data_mins[3], data_maxs[3], grid_phys_mins[3], grid_phys_maxs[3], grid_step_size[3];
    int gni[3] = { glo_num_idx[0], glo_num_idx[1], glo_num_idx[2] };

    dense((alg)alg_type, num_given_bounds, gmins, gmaxs, false, proj_plane, mass,
          data_mins, data_maxs, grid_phys_mins, grid_phys_maxs, grid_step_size, eps, gni, master);

    size_t nx = gni[0], ny = gni[1];
    std::memset(global_grid, 0, sizeof(float) * nx * ny * (size_t)gni[2]);
    for (int i = 0; i < nblocks; ++i)
    {
        int bmin[3], bmax[3], bnum[3];
        BlockGridParams(dbs[i], bmin, bmax, bnum, grid_phys_mins, grid_step_size, eps,
                        data_mins, data_maxs, gni);
        for (int z = 0; z < bnum[2]; ++z)
            for (int y = 0; y < bnum[1]; ++y)
                for (int x = 0; x < bnum[0]; ++x)
                    global_grid[((size_t)(bmin[2] + z) * ny + (bmin[1] + y)) * nx + (bmin[0] + x)] =
                        dbs[i]->density[((size_t)z * bnum[1] + y) * bnum[0] + x];
    }
    for (int i = 0; i < 3; ++i)
    {
        grid_out6[i] = grid_phys_mins[i];
        grid_out6[3 + i] = grid_step_size[i];
        data_out6[i] = data_mins[i];
        data_out6[3 + i] = data_maxs[i];
    }

    tess_shim_reduce_record.n = 0;
    double times[DENSE_MAX_TIMES] = {0};
    dense_stats(times, master, grid_step_size, grid_phys_mins, gni);
    for (int i = 0; i < 3; ++i)
        stats3[i] = tess_shim_reduce_record.value[i];

    for (DBlock* b : dbs)
        free_dblock(b);
}

// dense() followed by WriteGrid (src/dense.cpp:751-870, which runs
// ProjectGrid, :881-1023, when projecting) to outfile, in the order
// examples/dense/main.cpp:170-181 calls them, on the x-y plane.  block_out
// (may be NULL) receives every block's density array as dense() leaves it
// (before ProjectGrid), concatenated in block order; its length is the sum of
// the blocks' b->num_grid_pts, which block_sizes (may be NULL) receives per
// block.  stats3 as ref_dense.  Block gids must be 0..nblocks-1 (ProjectGrid
// indexes its geometry table by gid).
void ref_dense_write(int alg_type, int nblocks, const ref_block* blocks,
                     int num_given_bounds, const float* given_mins, const float* given_maxs,
                     float mass, float eps, const int* glo_num_idx, int project, const char* outfile,
                     float* block_out, int* block_sizes, double* stats3)
{
    diy::Master master;
    std::vector<DBlock*> dbs;
    add_blocks(master, dbs, nblocks, blocks);
    diy::RoundRobinAssigner assigner(1, nblocks);

    float gmins[3] = {0, 0, 0}, gmaxs[3] = {0, 0, 0};
    if (given_mins) for (int i = 0; i < 3; ++i) gmins[i] = given_mins[i];
    if (given_maxs) for (int i = 0; i < 3; ++i) gmaxs[i] = given_maxs[i];
    float proj_plane[3] = {0, 0, 1};
    float data_mins[3], data_maxs[3], grid_phys_mins[3], grid_phys_maxs[3], grid_step_size[3];
    int gni[3] = { glo_num_idx[0], glo_num_idx[1], glo_num_idx[2] };

    dense((alg)alg_type, num_given_bounds, gmins, gmaxs, project != 0, proj_plane, mass,
          data_mins, data_maxs, grid_phys_mins, grid_phys_maxs, grid_step_size, eps, gni, master);

    size_t off = 0;
    for (int i = 0; i < nblocks; ++i)
    {
        if (block_sizes) block_sizes[i] = dbs[i]->num_grid_pts;
        if (block_out) std::memcpy(block_out + off, dbs[i]->density, sizeof(float) * dbs[i]->num_grid_pts);
        off += dbs[i]->num_grid_pts;
    }
    tess_shim_reduce_record.n = 0;
    double times[DENSE_MAX_TIMES] = {0};
    dense_stats(times, master, grid_step_size, grid_phys_mins, gni);
    for (int i = 0; i < 3; ++i)
        stats3[i] = tess_shim_reduce_record.value[i];

    WriteGrid(nblocks, nblocks, (char*)outfile, project != 0, gni, eps, data_mins, data_maxs,
              num_given_bounds, gmins, gmaxs, master, assigner);

    for (DBlock* b : dbs)
        free_dblock(b);
}

// side_of_plane (src/tet.cpp:70-119) on a box given as min xyz, max xyz
int ref_side_of_plane(const float* box6, const int* tet, const float* particles, int j)
{
    diy::ContinuousBounds box(3);
    for (int i = 0; i < 3; ++i) { box.min[i] = box6[i]; box.max[i] = box6[3 + i]; }
    return side_of_plane(box, (tet_t*)tet, (float*)particles, j);
}

// distance (src/tet.cpp:146-153)
float ref_distance(const float* u, const float* v)
{
    return distance((float*)u, (float*)v);
}

// BlockGridParams (src/dense.cpp:575-648) for one block
void ref_block_grid_params(const ref_block* rb, const float* grid_phys_mins, const float* grid_step_size,
                           float eps, const float* data_mins, const float* data_maxs, const int* glo_num_idx,
                           int* out9)
{
    DBlock* b = make_dblock(*rb);
    BlockGridParams(b, out9, out9 + 3, out9 + 6, (float*)grid_phys_mins, (float*)grid_step_size, eps,
                    (float*)data_mins, (float*)data_maxs, (int*)glo_num_idx);
    free_dblock(b);
}

}
