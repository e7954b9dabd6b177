// Test driver of the compiled drop-in (tess2_gb300/dropin/*.cpp): builds
// tess2-style blocks (DBlock in a single-rank DIY master) from plain arrays
// and calls the drop-in exactly as tess2's examples/dense/main.cpp does --
// dense(), WriteGrid(), dense_stats() -- then hands the blocks' density
// arrays back.  Test infrastructure only.
#include <cstdlib>
#include <cstring>
#include <vector>
#include "tess/dense.hpp"
#include "tess/tess.h"
#include "tess/tet-neighbors.h"
#include "tess/volume.h"

struct tess_shim_reduce_log tess_shim_reduce_record;

// same layout as tess_oracle.h's orc_block
struct drop_block
{
    int          gid;
    float        bounds_min[3], bounds_max[3];
    float        data_min[3], data_max[3];
    int          num_orig_particles;
    int          num_particles;
    const float* particles;
    int          num_tets;
    const int*   tets;
    const int*   vert_to_tet;
};

extern "C" {

// dense() + WriteGrid() over nb blocks; block b's array goes to
// block_out + offset (sizes[b] floats each, in block order); stats3 =
// grid_phys_mins, grid_step_size (6 floats)
int dropin_dense(int alg_type, int nb, const drop_block* blocks, const int* glo_num_idx, float mass, float eps,
                 int project, const char* outfile, float* block_out, long long cap, int* sizes, float* grid6)
{
    diy::Master master;
    std::vector<DBlock*> own;
    for (int i = 0; i < nb; ++i)
    {
        const drop_block& r = blocks[i];
        DBlock* b = new DBlock;
        std::memset(static_cast<dblock_t*>(b), 0, sizeof(dblock_t));
        b->gid = r.gid;
        for (int k = 0; k < 3; ++k)
        {
            b->bounds.min[k] = r.bounds_min[k];
            b->bounds.max[k] = r.bounds_max[k];
            b->data_bounds.min[k] = r.data_min[k];
            b->data_bounds.max[k] = r.data_max[k];
        }
        b->num_orig_particles = r.num_orig_particles;
        b->num_particles = r.num_particles;
        b->particles = (float*)std::malloc(sizeof(float) * 3 * (r.num_particles ? r.num_particles : 1));
        std::memcpy(b->particles, r.particles, sizeof(float) * 3 * r.num_particles);
        b->num_tets = r.num_tets;
        b->tets = (tet_t*)std::malloc(sizeof(tet_t) * (r.num_tets ? r.num_tets : 1));
        std::memcpy(b->tets, r.tets, sizeof(tet_t) * r.num_tets);
        b->vert_to_tet = (int*)std::malloc(sizeof(int) * (r.num_particles ? r.num_particles : 1));
        std::memcpy(b->vert_to_tet, r.vert_to_tet, sizeof(int) * r.num_particles);
        b->density = NULL;
        master.add(r.gid, b, new diy::Link);
        own.push_back(b);
    }
    float data_mins[3], data_maxs[3], gmin[3], gmax[3], step[3];
    float proj_plane[3] = { 0.0f, 0.0f, 1.0f };
    int gni[3] = { glo_num_idx[0], glo_num_idx[1], glo_num_idx[2] };
    dense((alg)alg_type, 0, NULL, NULL, project != 0, proj_plane, mass, data_mins, data_maxs, gmin, gmax, step,
          eps, gni, master);
    diy::RoundRobinAssigner assigner(1, nb);
    if (outfile)
        WriteGrid(nb, nb, (char*)outfile, project != 0, gni, eps, data_mins, data_maxs, 0, NULL, NULL, master,
                  assigner);
    double times[DENSE_MAX_TIMES] = { 0 };
    dense_stats(times, master, step, gmin, gni);
    long long off = 0;
    int rc = 0;
    for (int i = 0; i < nb; ++i)
    {
        sizes[i] = own[i]->num_grid_pts;
        if (off + sizes[i] > cap) { rc = 1; break; }
        std::memcpy(block_out + off, own[i]->density, sizeof(float) * sizes[i]);
        off += sizes[i];
    }
    for (int k = 0; k < 3; ++k) { grid6[k] = gmin[k]; grid6[3 + k] = step[k]; }
    for (DBlock* b : own)
    {
        std::free(b->particles);
        std::free(b->tets);
        std::free(b->vert_to_tet);
        delete[] b->density;
        delete b;
    }
    return rc;
}

// fill_circumcenters() then volume() of every vertex, as tools/draw.cpp calls them
// complete() for every vertex, then fill_vert_to_tet() on a block made from the arrays
void dropin_topology(const float* particles, int np, const int* tets, int nt, const int* v2t, int* complete_out,
                     int* v2t_out)
{
    for (int v = 0; v < np; ++v) complete_out[v] = v2t[v] < 0 ? 0 : complete(v, (tet_t*)tets, nt, v2t[v]);
    dblock_t b;
    std::memset(&b, 0, sizeof(b));
    b.num_particles = np;
    b.particles = (float*)particles;
    b.num_tets = nt;
    b.tets = (tet_t*)tets;
    b.vert_to_tet = (int*)std::malloc(sizeof(int));   // fill_vert_to_tet reallocs it, as the reference does
    fill_vert_to_tet(&b);
    std::memcpy(v2t_out, b.vert_to_tet, sizeof(int) * (size_t)np);
    std::free(b.vert_to_tet);
}

void dropin_volumes(const float* particles, int np, const int* tets, int nt, const int* v2t, float* cc_out,
                    float* vol_out)
{
    std::vector<float> cc;
    fill_circumcenters(cc, (tet_t*)tets, nt, (float*)particles);
    std::memcpy(cc_out, cc.data(), sizeof(float) * 3 * (size_t)nt);
    for (int v = 0; v < np; ++v)
        vol_out[v] = v2t[v] < 0 ? -1.0f : volume(v, (int*)v2t, (tet_t*)tets, nt, (float*)particles, cc);
}

}
