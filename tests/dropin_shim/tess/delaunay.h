/* Stand-in for tess2's include/tess/delaunay.h (test infrastructure): the
   per-block record the drop-in reads and writes, with the fields of tess2's
   dblock_t (include/tess/delaunay.h:38-63) in its order. */
#ifndef TESS_STANDIN_DELAUNAY_H
#define TESS_STANDIN_DELAUNAY_H
#include "tess/tet.h"
struct dblock_t
{
    int gid;
    void* Dt;
    int num_orig_particles;
    int num_particles;
    float* particles;
    int num_tets;
    struct tet_t* tets;
    int* rem_gids;
    int* rem_lids;
    int* vert_to_tet;
    float* density;
    int num_grid_pts;
    int complete;
};
#endif
