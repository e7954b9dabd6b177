// tess2's topology entry points on the GPU, with the reference's signatures
// and C linkage:
//
//   complete(v, tets, num_tets, t)   src/tet.cpp:337-378 (include/tess/tet-neighbors.h:19-26)
//   fill_vert_to_tet(dblock)         src/tess.cpp:767-787 (include/tess/tess.h:63-66)
//
// The reference defines them inside src/tet.cpp and src/tess.cpp among
// functions that stay on the host, so an integrating build compiles this
// file and leaves those two definitions out.
//
// complete() is called once per cell (src/dense.cpp:252), so the first call
// for a mesh (the same tets pointer and count) answers every vertex in one GPU
// call -- a tet per vertex from fill_vert_to_tet, then the star walk of each
// -- and later calls read the kept answers; tess2_gb300_forget_topology()
// drops them when a caller rewrites a mesh in place.  A vertex's answer does
// not depend on which of its tets the walk starts from, so the caller's t is
// not needed.  fill_vert_to_tet() keeps the reference's ownership: it
// reallocs dblock->vert_to_tet to num_particles ints and fills it (the last
// tet wins, -1 for a vertex in no tet), bit-identical.
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "tess/delaunay.h"
#include "tess/tess.h"
#include "tess/tet-neighbors.h"
#include "tess2_gb300.h"
#include "dropin_common.h"

namespace {

std::mutex g_mutex;
tessgpu_ctx* g_ctx = nullptr;
struct Kept
{
    const void* tets = nullptr;
    int num_tets = -1;
    std::vector<int> complete;
} g_kept;

tessgpu_ctx* context()
{
    if (!g_ctx && tessgpu_create(0, nullptr, &g_ctx) != TESSGPU_OK)
    {
        fprintf(stderr, "tess2 topology (GPU): no usable CUDA device\n");
        abort();
    }
    return g_ctx;
}

void check(tessgpu_status s, const char* what)
{
    if (s != TESSGPU_OK)
    {
        fprintf(stderr, "%s (GPU): %s\n", what, tessgpu_last_error(g_ctx));
        abort();
    }
}

}  // namespace

extern "C" void tess2_gb300_forget_topology()
{
    std::lock_guard<std::mutex> lock(g_mutex);
    g_kept = Kept();
}

// 1 when v's Voronoi cell is complete (no hull face in its star), else 0
extern "C" int complete(int v, tet_t* tets, int num_tets, int t)
{
    (void)t;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_kept.tets != tets || g_kept.num_tets != num_tets)
    {
        const int n = tess2_gb300_vertex_count(tets, num_tets);
        g_kept.complete.assign(n > 0 ? n : 1, 0);
        if (n > 0)
        {
            // the walk is topological: the positions only have to be valid floats
            std::vector<float> pos(3 * (size_t)n, 0.0f);
            std::vector<int> v2t(n);
            check(tessgpu_fill_vert_to_tet(context(), n, reinterpret_cast<const int*>(tets), num_tets, v2t.data()),
                  "complete");
            check(tessgpu_complete_all(context(), pos.data(), n, reinterpret_cast<const int*>(tets), num_tets,
                                       v2t.data(), n, g_kept.complete.data()),
                  "complete");
        }
        g_kept.tets = tets;
        g_kept.num_tets = num_tets;
    }
    return v >= 0 && v < (int)g_kept.complete.size() ? g_kept.complete[v] : 0;
}

extern "C" void fill_vert_to_tet(struct dblock_t* dblock)
{
    dblock->vert_to_tet = (int*)realloc(dblock->vert_to_tet, sizeof(int) * (size_t)dblock->num_particles);
    if (dblock->num_particles <= 0) return;
    std::lock_guard<std::mutex> lock(g_mutex);
    check(tessgpu_fill_vert_to_tet(context(), dblock->num_particles, reinterpret_cast<const int*>(dblock->tets),
                                   dblock->num_tets, dblock->vert_to_tet),
          "fill_vert_to_tet");
}
