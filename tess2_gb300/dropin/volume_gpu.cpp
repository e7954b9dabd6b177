// tess2's Voronoi volume functions on the GPU, as a drop-in for tess2's
// src/volume.cpp (include/tess/volume.h:7-16):
//
//   fill_circumcenters(circumcenters, tets, num_tets, particles)
//   volume(v, verts_to_tets, tets, num_tets, particles, circumcenters)
//
// with the reference's signatures and bit-identical results.  volume() is
// called once per vertex (tools/draw.cpp:1235 loops over them), so the first
// call for a mesh computes every cell's volume in one GPU call and keeps
// them; later calls for the same arrays (the same pointers and sizes) read
// the kept values.  A caller that changes a mesh's arrays in place between
// calls calls tess2_gb300_forget_volumes() first.  The vertex count, which
// the signatures do not carry, is one more than the largest vertex index of
// the tets.
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "tess/volume.h"
#include "tess2_gb300.h"
#include "dropin_common.h"

namespace {

std::mutex g_mutex;
tessgpu_ctx* g_ctx = nullptr;
struct Kept
{
    const void *tets = nullptr, *particles = nullptr, *v2t = nullptr, *cc = nullptr;
    int num_tets = -1;
    std::vector<float> vol;
} g_kept;

tessgpu_ctx* context()
{
    if (!g_ctx && tessgpu_create(0, nullptr, &g_ctx) != TESSGPU_OK)
    {
        fprintf(stderr, "volume (GPU): no usable CUDA device\n");
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

extern "C" void tess2_gb300_forget_volumes()
{
    std::lock_guard<std::mutex> lock(g_mutex);
    g_kept = Kept();
}

// src/volume.cpp:6-11
void fill_circumcenters(std::vector<float>& circumcenters, tet_t* tets, int num_tets, float* particles)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    circumcenters.resize(3 * (size_t)num_tets);
    if (num_tets <= 0) return;
    check(tessgpu_fill_circumcenters(context(), particles, tess2_gb300_vertex_count(tets, num_tets),
                                     reinterpret_cast<const int*>(tets), num_tets, circumcenters.data()),
          "fill_circumcenters");
}

// src/volume.cpp:13-54: -1 for an infinite cell
float volume(int v, int* verts_to_tets, tet_t* tets, int num_tets, float* particles,
             const std::vector<float>& circumcenters)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_kept.tets != tets || g_kept.num_tets != num_tets || g_kept.particles != particles ||
        g_kept.v2t != verts_to_tets || g_kept.cc != circumcenters.data())
    {
        const int n = tess2_gb300_vertex_count(tets, num_tets);
        g_kept.vol.assign(n > 0 ? n : 1, -1.0f);
        if (n > 0)
            check(tessgpu_volumes(context(), particles, n, reinterpret_cast<const int*>(tets), num_tets,
                                  verts_to_tets, n, g_kept.vol.data(), nullptr),
                  "volume");
        g_kept.tets = tets;
        g_kept.num_tets = num_tets;
        g_kept.particles = particles;
        g_kept.v2t = verts_to_tets;
        g_kept.cc = circumcenters.data();
    }
    return v >= 0 && v < (int)g_kept.vol.size() ? g_kept.vol[v] : -1.0f;
}
