// Shared by the drop-in sources: the vertex count of a tet array, which
// tess2's per-vertex signatures do not carry (one more than the largest
// vertex index).
#pragma once
#include "tess/tet.h"

inline int tess2_gb300_vertex_count(const tet_t* tets, int num_tets)
{
    int n = 0;
    for (int t = 0; t < num_tets; ++t)
        for (int k = 0; k < 4; ++k)
            if (tets[t].verts[k] + 1 > n) n = tets[t].verts[k] + 1;
    return n;
}
