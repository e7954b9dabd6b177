/* Stand-in for tess2's include/tess/volume.h (test infrastructure): the two
   prototypes of include/tess/volume.h:7-16. */
#ifndef TESS_STANDIN_VOLUME_H
#define TESS_STANDIN_VOLUME_H
#include <vector>
#include "tet.hpp"
void fill_circumcenters(std::vector<float>& circumcenters, tet_t* tets, int num_tets, float* particles);
float volume(int v, int* verts_to_tets, tet_t* tets, int num_tets, float* particles,
             const std::vector<float>& circumcenters);
#endif
