/* Stand-in for tess2's include/tess/tet-neighbors.h (test infrastructure): the
   declaration of complete (include/tess/tet-neighbors.h:19-26), C linkage. */
#ifndef TESS_STANDIN_TET_NEIGHBORS_H
#define TESS_STANDIN_TET_NEIGHBORS_H
#include "tess/tet.h"
#ifdef __cplusplus
extern "C"
#endif
int complete(int v, struct tet_t* tets, int num_tets, int t);
#endif
