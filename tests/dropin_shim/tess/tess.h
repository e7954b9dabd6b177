/* Stand-in for tess2's include/tess/tess.h (test infrastructure): the one
   declaration the drop-in defines, fill_vert_to_tet (include/tess/tess.h:63-66),
   with the reference's C linkage. */
#ifndef TESS_STANDIN_TESS_H
#define TESS_STANDIN_TESS_H
#include "tess/delaunay.h"
#ifdef __cplusplus
extern "C"
#endif
void fill_vert_to_tet(struct dblock_t* dblock);
#endif
