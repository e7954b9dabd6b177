/* Stand-in for tess2's include/tess/tet.h (test infrastructure): the tet_t
   record the drop-in test builds blocks from, laid out as tess2's is
   (include/tess/tet.h:4-7): tets[i] lies opposite verts[i], -1 on the hull. */
#ifndef TESS_STANDIN_TET_H
#define TESS_STANDIN_TET_H
struct tet_t
{
    int verts[4];
    int tets[4];
};
#endif
