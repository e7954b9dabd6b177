/* Stand-in for tess2's include/tess/delaunay.hpp (test infrastructure):
   DBlock, the dblock_t plus its DIY bounds (include/tess/delaunay.hpp:18-23). */
#ifndef TESS_STANDIN_DELAUNAY_HPP
#define TESS_STANDIN_DELAUNAY_HPP
#include <diy/types.hpp>
#include "tess/delaunay.h"
struct DBlock : dblock_t
{
    diy::ContinuousBounds bounds { 3 };
    diy::ContinuousBounds data_bounds { 3 };
    diy::ContinuousBounds box { 3 };
};
#endif
