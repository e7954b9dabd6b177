/* Stand-in for tess2's include/tess/tet.hpp (test infrastructure). */
#ifndef TESS_STANDIN_TET_HPP
#define TESS_STANDIN_TET_HPP
#include "tet.h"
#endif
