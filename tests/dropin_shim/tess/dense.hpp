/* Stand-in for tess2's include/tess/dense.hpp (test infrastructure): the
   estimator enum, the timing slots and the driver-level prototypes the
   drop-in defines (include/tess/dense.hpp:33-38, 63-89, 195-207, 235-239). */
#ifndef TESS_STANDIN_DENSE_HPP
#define TESS_STANDIN_DENSE_HPP
#include <vector>
#include "mpi.h"
#include <diy/master.hpp>
#include <diy/assigner.hpp>
#include "tess/delaunay.hpp"
enum alg { DENSE_TESS, DENSE_CIC, DENSE_NUM_ALGS };
enum { INPUT_TIME, COMP_TIME, OUTPUT_TIME, TOTAL_TIME, TESS_TIME, DENSE_MAX_TIMES };
void dense(alg alg_type, int num_given_bounds, float* given_mins, float* given_maxs, bool project,
           float* proj_plane, float mass, float* data_mins, float* data_maxs, float* grid_phys_mins,
           float* grid_phys_maxs, float* grid_step_size, float eps, int* glo_num_idx, diy::Master& master);
void WriteGrid(int mblocks, int tblocks, char* outfile, bool project, int* glo_num_idx, float eps, float* data_mins,
               float* data_maxs, int num_given_bounds, float* given_mins, float* given_maxs, diy::Master& master,
               diy::Assigner& assigner);
void dense_stats(double* times, diy::Master& master, float* grid_step_size, float* grid_phys_mins, int* glo_num_idx);
#endif
