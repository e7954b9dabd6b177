// tess2's density estimator on the GPU, as a drop-in for tess2's src/dense.cpp.
//
// A tess2 build compiles this file in place of src/dense.cpp (against its own
// include/tess headers, DIY and MPI) and links libtess2_gb300.so.  It defines
// the functions tess2's drivers call, with the reference's signatures:
//
//   dense()        include/tess/dense.hpp:75-89   (src/dense.cpp:30-103)
//   WriteGrid()    include/tess/dense.hpp:195-207 (src/dense.cpp:751-870)
//   dense_stats()  include/tess/dense.hpp:235-239 (src/dense.cpp:1284-1333)
//
// and keeps the process-wide statistics dense_stats() reports
// (max_dense, tot_mass, check_mass; src/dense.cpp:25-27).  The per-cell
// helpers of dense.hpp (CellBounds, CellGridPts, PtInCell, ...) run inside
// the GPU kernels and are not defined here.
//
// dense() fills each block's density array the way init_dense/est_dense/
// recvd_pts leave it: b->density = new float[b->num_grid_pts] over the
// block's BlockGridParams box (freed by tess2 with delete[]).  The estimator
// is the call's alg (DENSE_TESS or DENSE_CIC); TESS2_GB300_ESTIMATOR=dtfe in
// the environment selects the tet-linear DTFE estimator instead, and
// TESS2_GB300_MODE=fp64 its FP64 arithmetic.  TESS2_GB300_DEVICE picks the
// CUDA device (default: the MPI rank modulo the device count).
//
// Ranks: all blocks of a rank run in one GPU call.  With several ranks,
// DENSE_TESS and DENSE_CIC deposits that fall into other ranks' blocks are
// exchanged by summing the ranks' global grids (MPI_Allreduce), which is the
// reference's enqueue/exchange/recvd_pts in one step; DTFE writes only each
// block's own box and needs no exchange.  Projection (project with
// proj_plane (0,0,1), the one plane the reference's index() accepts) runs on
// one rank.  Errors print a message and call MPI_Abort, as the reference's
// fatal paths do.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <fcntl.h>
#include <unistd.h>
#include <cuda_runtime.h>

#include "tess/dense.hpp"
#include "tess2_gb300.h"

// process-wide statistics (src/dense.cpp:25-27): dense() sets them, dense_stats() reduces them
static float  max_dense = 0.0f;
static double tot_mass = 0.0;
static float  check_mass = 0.0f;

namespace {

tessgpu_ctx* g_ctx = nullptr;
int          g_alg = 0;            // the estimator of the last dense() call
tessgpu_dense_params g_params;     // and its parameters (WriteGrid needs the same grid)

void fatal(MPI_Comm comm, const char* what)
{
    fprintf(stderr, "dense (GPU): %s%s%s\n", what, g_ctx ? ": " : "", g_ctx ? tessgpu_last_error(g_ctx) : "");
    MPI_Abort(comm, 1);
}

tessgpu_ctx* context(MPI_Comm comm)
{
    if (g_ctx)
        return g_ctx;
    int rank = 0, dev = 0, ndev = 0;
    MPI_Comm_rank(comm, &rank);
    const char* env = getenv("TESS2_GB300_DEVICE");
    if (env && *env)
        dev = atoi(env);
    else if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0)
        dev = rank % ndev;
    if (tessgpu_create(dev, nullptr, &g_ctx) != TESSGPU_OK)
    {
        g_ctx = nullptr;
        fatal(comm, "no usable CUDA device");
    }
    return g_ctx;
}

bool env_is(const char* name, const char* value)
{
    const char* e = getenv(name);
    return e && std::strcmp(e, value) == 0;
}

// the blocks of this rank as tessgpu_block descriptors over tess2's own arrays
std::vector<tessgpu_block> local_blocks(diy::Master& master)
{
    std::vector<tessgpu_block> tb(master.size());
    for (size_t i = 0; i < master.size(); ++i)
    {
        DBlock* b = master.block<DBlock>((int)i);
        tessgpu_block& t = tb[i];
        std::memset(&t, 0, sizeof(t));
        t.gid = b->gid;
        for (int k = 0; k < 3; ++k)
        {
            t.bounds_min[k] = b->bounds.min[k];
            t.bounds_max[k] = b->bounds.max[k];
            t.data_min[k] = b->data_bounds.min[k];
            t.data_max[k] = b->data_bounds.max[k];
        }
        t.num_orig_particles = b->num_orig_particles;
        t.num_particles = b->num_particles;
        t.particles = b->particles;
        t.num_tets = b->num_tets;
        t.tets = reinterpret_cast<const int*>(b->tets);   // tet_t: int verts[4], tets[4]
        t.vert_to_tet = b->vert_to_tet;
    }
    return tb;
}

}  // namespace

// src/dense.cpp:30-103
void dense(alg alg_type, int num_given_bounds, float* given_mins, float* given_maxs, bool project,
           float* proj_plane, float mass, float* data_mins, float* data_maxs, float* grid_phys_mins,
           float* grid_phys_maxs, float* grid_step_size, float eps, int* glo_num_idx, diy::Master& master)
{
    MPI_Comm comm = master.communicator();
    int nranks = 1;
    MPI_Comm_size(comm, &nranks);
    tessgpu_ctx* ctx = context(comm);
    std::vector<tessgpu_block> tb = local_blocks(master);
    const int nb = (int)tb.size();

    // DataBounds (src/dense.cpp:1221-1275): the blocks' bounds, all-reduced
    float mn[3] = { 1e30f, 1e30f, 1e30f }, mx[3] = { -1e30f, -1e30f, -1e30f };
    for (int i = 0; i < nb; ++i)
        for (int k = 0; k < 3; ++k)
        {
            if (tb[i].bounds_min[k] < mn[k]) mn[k] = tb[i].bounds_min[k];
            if (tb[i].bounds_max[k] > mx[k]) mx[k] = tb[i].bounds_max[k];
        }
    MPI_Allreduce(mn, data_mins, 3, MPI_FLOAT, MPI_MIN, comm);
    MPI_Allreduce(mx, data_maxs, 3, MPI_FLOAT, MPI_MAX, comm);

    if (project && (proj_plane[0] != 0.0f || proj_plane[1] != 0.0f || proj_plane[2] != 1.0f))
        fatal(comm, "projection onto a plane other than x-y (the reference's index() asserts the x-y plane)");
    if (project && nranks > 1)
        fatal(comm, "projection runs on one rank");

    tessgpu_dense_params p;
    std::memset(&p, 0, sizeof(p));
    p.alg = env_is("TESS2_GB300_ESTIMATOR", "dtfe") ? TESSGPU_DENSE_DTFE
                                                    : (alg_type == DENSE_CIC ? TESSGPU_DENSE_CIC : TESSGPU_DENSE_TESS);
    p.mode = env_is("TESS2_GB300_MODE", "fp64") ? TESSGPU_MODE_FP64 : TESSGPU_MODE_MIXED;
    p.num_given_bounds = num_given_bounds;
    for (int k = 0; k < 3 && k < num_given_bounds; ++k)
    {
        p.given_mins[k] = given_mins[k];
        p.given_maxs[k] = given_maxs[k];
    }
    p.mass = mass;
    p.eps = eps;
    for (int k = 0; k < 3; ++k)
    {
        p.glo_num_idx[k] = glo_num_idx[k];
        p.data_mins[k] = data_mins[k];
        p.data_maxs[k] = data_maxs[k];
    }
    p.use_data_bounds = 1;
    p.project = project ? 1 : 0;
    g_alg = p.alg;
    g_params = p;

    // init_dense (src/dense.cpp:106-127): each block's array over its box
    std::vector<float*> arrays(nb > 0 ? nb : 1, nullptr);
    std::vector<int> box9(9 * (nb > 0 ? nb : 1));
    for (int i = 0; i < nb; ++i)
    {
        DBlock* b = master.block<DBlock>(i);
        const long long n = tessgpu_block_grid_points(nb, tb.data(), i, &p, &box9[9 * i]);
        delete[] b->density;
        b->density = new float[n > 0 ? n : 1];
        b->num_grid_pts = (int)(n > 0 ? n : 0);
        arrays[i] = b->density;
    }

    tessgpu_dense_info info;
    const bool exchange = nranks > 1 && p.alg != TESSGPU_DENSE_DTFE;
    if (!exchange)
    {
        if (tessgpu_dense(ctx, nb, tb.data(), &p, nullptr, arrays.data(), &info) != TESSGPU_OK)
            fatal(comm, "tessgpu_dense failed");
    }
    else
    {
        // deposits that land in other ranks' blocks: sum the ranks' global grids
        const size_t G = (size_t)glo_num_idx[0] * glo_num_idx[1] * glo_num_idx[2];
        std::vector<float> global(G);
        if (tessgpu_dense(ctx, nb, tb.data(), &p, global.data(), nullptr, &info) != TESSGPU_OK)
            fatal(comm, "tessgpu_dense failed");
        for (size_t off = 0; off < G; off += (1u << 30))
        {
            const int cnt = (int)std::min<size_t>(G - off, (size_t)1 << 30);
            MPI_Allreduce(MPI_IN_PLACE, global.data() + off, cnt, MPI_FLOAT, MPI_SUM, comm);
        }
        const size_t nx = glo_num_idx[0], ny = glo_num_idx[1];
        for (int i = 0; i < nb; ++i)
        {
            const int* mi = &box9[9 * i];
            const int* num = &box9[9 * i + 6];
            float* a = arrays[i];
            for (int z = 0; z < num[2]; ++z)
                for (int y = 0; y < num[1]; ++y)
                    std::memcpy(a + ((size_t)z * num[1] + y) * num[0],
                                global.data() + ((size_t)(mi[2] + z) * ny + (mi[1] + y)) * nx + mi[0],
                                sizeof(float) * num[0]);
        }
    }
    for (int k = 0; k < 3; ++k)
    {
        grid_phys_mins[k] = info.grid_phys_mins[k];
        grid_phys_maxs[k] = info.grid_phys_maxs[k];
        grid_step_size[k] = info.grid_step_size[k];
    }

    // this rank's statistics over its blocks' arrays
    const double dv = project ? (double)grid_step_size[0] * grid_step_size[1]
                              : (double)grid_step_size[0] * grid_step_size[1] * grid_step_size[2];
    max_dense = 0.0f;
    tot_mass = 0.0;
    for (int i = 0; i < nb; ++i)
        for (int j = 0; j < master.block<DBlock>(i)->num_grid_pts; ++j)
        {
            const float d = arrays[i][j];
            if (d > max_dense) max_dense = d;
            tot_mass += (double)d * dv;
        }
    if (p.alg == TESSGPU_DENSE_DTFE)
    {
        // the DTFE field integrates to the mass of the triangulated particles
        double m = 0.0;
        for (int i = 0; i < nb; ++i) m += (double)tb[i].num_orig_particles * mass;
        check_mass = (float)m;
    }
    else
        check_mass = (float)info.check_mass;
}

// src/dense.cpp:751-870: the global grid as raw native float32, x fastest
// ((nz, ny, nx), or (ny, nx) after ProjectGrid), the file truncated first
void WriteGrid(int mblocks, int tblocks, char* outfile, bool project, int* glo_num_idx, float eps, float* data_mins,
               float* data_maxs, int num_given_bounds, float* given_mins, float* given_maxs, diy::Master& master,
               diy::Assigner& assigner)
{
    (void)mblocks; (void)tblocks; (void)eps; (void)data_mins; (void)data_maxs; (void)num_given_bounds;
    (void)given_mins; (void)given_maxs; (void)assigner; (void)glo_num_idx;
    MPI_Comm comm = master.communicator();
    int nranks = 1, rank = 0;
    MPI_Comm_size(comm, &nranks);
    MPI_Comm_rank(comm, &rank);
    tessgpu_ctx* ctx = context(comm);
    if (nranks == 1)
    {
        // the last dense() call's global grid, projected when it projected
        if (tessgpu_write_last_grid(ctx, outfile) != TESSGPU_OK)
            fatal(comm, "WriteGrid failed");
        return;
    }
    if (project)
        fatal(comm, "projection runs on one rank");
    // every rank writes its blocks' boxes at their places in the file
    if (rank == 0)
    {
        const int fd = open(outfile, O_WRONLY | O_CREAT | O_TRUNC, 0644);
        if (fd < 0) fatal(comm, "cannot open the output file");
        close(fd);
    }
    MPI_Barrier(comm);
    const int fd = open(outfile, O_WRONLY);
    if (fd < 0) fatal(comm, "cannot open the output file");
    std::vector<tessgpu_block> tb = local_blocks(master);
    const size_t nx = g_params.glo_num_idx[0], ny = g_params.glo_num_idx[1];
    for (size_t i = 0; i < tb.size(); ++i)
    {
        int box9[9];
        tessgpu_block_grid_points((int)tb.size(), tb.data(), (int)i, &g_params, box9);
        const float* a = master.block<DBlock>((int)i)->density;
        for (int z = 0; z < box9[8]; ++z)
            for (int y = 0; y < box9[7]; ++y)
            {
                const size_t off = (((size_t)(box9[2] + z) * ny + (box9[1] + y)) * nx + box9[0]) * sizeof(float);
                const size_t len = sizeof(float) * box9[6];
                if (pwrite(fd, a + ((size_t)z * box9[7] + y) * box9[6], len, (off_t)off) != (ssize_t)len)
                    fatal(comm, "WriteGrid: write failed");
            }
    }
    close(fd);
    MPI_Barrier(comm);
}

// src/dense.cpp:1284-1333: the statistics of the last dense() call, reduced over the ranks
void dense_stats(double* times, diy::Master& master, float* grid_step_size, float* grid_phys_mins, int* glo_num_idx)
{
    MPI_Comm comm = master.communicator();
    int rank = 0;
    MPI_Comm_rank(comm, &rank);
    float glo_max_dense = 0.0f, glo_check_mass = 0.0f;
    double glo_tot_mass = 0.0;
    MPI_Reduce(&max_dense, &glo_max_dense, 1, MPI_FLOAT, MPI_MAX, 0, comm);
    MPI_Reduce(&tot_mass, &glo_tot_mass, 1, MPI_DOUBLE, MPI_SUM, 0, comm);
    MPI_Reduce(&check_mass, &glo_check_mass, 1, MPI_FLOAT, MPI_SUM, 0, comm);
    if (rank != 0)
        return;
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k)
    {
        lo[k] = grid_phys_mins[k];                                           // idx2phys of index 0
        hi[k] = (float)(glo_num_idx[k] - 1) * grid_step_size[k] + grid_phys_mins[k];
    }
    fprintf(stderr, "--------------Summary (GPU)--------------\n");
    fprintf(stderr, "Global 3D grid size = %d x %d x %d\n", glo_num_idx[0], glo_num_idx[1], glo_num_idx[2]);
    fprintf(stderr, "Physical grid extends from min [%.4e %.4e %.4e]\nto max [%.4e %.4e %.4e]\n"
                    "by steps of [%.4e %.4e %.4e]\n",
            lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], grid_step_size[0], grid_step_size[1], grid_step_size[2]);
    fprintf(stderr, "max_dense = %.3e tot_mass = %.3e (should be %.3e)\n", glo_max_dense, glo_tot_mass,
            glo_check_mass);
    fprintf(stderr, "Total time = %.3lf s = \n%.3lf s input + %.3lf s density computation + %.3lf s output\n",
            times[TOTAL_TIME], times[INPUT_TIME], times[COMP_TIME], times[OUTPUT_TIME]);
    fprintf(stderr, "-----------------------------------------\n");
}
