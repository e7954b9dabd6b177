/*
 * tess2_gb300 — GB300 (sm_103a) implementation of tess2's post-Delaunay
 * geometry and density-estimation path, behind a plain C ABI.
 *
 * Everything here takes plain pointers and sizes.  Two families:
 *
 *  - Host-buffer entry points (tessgpu_fill_vert_to_tet, ..., tessgpu_dense):
 *    the calls a tess2 caller makes where it calls the reference today.  They
 *    take the same arrays as the reference functions they replace (cited on
 *    each), copy them to the GPU, run, and copy results back.
 *
 *  - Device-resident batches (tessgpu_batch_*): blocks whose particles and
 *    tets already live in GPU memory, for in-situ callers and for timing
 *    the kernels without host copies.
 *
 * Tets use tess2's tet_t layout (include/tess/tet.h:4-7 in the reference):
 * int verts[4]; int tets[4]; where tets[i] is the neighbour opposite
 * verts[i] and -1 marks the convex hull.  Particles are float x,y,z triples.
 * Density grids are float32, x fastest, as WriteGrid writes them
 * (src/dense.cpp:831-850).
 *
 * Errors: every call returns a tessgpu_status; tessgpu_last_error() gives a
 * message.  Device-side failures (a star or edge ring larger than the
 * kernel's bound, malformed adjacency) are reported through a status word the
 * kernels write; kernels never trap and every device loop is bounded.
 */
#ifndef TESS2_GB300_H
#define TESS2_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tessgpu_status
{
    TESSGPU_OK                 = 0,
    TESSGPU_ERR_INVALID        = 1,   /* bad argument */
    TESSGPU_ERR_CUDA           = 2,   /* CUDA runtime error (message in tessgpu_last_error) */
    TESSGPU_ERR_NO_DEVICE      = 3,
    TESSGPU_ERR_STAR_OVERFLOW  = 4,   /* a vertex star exceeded TESSGPU_MAX_STAR tets */
    TESSGPU_ERR_FACE_OVERFLOW  = 5,   /* a Voronoi cell exceeded TESSGPU_MAX_FACES faces */
    TESSGPU_ERR_LINK_OVERFLOW  = 6,   /* an edge ring exceeded TESSGPU_MAX_LINK tets */
    TESSGPU_ERR_BAD_MESH       = 7,   /* an index out of range or a broken adjacency */
    TESSGPU_ERR_UNSUPPORTED    = 8,
    TESSGPU_ERR_IO             = 9,   /* a file could not be opened or written */
    TESSGPU_ERR_TIMEOUT        = 10,  /* a bounded wait inside a kernel ran out */
    TESSGPU_ERR_CAPACITY       = 11   /* a device work list outgrew its buffer (the DTFE
                                         calls retry once with a larger one) */
} tessgpu_status;

/* bounds of the device loops; larger inputs report the overflow codes */
#define TESSGPU_MAX_STAR   512
#define TESSGPU_MAX_FACES  128
#define TESSGPU_MAX_LINK   256

/* density estimators: DENSE_TESS and DENSE_CIC keep the reference's enum
   values (include/tess/dense.hpp:33-38); DTFE is the tet-linear estimator */
typedef enum tessgpu_alg
{
    TESSGPU_DENSE_TESS = 0,
    TESSGPU_DENSE_CIC  = 1,
    TESSGPU_DENSE_DTFE = 2
} tessgpu_alg;

/* arithmetic of the DTFE path */
typedef enum tessgpu_mode
{
    TESSGPU_MODE_MIXED = 0,   /* FP32 geometry, FP64 fix-up of ill-conditioned tets */
    TESSGPU_MODE_FP64  = 1    /* every geometric quantity in FP64 */
} tessgpu_mode;

typedef struct tessgpu_ctx tessgpu_ctx;
typedef struct tessgpu_batch tessgpu_batch;

/* One DIY block: dblock_t (include/tess/delaunay.h:38-63) plus the DBlock
   bounds (include/tess/delaunay.hpp:18-23).  Pointers are host memory for
   the host-buffer calls and device memory for tessgpu_batch_wrap_device. */
typedef struct tessgpu_block
{
    int          gid;
    float        bounds_min[3], bounds_max[3];       /* DBlock::bounds */
    float        data_min[3], data_max[3];           /* DBlock::data_bounds */
    int          num_orig_particles;
    int          num_particles;
    const float* particles;                          /* 3 * num_particles */
    int          num_tets;
    const int*   tets;                               /* 8 * num_tets (tet_t) */
    const int*   vert_to_tet;                        /* num_particles, or NULL: computed on the GPU */
} tessgpu_block;

/* Grid and estimator parameters of dense() (src/dense.cpp:30-44). */
typedef struct tessgpu_dense_params
{
    int   alg;                  /* tessgpu_alg */
    int   mode;                 /* tessgpu_mode (DTFE only) */
    int   num_given_bounds;     /* 0..3 */
    float given_mins[3], given_maxs[3];
    float mass;                 /* mass of one particle */
    float eps;                  /* floating point tolerance (the reference's drivers use 1e-4) */
    int   glo_num_idx[3];       /* global grid points per axis */
    int   use_data_bounds;      /* 1: data_mins/maxs below are the data bounds (DataBounds'
                                   all-reduce over every rank's blocks); 0: the union of the
                                   given blocks' bounds, as DataBounds computes on one rank */
    float data_mins[3], data_maxs[3];
    int   project;              /* 1: project onto the x-y plane (dense()'s project with
                                   proj_plane (0,0,1), the one plane the reference's
                                   index() supports, src/dense.cpp:1077): densities are
                                   mass per area, summed over z (see tessgpu_project_grid) */
} tessgpu_dense_params;

/* Outputs of dense() besides the grid (src/dense.cpp:37-43, 1294-1300). */
typedef struct tessgpu_dense_info
{
    float  data_mins[3], data_maxs[3];
    float  grid_phys_mins[3], grid_phys_maxs[3], grid_step_size[3];
    double max_dense;           /* largest grid density */
    double tot_mass;            /* total deposited mass */
    double check_mass;          /* cells that deposited (DENSE_TESS) or particles (DENSE_CIC) */
    long long grid_pts_assigned;/* DTFE: grid points inside some tet */
    long long fp64_tets;        /* DTFE mixed: tets recomputed in FP64 */
    long long exact_tests;      /* DTFE: point-in-tet tests decided by exact arithmetic */
    long long rows_visited;     /* DTFE: grid rows the rasteriser examined */
    long long points_tested;    /* DTFE: grid points the rasteriser classified */
    int       raster_variant;   /* DTFE: launch configuration the autotuner chose for this batch */
    float     raster_variant_ms[8]; /* DTFE: the autotuner's best time of each configuration (0 if not run) */
    int       grid_layers;      /* project: z layers of the device grid; 0 for a 3-D grid */
    long long grid_floats;      /* floats of the device grid tessgpu_batch_dense wrote */
    long long cell_probes;      /* DENSE_TESS: PtInCell calls of the scanline (src/dense.cpp:1475-1701) */
    long long face_tests;       /* DENSE_TESS: face-plane tests of those calls (probes x faces) */
    long long brick_pairs;      /* DTFE, brick rasteriser: (tet, brick) candidate pairs binned */
} tessgpu_dense_info;

/* ---- context ---------------------------------------------------------- */

/* Create a context on a CUDA device; stream may be NULL (the legacy default
   stream) or a cudaStream_t the caller owns.  A context and its batches are
   used by one host thread at a time: its calls share a status word and
   scratch buffers on the device (threads that work concurrently make one
   context each). */
tessgpu_status tessgpu_create(int device, void* stream, tessgpu_ctx** out);
void           tessgpu_destroy(tessgpu_ctx* ctx);
const char*    tessgpu_last_error(const tessgpu_ctx* ctx);
tessgpu_status tessgpu_sync(tessgpu_ctx* ctx);
/* number of kernel launches issued by this context so far */
long long      tessgpu_launch_count(const tessgpu_ctx* ctx);

/* Stage timing: when on, every dense call records CUDA events on the
   context's stream between its stages; tessgpu_stage_times then returns up to
   cap (name, milliseconds) pairs of the last call (after it has finished).
   When a DTFE batch runs its blocks on two streams (TESSGPU_BATCH_OVERLAP=1;
   by default each stage runs over all blocks in one launch), the per-stage
   entries are sums over the blocks of spans timed on each block's stream,
   which overlap one another; the pipelined host-buffer DTFE call reports its
   upload, compute and download spans the same way. */
tessgpu_status tessgpu_set_timing(tessgpu_ctx* ctx, int on);
int            tessgpu_stage_times(tessgpu_ctx* ctx, const char** names, float* ms, int cap);

/* ---- host-buffer entry points ----------------------------------------- */

/* replaces fill_vert_to_tet (src/tess.cpp:767-787): for each vertex the
   highest-numbered tet that contains it, -1 for none */
tessgpu_status tessgpu_fill_vert_to_tet(tessgpu_ctx* ctx, int num_particles, const int* tets,
                                        int num_tets, int* vert_to_tet);

/* replaces fill_circumcenters (src/volume.cpp:6-11) and circumcenter
   (src/tet.cpp:37-66): 3 floats per tet, bit-identical to the reference */
tessgpu_status tessgpu_fill_circumcenters(tessgpu_ctx* ctx, const float* particles, int num_particles,
                                          const int* tets, int num_tets, float* circumcenters);

/* replaces reorder_neighbors (src/tess-qhull.c:161-225), run after Qhull's
   output is copied into tet_t records: reorders each tet's four neighbours in
   place so that tets[i] lies opposite verts[i] (-1 on the hull). */
tessgpu_status tessgpu_reorder_neighbors(tessgpu_ctx* ctx, int* tets, int num_tets);
/* the same on tet_t records already in device memory */
tessgpu_status tessgpu_reorder_neighbors_device(tessgpu_ctx* ctx, int* d_tets, int num_tets);

/* One neighbour link of a block (an RCLink entry, include/tess/tess.hpp):
   the neighbour's core bounds and its wrap direction (-1, 0 or 1 per axis;
   all 0 without periodic boundaries), applied as DIY's wrap_bounds does:
   bounds += wrap * (data_max - data_min) of the block's data bounds. */
typedef struct tessgpu_link
{
    float bounds_min[3], bounds_max[3];
    int   wrap[3];
} tessgpu_link;

/* replaces incomplete_cells (src/tess.cpp:492-628), the per-tet step that
   picks the particles a block sends to its neighbours in tess2's ghost
   exchange rounds, for one block with num_links <= 64 links, testing links
   [last_neighbor, num_links).  send_mask[p] for each original particle p:
   bit i set when the reference's to_send[p] holds link i.  enqueued (may be
   NULL) receives the number of (particle, link) pairs, its return value.  A
   block without tets sends every original particle to every tested link, as
   the reference's release builds do (its debug builds assert that each such
   particle lies in a tet). */
tessgpu_status tessgpu_incomplete_cells(tessgpu_ctx* ctx, const tessgpu_block* block, int num_links,
                                        const tessgpu_link* links, int last_neighbor,
                                        unsigned long long* send_mask, long long* enqueued);

/* replaces complete (src/tet.cpp:337-378) for vertices [0, n): 1 finite
   Voronoi cell, 0 cell on the hull, -1 where vert_to_tet is -1 */
tessgpu_status tessgpu_complete_all(tessgpu_ctx* ctx, const float* particles, int num_particles,
                                    const int* tets, int num_tets, const int* vert_to_tet,
                                    int n, int* out);

/* replaces volume (src/volume.cpp:13-54) for vertices [0, n): Voronoi cell
   volume bit-identical to the reference, -1 for infinite cells or vertices
   in no tet.  areas (optional, may be NULL) receives the Voronoi cell's total
   face area. */
tessgpu_status tessgpu_volumes(tessgpu_ctx* ctx, const float* particles, int num_particles,
                               const int* tets, int num_tets, const int* vert_to_tet,
                               int n, float* volumes, float* areas);

/* FP64 Voronoi cell volumes for vertices [0, n) (-1 for infinite cells). */
tessgpu_status tessgpu_volumes_f64(tessgpu_ctx* ctx, const float* particles, int num_particles,
                                   const int* tets, int num_tets, const int* vert_to_tet,
                                   int n, double* volumes);

/* replaces dense (src/dense.cpp:30-103) over nblocks blocks.  global_grid
   (may be NULL) receives the whole grid, glo_num_idx[0]*[1]*[2] floats, x
   fastest (what WriteGrid writes); with params->project it receives the
   projected glo_num_idx[0]*[1] floats after ProjectGrid's sum over z, which
   is what WriteGrid writes then.  block_density (may be NULL) is an array of
   nblocks host pointers; block b's array must hold
   tessgpu_block_grid_points(...) floats and receives that block's density as
   init_dense/est_dense/recvd_pts leave it (projected: the block's own z range
   only, before ProjectGrid).  info may be NULL. */
tessgpu_status tessgpu_dense(tessgpu_ctx* ctx, int nblocks, const tessgpu_block* blocks,
                             const tessgpu_dense_params* params, float* global_grid,
                             float** block_density, tessgpu_dense_info* info);

/* BlockGridParams (src/dense.cpp:575-648) of block b for the grid that
   dense() derives from params; writes min_idx[3], max_idx[3], num_idx[3] to
   out9 and returns the block's number of grid points (num_idx[0]*num_idx[1]
   when projecting, as init_dense allocates, src/dense.cpp:118-121). */
long long      tessgpu_block_grid_points(int nblocks, const tessgpu_block* blocks, int b,
                                         const tessgpu_dense_params* params, int* out9);

/* ---- device-resident batches ------------------------------------------ */

/* Copy nblocks host blocks to the GPU once (particles, tets, vert_to_tet). */
tessgpu_status tessgpu_batch_upload(tessgpu_ctx* ctx, int nblocks, const tessgpu_block* blocks,
                                    tessgpu_batch** out);
/* Wrap blocks whose particles/tets (and optionally vert_to_tet) pointers are
   device memory; nothing is copied and the caller keeps ownership. */
tessgpu_status tessgpu_batch_wrap_device(tessgpu_ctx* ctx, int nblocks, const tessgpu_block* blocks,
                                         tessgpu_batch** out);
void           tessgpu_batch_free(tessgpu_batch* batch);

/* dense() on a device batch into a device grid (d_grid: glo_num_idx product
   floats, x fastest).  Nothing is copied to or from the host except info.
   With params->project, d_grid holds L layers of glo_num_idx[0]*[1] floats,
   one per distinct z range of the blocks' BlockGridParams boxes (layer 0 the
   lowest): layer l holds what the blocks of that z range hold after dense()
   and before ProjectGrid; tessgpu_project_grid sums them. */
tessgpu_status tessgpu_batch_dense(tessgpu_ctx* ctx, tessgpu_batch* batch,
                                   const tessgpu_dense_params* params, float* d_grid,
                                   tessgpu_dense_info* info);

/* ---- independent particle sets ---------------------------------------- */

/* Floats of the output of tessgpu_batch_dense_sets for nsets sets whose grids
   have glo_num_idx[3b..3b+2] points; offsets (may be NULL) receives each set's
   first float.  -1 for a grid with fewer than 2 points on an axis. */
long long      tessgpu_sets_grid_floats(int nsets, const int* glo_num_idx, long long* offsets);

/* DTFE of many independent particle sets at once: every block of the batch is
   one set, processed as dense() over that block alone (its bounds are the data
   bounds) onto its own grid of glo_num_idx[3b..3b+2] points, written to device
   memory d_out + offsets[b] (tessgpu_sets_grid_floats), x fastest.  The
   reference runs DIY blocks independently through master.foreach
   (src/dense.cpp:130-164); here all sets share each stage's launch, and one
   rasteriser launch covers every set: the row kernel over all sets' tets, or,
   in a context made with TESSGPU_RASTER=bricks, the persistent brick kernel
   whose CTAs take (brick, chunk) items of every set from one device counter.
   graph != 0: the step is recorded into
   a CUDA graph on the first call with these sets, grids and output, and
   replayed by later calls (the brick shape is autotuned on the first call of
   a context, outside the graph).  The batch's descriptors must not change
   while it keeps a recorded step.  info may be NULL. */
tessgpu_status tessgpu_batch_dense_sets(tessgpu_ctx* ctx, tessgpu_batch* batch, const int* glo_num_idx,
                                        float mass, float eps, int mode, float* d_out, int graph,
                                        tessgpu_dense_info* info);

/* incomplete_cells for every block of a device batch: block b's links are
   links[link_offsets[b] .. link_offsets[b+1]) (host arrays, at most 64 per
   block), tested from last_neighbor[b] (NULL: all from 0); d_send_mask
   (device) receives one mask per original particle of the batch, blocks in
   order; enqueued (host, may be NULL) one count per block. */
tessgpu_status tessgpu_batch_incomplete_cells(tessgpu_ctx* ctx, tessgpu_batch* batch, const int* link_offsets,
                                              const tessgpu_link* links, const int* last_neighbor,
                                              unsigned long long* d_send_mask, long long* enqueued);

/* floats d_grid of tessgpu_batch_dense needs for these blocks and params, and
   (layers, may be NULL) its number of z layers: 0 for a 3-D grid */
long long      tessgpu_dense_grid_floats(int nblocks, const tessgpu_block* blocks,
                                         const tessgpu_dense_params* params, int* layers);

/* ---- output: ProjectGrid and WriteGrid -------------------------------- */

/* ProjectGrid (src/dense.cpp:881-1023) on device memory: d_out[i] is the sum
   over l = 0 .. num_layers-1, in that order, of d_layers[l * layer_floats + i]
   (the z=0 block of each column adds the blocks above it in block order). */
tessgpu_status tessgpu_project_grid(tessgpu_ctx* ctx, const float* d_layers, int num_layers,
                                    long long layer_floats, float* d_out);

/* WriteGrid's file (src/dense.cpp:751-870): num_floats floats of device
   memory written to path as raw native float32 in the given order (x
   fastest for a grid), the file truncated first.  The data goes device ->
   pinned staging buffers -> file; the copy of one chunk overlaps the write
   of the previous one.  Fails with TESSGPU_ERR_IO. */
tessgpu_status tessgpu_write_grid(tessgpu_ctx* ctx, const float* d_grid, long long num_floats,
                                  const char* path);

/* WriteGrid as tess2 calls it after dense(): writes the global grid of this
   context's last tessgpu_dense call, projected when that call projected. */
tessgpu_status tessgpu_write_last_grid(tessgpu_ctx* ctx, const char* path);

/* Validation outputs of the last tessgpu_batch_dense call, copied to host:
   cell_counts (DENSE_TESS: per original particle of every block in order,
   the reference's CellGridPts result, -1 for a skipped cell), owner (DTFE:
   the block-local tet index that holds each grid point, -1 for none),
   rho (DTFE: per particle of every block in order).  Each may be NULL;
   sizes are the caller's to know.  Requires tessgpu_batch_keep_debug(batch, 1)
   before the tessgpu_batch_dense call. */
tessgpu_status tessgpu_batch_keep_debug(tessgpu_batch* batch, int on);
tessgpu_status tessgpu_batch_debug_outputs(tessgpu_ctx* ctx, tessgpu_batch* batch, int* cell_counts,
                                           int* owner, float* rho);

/* ---- allocation-free entry point -------------------------------------- */

/* Largest particle count tessgpu_dtfe_densities_noalloc accepts: its scratch
   is a fixed 32 MiB array inside the library (two 64-bit words per particle). */
#define TESSGPU_NOALLOC_MAX_PARTICLES (1 << 21)

/* DTFE vertex densities of one block (rho_v = 4 m / star volume, as the
   DENSE_DTFE path computes them) for callers that cannot allocate GPU
   memory, e.g. an in-situ analysis running inside a simulation whose own
   allocator has reserved the device, or code that must not call cudaMalloc
   / cudaFree because those can synchronise the device.  It has no
   counterpart in the reference.
   d_particles (3 floats per particle), d_tets (tet_t records) and d_rho
   (one float per particle) are device memory the caller owns; bounds6 is a
   host array {min x, y, z, max x, y, z} of the data bounds, as dense() uses;
   mode is tessgpu_mode; stream may be NULL.  The function allocates nothing:
   its scratch is a static device array shared by all calls, which keeps the
   last call's contents (each call clears what it uses), so calls that
   overlap on the GPU race and must be serialised by the caller.  Each call
   looks up that array's address on the current device.  More than
   TESSGPU_NOALLOC_MAX_PARTICLES particles is rejected with
   TESSGPU_ERR_INVALID.  Returns after the densities are written: the call
   synchronises the stream and reads a status word back, so it cannot be
   used while the stream is being captured into a CUDA graph. */
tessgpu_status tessgpu_dtfe_densities_noalloc(const float* d_particles, int num_particles, const int* d_tets,
                                              int num_tets, const float* bounds6, float mass, int mode,
                                              float* d_rho, void* stream);

/* ---- the DTFE surrogate's kernels ------------------------------------ */
/* A 3-D convolutional network that maps a cloud-in-cell density grid to the
   DTFE grid.  Device pointers; activations bf16 (FP32 for the f32
   outputs), chunk-planar: channel c of voxel v = (z * Y + y) * X + x at
   element ((c / 8) * V + v) * 8 + c % 8, V = X * Y * Z; weights bf16
   [27 taps][c_out][c_in], tap = (dz * 3 + dy) * 3 + dx for offsets -1..1,
   zero outside the grid.  stream may be NULL.  Nothing is synchronised. */

/* y = act(conv3x3x3(x, w) + bias): act = relu when relu != 0; bias may be
   NULL; y_bf16 and/or y_f32 receive it.  X a multiple of 16, c_in of 16,
   c_out of 8 and at most 64.  Tensor cores (bf16 in, f32 accumulation):
   tcgen05 with tensor-memory accumulators when c_in and c_out are 16 or 32,
   mma.sync otherwise.  The data gradient is the same call on the output
   gradient with the weights tessgpu_conv3d_prepare_weights flips. */
tessgpu_status tessgpu_conv3d_fwd(const void* x, int X, int Y, int Z, int c_in, int c_out, const void* w,
                                  const float* bias, int relu, void* y_bf16, float* y_f32, void* stream);
/* dw[tap][co][ci] += sum_v dy[v][co] x[v + tap][ci] and db[co] += sum_v dy[v][co]
   (FP32 sums; db may be NULL); c_in * c_out <= 4096.  tcgen05 (bf16 products,
   FP32 accumulation in tensor memory) when c_in and c_out are 16 or 32, FP32
   on the CUDA cores otherwise. */
tessgpu_status tessgpu_conv3d_wgrad(const void* x, const void* dy, int X, int Y, int Z, int c_in, int c_out,
                                    float* dw, float* db, void* stream);
/* bf16 weights for the forward pass and, flipped and transposed
   ([26 - tap][ci][co]), for the data gradient, from FP32 weights */
tessgpu_status tessgpu_conv3d_prepare_weights(const float* w, int c_out, int c_in, void* w_bf16, void* wt_bf16,
                                              void* stream);
/* engine 0 (the default): tcgen05 where the channel counts allow; 1: the
   mma.sync forward and the FP32 weight gradient for every shape.
   Process-wide. */
tessgpu_status tessgpu_conv3d_set_engine(int engine);
/* Synchronises stream; TESSGPU_ERR_TIMEOUT (and the flag cleared) when a
   tcgen05 convolution gave up on a bounded wait since the last check. */
tessgpu_status tessgpu_conv3d_check(void* stream);
/* out = g * (y > 0), bf16 (n values) */
tessgpu_status tessgpu_relu_grad(const float* g, const void* y, long long n, void* out, void* stream);
/* one Adam step (bias-corrected; step counts from 1) on FP32 weights */
tessgpu_status tessgpu_adam(float* w, const float* g, float* m, float* v, int n, float lr, float beta1, float beta2,
                            float eps, int step, void* stream);

/* ---- the surrogate's U-Net (tess2_gb300/unet.py) ----
   Same chunk-planar bf16 layout: channel c of voxel v at ((c / 8) * V + v) * 8
   + c % 8.  Grids: X a multiple of 128, or X in {16, 32, 64} with Y a multiple
   of 128 / X; V = X * Y * Z.  A call writes only the planes it names; the
   caller sizes the buffers.

   y[planes y_plane0 .. y_plane0 + c_out / 8) = 3x3x3 convolution of x (c_in
   channels, a multiple of 16) with the packed weights w, plus bias (may be
   NULL), then ReLU when relu != 0, or, when mask is given (c_out channels),
   set to 0 wherever mask <= 0 (the ReLU of a data gradient).  c_out a
   multiple of 32.  tcgen05 implicit GEMM, FP32 accumulation in tensor memory,
   bf16 output.  For the data gradient pass the packed data-gradient weights
   with c_in and c_out exchanged. */
tessgpu_status tessgpu_unet_conv(const void* x, int X, int Y, int Z, int c_in, const void* w, int c_out,
                                 const float* bias, int relu, const void* mask, void* y, int y_plane0, void* stream);
/* dw[tap][co][ci] += sum_v dy[v][co] x[v + tap][ci] (FP32 [27][c_out][c_in])
   and db[co] += sum_v dy[v][co] (db may be NULL); tcgen05, K = voxels. */
tessgpu_status tessgpu_unet_wgrad(const void* x, const void* dy, int X, int Y, int Z, int c_in, int c_out, float* dw,
                                  float* db, void* stream);
/* FP32 w[27][c_out][c_in] -> bf16 w_fwd[27][c_in/8][c_out][8] (forward) and
   w_bwd[26 - tap][c_out/8][c_in][8] (data gradient) */
tessgpu_status tessgpu_unet_pack_weights(const float* w, int c_out, int c_in, void* w_fwd, void* w_bwd, void* stream);
/* y (X/2, Y/2, Z/2) = 2x2x2 means of x (X, Y, Z), c channels */
tessgpu_status tessgpu_unet_pool(const void* x, int X, int Y, int Z, int c, void* y, void* stream);
/* dx (X, Y, Z) = (act > 0) ? skip[planes skip_plane0 ..] + dy(coarse) / 8 : 0;
   skip may be NULL (then 0) */
tessgpu_status tessgpu_unet_pool_grad(const void* dy, const void* skip, int skip_plane0, const void* act, int X, int Y,
                                      int Z, int c, void* dx, void* stream);
/* y[planes y_plane0 ..] (X, Y, Z) = x (X/2, Y/2, Z/2) at the coarse voxel */
tessgpu_status tessgpu_unet_upsample(const void* x, int X, int Y, int Z, int c, void* y, int y_plane0, void* stream);
/* dx (X/2, Y/2, Z/2) = sum of dy[planes dy_plane0 ..] over the 8 fine voxels */
tessgpu_status tessgpu_unet_upsample_grad(const void* dy, int dy_plane0, int X, int Y, int Z, int c, void* dx,
                                          void* stream);
/* x (16 channels, plane 1 already zero): channel 0 = field, channels 1-7 = 0 */
tessgpu_status tessgpu_unet_input(const float* field, long long V, void* x, void* stream);
/* Where the particles sit in the voxels of an X x Y x Z grid of points
   grid_min + i * grid_step (host arrays of 3): moments (device, 10 planes of
   X*Y*Z floats, zeroed by the call) receives per voxel, over the particles
   whose nearest grid point it is, with u = (p - point) / grid_step: the
   count, the sums of u_x, u_y, u_z and of u_x u_x, u_y u_y, u_z u_z,
   u_x u_y, u_x u_z, u_y u_z.  xyz: device, 3 floats per particle. */
tessgpu_status tessgpu_unet_cell_moments(const float* xyz, long long n, const float* grid_min, const float* grid_step,
                                         int X, int Y, int Z, float* moments, void* stream);
/* x (16 channels) from the field and those moments: 0 field, 1 log(1 + count),
   2-4 twice the mean offset, 5-10 twelve times the offsets' central second
   moments (xx, yy, zz, xy, xz, yz; zero below two particles), 11-15 zero */
tessgpu_status tessgpu_unet_input_moments(const float* field, const float* moments, long long V, void* x,
                                          void* stream);
/* pred = field + w[c] + sum_k w[k] act[k] (c <= 32 channels); with target
   and loss, *loss += sum (pred - target)^2 (FP64) */
tessgpu_status tessgpu_unet_head(const void* act, int c, const float* w, const float* field, long long V, float* pred,
                                 const float* target, double* loss, void* stream);
/* gradient of scale * sum (pred - target)^2 through the head: dact = (act >
   0) ? w * g : 0 with g = 2 scale (pred - target); dw[k] += sum g act[k],
   dw[c] += sum g */
tessgpu_status tessgpu_unet_head_grad(const void* act, int c, const float* w, const float* pred, const float* target,
                                      long long V, float scale, void* dact, float* dw, void* stream);
/* Synchronises stream; TESSGPU_ERR_TIMEOUT (and the flag cleared) when a U-Net
   tensor-core kernel gave up on a bounded wait since the last check. */
tessgpu_status tessgpu_unet_check(void* stream);

#ifdef __cplusplus
}
#endif
#endif
