// C ABI of tess2_gb300 (include/tess2_gb300.h): contexts, device batches,
// host-buffer entry points that replace the reference's calls, and the host
// side of dense() (grid parameters and block grid ranges).
//
// Host code here must evaluate GridStepParams/BlockGridParams with the
// reference's FP32 rounding, so this file is built with
// -Xcompiler -ffp-contract=off (gcc on aarch64 would otherwise fuse a*b+c).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "kernels.h"
#include "dtfe_common.cuh"

using namespace tg;

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct tessgpu_ctx
{
    int          device = 0;
    cudaStream_t stream = nullptr;
    std::string  err;
    long long    launches = 0;
    Status*      d_status = nullptr;
    Status*      h_status = nullptr;     // pinned
    float*       d_max = nullptr;
    // grow-only buffers reused by the host-buffer entry points
    std::vector<std::pair<void*, size_t>> pool;
    // rasteriser launch configuration chosen by the autotuner, per mode
    int                      raster_variant[2] = { -1, -1 };
    float                    tune_ms[2][8] = { { 0 } };
    // stage timing
    bool                     timing = false;
    std::vector<cudaEvent_t> events;
    std::vector<const char*> marks;
    int                      nmarks = 0;
    // stages that run on several streams: events recorded on the stage's own
    // stream, and (name, first event, last event) spans summed per name
    std::vector<cudaEvent_t> sevents;
    int                      nsev = 0;
    std::vector<std::pair<const char*, std::pair<int, int>>> spans;
    // WriteGrid: pinned staging buffers, and the global grid of the last tessgpu_dense call
    float*                   h_stage[2] = { nullptr, nullptr };
    cudaEvent_t              stage_ev[2] = { nullptr, nullptr };
    const float*             last_grid = nullptr;
    long long                last_grid_floats = 0;
    // the pipelined host-buffer DTFE call: copy streams and events
    cudaStream_t             h2d = nullptr, d2h = nullptr, cs2 = nullptr;
    cudaStream_t             cap = nullptr;         // stream CUDA graphs are recorded on
    std::vector<cudaEvent_t> pipe_ev;
    cudaEvent_t              first_ev[5] = { nullptr, nullptr, nullptr, nullptr, nullptr };
    // brick rasteriser: pair-list size the last call needed (0: not known yet)
    long long                pair_cap_hint = 0;
    bool                     in_retry = false;
    bool                     rows = true;           // the row kernel for dense() (raster_rows() when made)
    int                      pageable_access = -1;  // the device reads and writes pageable host memory (-1: not asked)
    int                      sets_variant[2] = { -1, -1 };   // brick shape of tessgpu_batch_dense_sets, per mode
};

// an event on stream s for a span (timing on), its index; -1 otherwise
static int smark(tessgpu_ctx* c, cudaStream_t s)
{
    if (!c->timing) return -1;
    if (c->nsev >= (int)c->sevents.size())
    {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c->sevents.push_back(e);
    }
    cudaEventRecord(c->sevents[c->nsev], s);
    return c->nsev++;
}

static void span(tessgpu_ctx* c, const char* name, int e0, int e1)
{
    if (e0 >= 0 && e1 >= 0) c->spans.push_back({ name, { e0, e1 } });
}

static void mark(tessgpu_ctx* c, const char* name)
{
    if (!c->timing) return;
    if (c->nmarks >= (int)c->events.size())
    {
        cudaEvent_t e;
        cudaEventCreate(&e);
        c->events.push_back(e);
        c->marks.push_back(nullptr);
    }
    cudaEventRecord(c->events[c->nmarks], c->stream);
    c->marks[c->nmarks] = name;
    c->nmarks++;
}

extern "C" tessgpu_status tessgpu_set_timing(tessgpu_ctx* ctx, int on)
{
    if (!ctx) return TESSGPU_ERR_INVALID;
    ctx->timing = on != 0;
    return TESSGPU_OK;
}

extern "C" int tessgpu_stage_times(tessgpu_ctx* ctx, const char** names, float* ms, int cap)
{
    if (!ctx || ctx->nmarks < 2) return 0;
    cudaEventSynchronize(ctx->events[ctx->nmarks - 1]);
    int n = 0;
    for (int i = 1; i < ctx->nmarks && n < cap; ++i, ++n)
    {
        float t = 0.0f;
        cudaEventElapsedTime(&t, ctx->events[i - 1], ctx->events[i]);
        if (names) names[n] = ctx->marks[i];
        if (ms) ms[n] = t;
    }
    // spans: per name, the sum of its launches' durations on their own streams
    std::vector<const char*> seen;
    for (size_t i = 0; i < ctx->spans.size(); ++i)
    {
        const char* nm = ctx->spans[i].first;
        if (std::find(seen.begin(), seen.end(), nm) != seen.end()) continue;
        seen.push_back(nm);
        float tot = 0.0f;
        for (size_t j = i; j < ctx->spans.size(); ++j)
            if (ctx->spans[j].first == nm)
            {
                float t = 0.0f;
                cudaEventSynchronize(ctx->sevents[ctx->spans[j].second.second]);
                cudaEventElapsedTime(&t, ctx->sevents[ctx->spans[j].second.first],
                                     ctx->sevents[ctx->spans[j].second.second]);
                tot += t;
            }
        if (n < cap)
        {
            if (names) names[n] = nm;
            if (ms) ms[n] = tot;
            ++n;
        }
    }
    return n;
}

static tessgpu_status set_err(tessgpu_ctx* c, tessgpu_status code, const std::string& msg)
{
    if (c) c->err = msg;
    return code;
}

static tessgpu_status cuda_check(tessgpu_ctx* c, cudaError_t e, const char* what)
{
    if (e == cudaSuccess)
        return TESSGPU_OK;
    return set_err(c, TESSGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                        \
    do {                                                                \
        tessgpu_status _s = cuda_check(ctx, (call), #call);            \
        if (_s != TESSGPU_OK) return _s;                                \
    } while (0)

// The DTFE rasteriser of dense() calls: the per-tet row kernel (k_raster, with
// its separate FP64 fix-up pass) unless TESSGPU_RASTER=bricks selects the
// brick kernel (k_raster_bricks).  The row kernel is the faster one on this
// GPU (its per-tet set-up runs once per tet; the brick kernel repeats it for
// every brick a tet overlaps and bins the tets first).  Independent sets
// (tessgpu_batch_dense_sets) always use the brick kernel.
static bool raster_rows()
{
    const char* e = getenv("TESSGPU_RASTER");
    return !(e && std::strcmp(e, "bricks") == 0);
}

static void* pool_get(tessgpu_ctx* c, int slot, size_t bytes, cudaError_t* e)
{
    if ((int)c->pool.size() <= slot)
        c->pool.resize(slot + 1, { nullptr, 0 });
    auto& p = c->pool[slot];
    *e = cudaSuccess;
    if (p.second < bytes)
    {
        if (c->last_grid == p.first) { c->last_grid = nullptr; c->last_grid_floats = 0; }
        if (p.first) cudaFree(p.first);
        p.first = nullptr;
        p.second = 0;
        *e = cudaMalloc(&p.first, bytes ? bytes : 16);
        if (*e != cudaSuccess)
            return nullptr;
        p.second = bytes;
    }
    return p.first;
}

extern "C" tessgpu_status tessgpu_create(int device, void* stream, tessgpu_ctx** out)
{
    if (!out) return TESSGPU_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0)
    {
        cudaGetLastError();
        return TESSGPU_ERR_NO_DEVICE;
    }
    tessgpu_ctx* ctx = new tessgpu_ctx;
    ctx->device = device;
    ctx->stream = (cudaStream_t)stream;
    ctx->rows = raster_rows();
    tessgpu_status s;
    if ((s = cuda_check(ctx, cudaSetDevice(device), "cudaSetDevice")) != TESSGPU_OK ||
        (s = cuda_check(ctx, cudaMalloc(&ctx->d_status, sizeof(Status)), "cudaMalloc")) != TESSGPU_OK ||
        (s = cuda_check(ctx, cudaMalloc(&ctx->d_max, sizeof(float)), "cudaMalloc")) != TESSGPU_OK ||
        (s = cuda_check(ctx, cudaMallocHost(&ctx->h_status, sizeof(Status)), "cudaMallocHost")) != TESSGPU_OK)
    {
        tessgpu_destroy(ctx);
        return s;
    }
    *out = ctx;
    return TESSGPU_OK;
}

extern "C" void tessgpu_destroy(tessgpu_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (auto& p : ctx->pool)
        if (p.first) cudaFree(p.first);
    for (cudaEvent_t e : ctx->events)
        cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->sevents)
        cudaEventDestroy(e);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->d_max) cudaFree(ctx->d_max);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    for (int i = 0; i < 2; ++i)
    {
        if (ctx->h_stage[i]) cudaFreeHost(ctx->h_stage[i]);
        if (ctx->stage_ev[i]) cudaEventDestroy(ctx->stage_ev[i]);
    }
    for (cudaEvent_t e : ctx->pipe_ev)
        cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->first_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->h2d) cudaStreamDestroy(ctx->h2d);
    if (ctx->d2h) cudaStreamDestroy(ctx->d2h);
    if (ctx->cs2) cudaStreamDestroy(ctx->cs2);
    if (ctx->cap) cudaStreamDestroy(ctx->cap);
    delete ctx;
}

extern "C" const char* tessgpu_last_error(const tessgpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }
extern "C" long long tessgpu_launch_count(const tessgpu_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" tessgpu_status tessgpu_sync(tessgpu_ctx* ctx)
{
    if (!ctx) return TESSGPU_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    return TESSGPU_OK;
}

// ---------------------------------------------------------------------------
// dense() grid parameters on the host, in the reference's FP32 order
// ---------------------------------------------------------------------------
// DataBounds (src/dense.cpp:1221-1275): the union of the blocks' bounds, or
// the caller's all-reduced bounds when it processes a share of the blocks
static void data_bounds(int nb, const tessgpu_block* b, const tessgpu_dense_params* p, float* mn, float* mx)
{
    if (p->use_data_bounds)
    {
        for (int d = 0; d < 3; ++d) { mn[d] = p->data_mins[d]; mx[d] = p->data_maxs[d]; }
        return;
    }
    for (int i = 0; i < nb; ++i)
        for (int d = 0; d < 3; ++d)
        {
            if (i == 0 || b[i].bounds_min[d] < mn[d]) mn[d] = b[i].bounds_min[d];
            if (i == 0 || b[i].bounds_max[d] > mx[d]) mx[d] = b[i].bounds_max[d];
        }
}

// GridStepParams (src/dense.cpp:1712-1767)
static void grid_step_params(const tessgpu_dense_params* p, const float* dmin, const float* dmax, float* gmin,
                             float* gmax, float* step)
{
    float mds = dmax[0] - dmin[0];
    if (dmax[1] - dmin[1] > mds) mds = dmax[1] - dmin[1];
    if (dmax[2] - dmin[2] > mds) mds = dmax[2] - dmin[2];
    for (int i = 0; i < 3; ++i)
    {
        gmin[i] = dmin[i] - (mds - (dmax[i] - dmin[i])) / 2.0;
        gmax[i] = dmax[i] + (mds - (dmax[i] - dmin[i])) / 2.0;
    }
    for (int i = 0; i < 3 && i < p->num_given_bounds; ++i)
    {
        gmin[i] = p->given_mins[i];
        gmax[i] = p->given_maxs[i];
    }
    for (int i = 0; i < 3; ++i)
        step[i] = (gmax[i] - gmin[i]) / (p->glo_num_idx[i] - 1);
}

static void h_idx2phys(const int* gi, float* pos, const float* step, const float* gmin)
{
    for (int i = 0; i < 3; ++i)
        pos[i] = gi[i] * step[i] + gmin[i];
}
static void h_phys2idx(const float* pos, int* gi, const float* step, const float* gmin)
{
    for (int i = 0; i < 3; ++i)
        gi[i] = (int)((pos[i] - gmin[i]) / step[i]);
}

// BlockGridParams (src/dense.cpp:575-648)
static void block_grid_params(const tessgpu_block& b, const float* gmin, const float* step, float eps,
                              const float* dmin, const float* dmax, const int* gni, int* mn, int* mx, int* num)
{
    float pos[3];
    h_phys2idx(b.bounds_min, mn, step, gmin);
    h_idx2phys(mn, pos, step, gmin);
    for (int i = 0; i < 3; ++i)
        if (pos[i] < b.bounds_min[i]) mn[i]++;
    h_phys2idx(b.bounds_max, mx, step, gmin);
    h_idx2phys(mx, pos, step, gmin);
    for (int i = 0; i < 3; ++i)
        if (pos[i] + step[i] <= b.bounds_max[i]) mx[i]++;
    for (int i = 0; i < 3; ++i)
        if (std::fabs(dmin[i] + mx[i] * step[i] - b.bounds_max[i]) < eps &&
            std::fabs(b.bounds_max[i] - dmax[i]) > step[i])
            mx[i]--;
    for (int i = 0; i < 3; ++i)
        if (std::fabs(b.bounds_min[i] - dmin[i]) < step[i]) mn[i] = 0;
    for (int i = 0; i < 3; ++i)
        if (std::fabs(b.bounds_max[i] - dmax[i]) < step[i]) mx[i] = gni[i] - 1;
    for (int i = 0; i < 3; ++i)
        num[i] = mx[i] - mn[i] + 1;
}

static bool valid_params(const tessgpu_dense_params* p)
{
    if (!p) return false;
    if (p->alg < 0 || p->alg > 2 || p->mode < 0 || p->mode > 1) return false;
    if (p->num_given_bounds < 0 || p->num_given_bounds > 3) return false;
    if (p->project != 0 && p->project != 1) return false;
    for (int i = 0; i < 3; ++i)
        if (p->glo_num_idx[i] < 2) return false;
    long long g = (long long)p->glo_num_idx[0] * p->glo_num_idx[1] * p->glo_num_idx[2];
    return g < (1LL << 40);
}

extern "C" long long tessgpu_block_grid_points(int nblocks, const tessgpu_block* blocks, int b,
                                               const tessgpu_dense_params* p, int* out9)
{
    if (nblocks <= 0 || !blocks || b < 0 || b >= nblocks || !valid_params(p)) return -1;
    float dmin[3], dmax[3], gmin[3], gmax[3], step[3];
    data_bounds(nblocks, blocks, p, dmin, dmax);
    grid_step_params(p, dmin, dmax, gmin, gmax, step);
    int mn[3], mx[3], num[3];
    block_grid_params(blocks[b], gmin, step, p->eps, dmin, dmax, p->glo_num_idx, mn, mx, num);
    if (out9)
        for (int i = 0; i < 3; ++i) { out9[i] = mn[i]; out9[3 + i] = mx[i]; out9[6 + i] = num[i]; }
    return (long long)num[0] * num[1] * (p->project ? 1 : num[2]);
}

// Layers of a projected grid: one per distinct first z index of the blocks'
// BlockGridParams boxes (clamped into the grid), ascending; zl[z] is the layer
// that holds grid index z.  In a regular decomposition a layer is one
// z-slab of blocks, and layer l at (x, y) is what the block of that slab
// covering (x, y) holds after dense(), before ProjectGrid.
static int z_layers(const std::vector<int>& block_zmin, int nz, std::vector<int>& zl)
{
    std::vector<int> starts;
    for (int z0 : block_zmin)
        starts.push_back(std::min(std::max(z0, 0), nz - 1));
    std::sort(starts.begin(), starts.end());
    starts.erase(std::unique(starts.begin(), starts.end()), starts.end());
    zl.assign(nz, 0);
    int l = 0;
    for (int z = 0; z < nz; ++z)
    {
        while (l + 1 < (int)starts.size() && starts[l + 1] <= z) ++l;
        zl[z] = l;
    }
    return starts.empty() ? 1 : (int)starts.size();
}

static int layer_of(const std::vector<int>& zl, int z0)
{
    return zl[std::min(std::max(z0, 0), (int)zl.size() - 1)];
}

extern "C" long long tessgpu_dense_grid_floats(int nblocks, const tessgpu_block* blocks,
                                               const tessgpu_dense_params* p, int* layers)
{
    if (nblocks <= 0 || !blocks || !valid_params(p)) return -1;
    const long long area = (long long)p->glo_num_idx[0] * p->glo_num_idx[1];
    if (!p->project)
    {
        if (layers) *layers = 0;
        return area * p->glo_num_idx[2];
    }
    std::vector<int> zmin(nblocks), zl;
    for (int b = 0; b < nblocks; ++b)
    {
        int out9[9] = { 0 };
        tessgpu_block_grid_points(nblocks, blocks, b, p, out9);
        zmin[b] = out9[2];
    }
    const int L = z_layers(zmin, p->glo_num_idx[2], zl);
    if (layers) *layers = L;
    return area * L;
}

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
struct tessgpu_batch
{
    tessgpu_ctx*           ctx = nullptr;
    bool                   pooled = false;   // buffers belong to the context pool
    int                    nb = 0;
    std::vector<tessgpu_block> blocks;       // host copy of the descriptors (pointers not owned)
    std::vector<BlockDesc> hb;
    std::vector<int>       hc_off;
    long long              N = 0, T = 0, C = 0;
    BlockDesc*             d_blocks = nullptr;
    int*                   d_c_off = nullptr;
    float4*                pos = nullptr;
    int4*                  tv = nullptr;
    int4*                  tn = nullptr;
    int*                   v2t = nullptr;
    float4*                cc = nullptr;
    double*                cc64 = nullptr;
    bool                   cc_ok = false, cc64_ok = false;
    // DTFE scratch
    StarSum*               W = nullptr;
    float*                 rho32 = nullptr;
    double*                rho64 = nullptr;
    int*                   fix_list = nullptr;
    int*                   fix_count = nullptr;
    // spatial processing order of the tets for the rasteriser, and the grid it was made for
    int*                   order = nullptr;
    int*                   order_key = nullptr;
    int*                   order_hist = nullptr;
    int*                   order_n = nullptr;
    bool                   order_ok = false;
    float                  order_grid[6] = { 0 };
    int                    order_dims[3] = { 0 };
    // validation outputs
    int                    raster_variant[2] = { -1, -1 };   // autotuned per mode
    bool                   keep_debug = false;
    int*                   d_cell_counts = nullptr;
    int*                   d_owner = nullptr;
    long long              owner_n = 0;
    int                    last_alg = -1;
    // independent particle sets (tessgpu_batch_dense_sets): the recorded step and what it was recorded for
    cudaGraph_t            sets_graph = nullptr;
    cudaGraphExec_t        sets_exec = nullptr;
    std::vector<long long> sets_key;
    std::vector<void*>     owned;            // device allocations to free (non-pooled)
};

enum PoolSlot
{
    SLOT_BLOCKS, SLOT_COFF, SLOT_POS, SLOT_TV, SLOT_TN, SLOT_V2T, SLOT_CC, SLOT_CC64, SLOT_W, SLOT_RHO32,
    SLOT_RHO64, SLOT_FIX, SLOT_FIXN, SLOT_STAGE, SLOT_RAWPTR, SLOT_RAWV2T, SLOT_GRID, SLOT_CELLS, SLOT_OUT,
    SLOT_OUT2, SLOT_COUNT, SLOT_ZLAYER, SLOT_GRID3, SLOT_PROJ, SLOT_LINKS, SLOT_LINKOFF, SLOT_MASK,
    SLOT_SENDS, SLOT_ORDER, SLOT_OKEY, SLOT_OHIST, SLOT_OCNT, SLOT_BRICKS, SLOT_PAIRS
};

static cudaError_t balloc(tessgpu_batch* bt, int slot, size_t bytes, void** out)
{
    cudaError_t e;
    if (bt->pooled)
    {
        *out = pool_get(bt->ctx, slot, bytes, &e);
        return e;
    }
    e = cudaMalloc(out, bytes ? bytes : 16);
    if (e == cudaSuccess)
        bt->owned.push_back(*out);
    return e;
}
#define BALLOC(slot, bytes, ptr)                                                            \
    do {                                                                                    \
        void* _p = nullptr;                                                                 \
        tessgpu_status _s = cuda_check(ctx, balloc(bt, (slot), (bytes), &_p), "cudaMalloc"); \
        if (_s != TESSGPU_OK) return _s;                                                    \
        *(void**)&(ptr) = _p;                                                               \
    } while (0)

extern "C" void tessgpu_batch_free(tessgpu_batch* bt)
{
    if (!bt) return;
    cudaSetDevice(bt->ctx->device);
    if (bt->sets_exec) cudaGraphExecDestroy(bt->sets_exec);
    if (bt->sets_graph) cudaGraphDestroy(bt->sets_graph);
    for (void* p : bt->owned)
        cudaFree(p);
    delete bt;
}

__global__ void k_pack_pos(const float* const* raw, const BlockDesc* blocks, int nb, int total, float4* pos)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < total; p += gridDim.x * blockDim.x)
    {
        int lo = 0, hi = nb - 1;
        while (lo < hi)
        {
            int mid = (lo + hi + 1) >> 1;
            if (blocks[mid].p_off <= p) lo = mid; else hi = mid - 1;
        }
        const float* r = raw[lo] + 3 * (size_t)(p - blocks[lo].p_off);
        pos[p] = make_float4(r[0], r[1], r[2], 0.0f);
    }
}

static int grid_small(long long n)
{
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

// build the device layout; device_ptrs says whether block pointers are device memory
static tessgpu_status batch_build(tessgpu_ctx* ctx, int nb, const tessgpu_block* blocks, bool device_ptrs,
                                  bool pooled, tessgpu_batch** out)
{
    if (!ctx || !out || nb <= 0 || !blocks) return set_err(ctx, TESSGPU_ERR_INVALID, "bad batch arguments");
    for (int i = 0; i < nb; ++i)
        if (blocks[i].num_particles < 0 || blocks[i].num_tets < 0 || blocks[i].num_orig_particles < 0 ||
            blocks[i].num_orig_particles > blocks[i].num_particles ||
            (blocks[i].num_particles && !blocks[i].particles) || (blocks[i].num_tets && !blocks[i].tets))
            return set_err(ctx, TESSGPU_ERR_INVALID, "block " + std::to_string(i) + " is malformed");
    CK(cudaSetDevice(ctx->device));
    tessgpu_batch* bt = new tessgpu_batch;
    *out = bt;
    bt->ctx = ctx;
    bt->pooled = pooled;
    bt->nb = nb;
    bt->blocks.assign(blocks, blocks + nb);
    bt->hb.resize(nb);
    bt->hc_off.resize(nb);
    long long N = 0, T = 0, C = 0;
    for (int i = 0; i < nb; ++i)
    {
        BlockDesc& d = bt->hb[i];
        std::memset(&d, 0, sizeof(d));
        d.gid = blocks[i].gid;
        for (int k = 0; k < 3; ++k) { d.bmin[k] = blocks[i].bounds_min[k]; d.bmax[k] = blocks[i].bounds_max[k]; }
        d.p_off = (int)N; d.np = blocks[i].num_particles; d.norig = blocks[i].num_orig_particles;
        d.t_off = (int)T; d.nt = blocks[i].num_tets;
        d.c_off = (int)C;
        bt->hc_off[i] = (int)C;
        N += blocks[i].num_particles;
        T += blocks[i].num_tets;
        C += blocks[i].num_orig_particles;
    }
    if (N >= (1LL << 31) || T >= (1LL << 31))
        return set_err(ctx, TESSGPU_ERR_INVALID, "batch larger than 2^31 particles or tets");
    bt->N = N; bt->T = T; bt->C = C;
    BALLOC(SLOT_BLOCKS, sizeof(BlockDesc) * nb, bt->d_blocks);
    BALLOC(SLOT_COFF, sizeof(int) * nb, bt->d_c_off);
    BALLOC(SLOT_POS, sizeof(float4) * N, bt->pos);
    BALLOC(SLOT_TV, sizeof(int4) * T, bt->tv);
    BALLOC(SLOT_TN, sizeof(int4) * T, bt->tn);
    BALLOC(SLOT_V2T, sizeof(int) * N, bt->v2t);
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(bt->d_blocks, bt->hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(bt->d_c_off, bt->hc_off.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, s));

    // raw pointer tables (device pointers to each block's particles / tet_t / vert_to_tet)
    std::vector<const void*> raw_pos(nb), raw_tets(nb), raw_v2t(nb);
    bool have_v2t = true;
    for (int i = 0; i < nb; ++i)
        if (blocks[i].num_particles && !blocks[i].vert_to_tet) have_v2t = false;
    float* stage_pos = nullptr;
    int* stage_tets = nullptr;
    int* stage_v2t = nullptr;
    if (!device_ptrs)
    {
        // one staging buffer: xyz, then tet_t, then vert_to_tet
        size_t bytes = sizeof(float) * 3 * N + sizeof(int) * 8 * T + (have_v2t ? sizeof(int) * N : 0);
        char* stage;
        BALLOC(SLOT_STAGE, bytes, stage);
        stage_pos = (float*)stage;
        stage_tets = (int*)(stage + sizeof(float) * 3 * N);
        stage_v2t = (int*)(stage + sizeof(float) * 3 * N + sizeof(int) * 8 * T);
        for (int i = 0; i < nb; ++i)
        {
            const BlockDesc& d = bt->hb[i];
            if (d.np)
                CK(cudaMemcpyAsync(stage_pos + 3 * (size_t)d.p_off, blocks[i].particles, sizeof(float) * 3 * d.np,
                                   cudaMemcpyHostToDevice, s));
            if (d.nt)
                CK(cudaMemcpyAsync(stage_tets + 8 * (size_t)d.t_off, blocks[i].tets, sizeof(int) * 8 * d.nt,
                                   cudaMemcpyHostToDevice, s));
            if (have_v2t && d.np)
                CK(cudaMemcpyAsync(stage_v2t + d.p_off, blocks[i].vert_to_tet, sizeof(int) * d.np,
                                   cudaMemcpyHostToDevice, s));
            raw_pos[i] = stage_pos + 3 * (size_t)d.p_off;
            raw_tets[i] = stage_tets + 8 * (size_t)d.t_off;
            raw_v2t[i] = stage_v2t + d.p_off;
        }
    }
    else
    {
        for (int i = 0; i < nb; ++i)
        {
            raw_pos[i] = blocks[i].particles;
            raw_tets[i] = blocks[i].tets;
            raw_v2t[i] = blocks[i].vert_to_tet;
        }
    }
    const void** d_raw;
    BALLOC(SLOT_RAWPTR, sizeof(void*) * 3 * nb, d_raw);
    std::vector<const void*> tbl(3 * nb);
    for (int i = 0; i < nb; ++i) { tbl[i] = raw_pos[i]; tbl[nb + i] = raw_tets[i]; tbl[2 * nb + i] = raw_v2t[i]; }
    CK(cudaMemcpyAsync(d_raw, tbl.data(), sizeof(void*) * 3 * nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), s));
    if (N)
    {
        k_pack_pos<<<grid_small(N), 256, 0, s>>>((const float* const*)d_raw, bt->d_blocks, nb, (int)N, bt->pos);
        ctx->launches++;
    }
    launch_ingest((const int* const*)(d_raw + nb), bt->d_blocks, nb, (int)T, bt->tv, bt->tn, ctx->d_status, s);
    ctx->launches += T ? 1 : 0;
    if (have_v2t)
    {
        launch_v2t_from_local((const int* const*)(d_raw + 2 * nb), bt->d_blocks, nb, (int)N, bt->v2t,
                              ctx->d_status, s);
        ctx->launches += N ? 1 : 0;
    }
    else
    {
        CK(cudaMemsetAsync(bt->v2t, 0xff, sizeof(int) * N, s));
        launch_vert_to_tet(bt->tv, (int)T, bt->v2t, s);
        ctx->launches += T ? 1 : 0;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (ctx->h_status->code)
        return set_err(ctx, (tessgpu_status)ctx->h_status->code,
                       "malformed mesh at item " + std::to_string(ctx->h_status->detail));
    return TESSGPU_OK;
}

extern "C" tessgpu_status tessgpu_batch_upload(tessgpu_ctx* ctx, int nb, const tessgpu_block* blocks,
                                               tessgpu_batch** out)
{
    tessgpu_status s = batch_build(ctx, nb, blocks, false, false, out);
    if (s != TESSGPU_OK && out && *out) { tessgpu_batch_free(*out); *out = nullptr; }
    return s;
}

extern "C" tessgpu_status tessgpu_batch_wrap_device(tessgpu_ctx* ctx, int nb, const tessgpu_block* blocks,
                                                    tessgpu_batch** out)
{
    tessgpu_status s = batch_build(ctx, nb, blocks, true, false, out);
    if (s != TESSGPU_OK && out && *out) { tessgpu_batch_free(*out); *out = nullptr; }
    return s;
}

extern "C" tessgpu_status tessgpu_batch_keep_debug(tessgpu_batch* bt, int on)
{
    if (!bt) return TESSGPU_ERR_INVALID;
    bt->keep_debug = on != 0;
    return TESSGPU_OK;
}

// ---------------------------------------------------------------------------
// dense on a batch
// ---------------------------------------------------------------------------
static tessgpu_status finish_status(tessgpu_ctx* ctx)
{
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const Status& st = *ctx->h_status;
    if (st.code)
    {
        static const char* names[] = { "ok", "invalid", "cuda", "no device", "vertex star larger than TESSGPU_MAX_STAR",
                                       "Voronoi cell with more than TESSGPU_MAX_FACES faces",
                                       "edge ring longer than TESSGPU_MAX_LINK", "malformed mesh", "unsupported",
                                       "i/o", "bounded wait ran out", "device work list larger than its buffer" };
        const char* nm = (st.code > 0 && st.code < 12) ? names[st.code] : "error";
        return set_err(ctx, (tessgpu_status)st.code, std::string(nm) + " at item " + std::to_string(st.detail));
    }
    return TESSGPU_OK;
}

static const float kTau = DTFE_TAU;   // mixed DTFE: FP64 for tets whose FP32 bound exceeds tau*|6V|

// ---------------------------------------------------------------------------
// DTFE rasteriser selection and the brick rasteriser's host side
// ---------------------------------------------------------------------------
// true when the blocks' grid boxes are disjoint and cover the whole grid, so
// that writing every box writes every grid point
static bool boxes_tile(const std::vector<BlockDesc>& hb, const int* gni)
{
    long long covered = 0;
    const int nb = (int)hb.size();
    for (int i = 0; i < nb; ++i)
    {
        long long v = 1;
        for (int k = 0; k < 3; ++k)
        {
            const int n = hb[i].gmax_idx[k] - hb[i].gmin_idx[k] + 1;
            if (n <= 0) return false;
            v *= n;
        }
        covered += v;
        for (int j = 0; j < i; ++j)
        {
            bool meet = true;
            for (int k = 0; k < 3; ++k)
                if (hb[i].gmax_idx[k] < hb[j].gmin_idx[k] || hb[j].gmax_idx[k] < hb[i].gmin_idx[k]) meet = false;
            if (meet) return false;
        }
    }
    return covered == (long long)gni[0] * gni[1] * gni[2];
}

// every block rasterises into the call's one grid (offset 0)
static void set_block_grids(std::vector<BlockDesc>& hb, const GridDesc& g)
{
    for (BlockDesc& d : hb)
    {
        for (int k = 0; k < 3; ++k)
        {
            d.grid.gmin[k] = g.gmin[k];
            d.grid.step[k] = g.step[k];
            d.grid.inv_step[k] = g.inv_step[k];
            d.grid.n[k] = g.n[k];
        }
        d.grid.off = 0;
    }
}

// cut every block's grid box into bricks of the variant's shape (aligned to
// the global grid); returns the number of bricks of all blocks
static long long assign_bricks(std::vector<BlockDesc>& hb, int variant)
{
    int sh[3];
    brick_shape(variant, &sh[0], &sh[1], &sh[2]);
    long long base = 0;
    for (BlockDesc& d : hb)
    {
        d.brick_base = (int)base;
        long long n = 1;
        for (int k = 0; k < 3; ++k)
        {
            if (d.gmin_idx[k] > d.gmax_idx[k])
            {
                d.brick_lo[k] = 0;
                d.brick_n[k] = 0;
            }
            else
            {
                d.brick_lo[k] = d.gmin_idx[k] >> sh[k];
                d.brick_n[k] = (d.gmax_idx[k] >> sh[k]) - d.brick_lo[k] + 1;
            }
            n *= d.brick_n[k];
        }
        base += n;
    }
    return base;
}

// the brick rasteriser's scratch (context pool): per-brick counts, offsets,
// cursors and item offsets, per-segment items and counters, the pair cursor,
// and the pair list (2 pairs per tet to start with; grown to what a call
// needed when it overflowed)
static tessgpu_status brick_bins(tessgpu_ctx* ctx, long long nbricks, int nb, long long T, BrickBins* b)
{
    cudaError_t e;
    const size_t nbr = (size_t)std::max(nbricks, 1LL);
    char* raw = (char*)pool_get(ctx, SLOT_BRICKS, 16 + sizeof(int) * (4 * nbr + 2 * (size_t)nb), &e);
    CK(e);
    b->pair_cursor = (unsigned long long*)raw;
    int* base = (int*)(raw + 16);
    b->cnt = base;
    b->off = base + nbr;
    b->cur = base + 2 * nbr;
    b->item_off = base + 3 * nbr;
    b->seg_items = base + 4 * nbr;
    b->counters = b->seg_items + nb;
    long long cap = std::max(ctx->pair_cap_hint, 2 * T + 65536);
    // TESSGPU_PAIR_CAP: a first size for tests of the overflow retry
    const char* env = getenv("TESSGPU_PAIR_CAP");
    if (env && *env && ctx->pair_cap_hint == 0)
        cap = std::max(atoll(env), 1LL);
    cap = std::min(cap, (long long)INT32_MAX);
    b->pairs = (int*)pool_get(ctx, SLOT_PAIRS, sizeof(int) * (size_t)cap, &e);
    CK(e);
    b->pair_cap = cap;
    return TESSGPU_OK;
}

// segment [k0, k1) of blocks: bin its tets into its bricks, then rasterise
static void bricks_bin(tessgpu_ctx* ctx, int variant, const BlockDesc* d_blocks, const std::vector<BlockDesc>& hb,
                       int k0, int k1, long long nbricks, const BrickBins& bins, const float4* pos, const int4* tv,
                       const GridDesc& g, float* grid, cudaStream_t s)
{
    const int nb = (int)hb.size();
    const int bb0 = hb[k0].brick_base, bb1 = k1 < nb ? hb[k1].brick_base : (int)nbricks;
    const int t0 = hb[k0].t_off, t1 = hb[k1 - 1].t_off + hb[k1 - 1].nt;
    launch_bin_bricks(variant, d_blocks, nb, k0, bb0, bb1, t0, t1 - t0, pos, tv, g, bins, grid, ctx->d_status, s);
    ctx->launches += t1 > t0 ? 4 : 1;
}

// the same in three steps, the count fused into the star volumes:
// bricks_reset, bricks_star (star volumes of tets [t0, t0 + nt) and their
// pair counts; may run in parts), bricks_place (scan, scatter, zeroing)
static void bricks_reset(tessgpu_ctx* ctx, const std::vector<BlockDesc>& hb, int k0, int k1, long long nbricks,
                         const BrickBins& bins, cudaStream_t s)
{
    const int nb = (int)hb.size();
    const int bb0 = hb[k0].brick_base, bb1 = k1 < nb ? hb[k1].brick_base : (int)nbricks;
    launch_bin_reset(bins, k0, bb0, bb1, s);
    (void)ctx;
}

static void bricks_star(tessgpu_ctx* ctx, int mode, int variant, const BlockDesc* d_blocks, int nb, long long t0,
                        long long nt, const float4* pos, const int4* tv, StarSum* W, double scale,
                        const GridDesc& g, const BrickBins& bins, cudaStream_t s)
{
    if (nt <= 0) return;
    launch_star_bin(mode, variant, d_blocks, nb, (int)t0, (int)nt, pos, tv, W, scale, g, bins.cnt, ctx->d_status, s);
    ctx->launches++;
}

static void bricks_place(tessgpu_ctx* ctx, int variant, const BlockDesc* d_blocks, const std::vector<BlockDesc>& hb,
                         int k0, int k1, long long nbricks, const BrickBins& bins, const float4* pos, const int4* tv,
                         const GridDesc& g, float* grid, cudaStream_t s)
{
    const int nb = (int)hb.size();
    const int bb0 = hb[k0].brick_base, bb1 = k1 < nb ? hb[k1].brick_base : (int)nbricks;
    const int t0 = hb[k0].t_off, t1 = hb[k1 - 1].t_off + hb[k1 - 1].nt;
    launch_bin_place(variant, d_blocks, nb, k0, bb0, bb1, t0, t1 - t0, pos, tv, g, bins, grid, ctx->d_status, s);
    ctx->launches += t1 > t0 && bb1 > bb0 ? 3 : 1;
}

static void bricks_raster(tessgpu_ctx* ctx, int mode, int variant, const BlockDesc* d_blocks,
                          const std::vector<BlockDesc>& hb, int k0, int k1, long long nbricks, const BrickBins& bins,
                          const float4* pos, const int4* tv, const float* rho32, const double* rho64,
                          const GridDesc& g, float* grid, int* owner, cudaStream_t s)
{
    const int nb = (int)hb.size();
    const int bb0 = hb[k0].brick_base, bb1 = k1 < nb ? hb[k1].brick_base : (int)nbricks;
    if (bb1 <= bb0) return;
    launch_raster_bricks(mode, variant, d_blocks, nb, k0, bb0, bb1, bins, pos, tv, rho32, rho64, g, grid, owner,
                         ctx->d_status, s);
    ctx->launches++;
}

// after a call failed with TESSGPU_ERR_CAPACITY: size the pair list for what
// it needed (the cursor holds the pairs every segment asked for)
static void grow_pairs(tessgpu_ctx* ctx)
{
    if ((int)ctx->pool.size() <= SLOT_BRICKS || !ctx->pool[SLOT_BRICKS].first) return;
    unsigned long long need = 0;
    if (cudaMemcpy(&need, ctx->pool[SLOT_BRICKS].first, sizeof(need), cudaMemcpyDeviceToHost) == cudaSuccess)
        ctx->pair_cap_hint = std::max(ctx->pair_cap_hint, (long long)(need + need / 4 + 65536));
    cudaGetLastError();
}

static tessgpu_status dtfe_batch_bricks(tessgpu_ctx* ctx, tessgpu_batch* bt, const tessgpu_dense_params* p,
                                        const GridDesc& g, const float* gmax, float* target, float* d_grid,
                                        const int* d_zl, int L, long long Gout, int var, long long nbricks,
                                        tessgpu_dense_info* info);

extern "C" tessgpu_status tessgpu_batch_dense(tessgpu_ctx* ctx, tessgpu_batch* bt, const tessgpu_dense_params* p,
                                              float* d_grid, tessgpu_dense_info* info)
{
    if (!ctx || !bt || !d_grid || !valid_params(p))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad dense arguments");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int nb = bt->nb;
    float dmin[3], dmax[3], gmin[3], gmax[3], step[3];
    data_bounds(nb, bt->blocks.data(), p, dmin, dmax);
    grid_step_params(p, dmin, dmax, gmin, gmax, step);
    GridDesc g;
    for (int i = 0; i < 3; ++i)
    {
        g.gmin[i] = gmin[i]; g.step[i] = step[i]; g.dmin[i] = dmin[i]; g.dmax[i] = dmax[i];
        g.n[i] = p->glo_num_idx[i];
    }
    g.eps = p->eps;
    g.mass = p->mass;
    // src/dense.cpp:241-242: volume, or area when projecting
    g.div = p->project ? step[0] * step[1] : step[0] * step[1] * step[2];
    for (int i = 0; i < 3; ++i)
        g.inv_step[i] = 1.0f / step[i];
    g.zlayer = nullptr;
    for (int i = 0; i < nb; ++i)
    {
        BlockDesc& d = bt->hb[i];
        block_grid_params(bt->blocks[i], gmin, step, p->eps, dmin, dmax, p->glo_num_idx, d.gmin_idx, d.gmax_idx,
                          d.gnum_idx);
        // kernels write only inside the grid, whatever the block bounds
        for (int k = 0; k < 3; ++k)
        {
            d.gmin_idx[k] = std::max(d.gmin_idx[k], 0);
            d.gmax_idx[k] = std::min(d.gmax_idx[k], p->glo_num_idx[k] - 1);
        }
    }
    set_block_grids(bt->hb, g);
    // DTFE with the brick rasteriser: the bricks of the chosen (or first) variant
    const bool bricks = p->alg == TESSGPU_DENSE_DTFE && !ctx->rows;
    int bvar = -1;
    long long nbricks = 0;
    if (bricks)
    {
        bvar = bt->raster_variant[p->mode] >= 0 ? bt->raster_variant[p->mode] : ctx->raster_variant[p->mode];
        const char* env = getenv("TESSGPU_RASTER_VARIANT");
        if (bvar < 0 && env && *env)
            bvar = ctx->raster_variant[p->mode] = std::min(std::max(atoi(env), 0), brick_variants() - 1);
        nbricks = assign_bricks(bt->hb, bvar < 0 ? 0 : bvar);
    }
    CK(cudaMemcpyAsync(bt->d_blocks, bt->hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), s));
    const long long area = (long long)p->glo_num_idx[0] * p->glo_num_idx[1];
    const long long G = area * p->glo_num_idx[2];
    // projected: d_grid holds L layers of the x-y plane; DENSE_TESS / DENSE_CIC
    // deposit into them directly, DTFE rasterises a 3-D scratch grid first
    int L = 0;
    int* d_zl = nullptr;
    float* target = d_grid;
    if (p->project)
    {
        std::vector<int> zmin(nb), zl;
        for (int i = 0; i < nb; ++i)
            zmin[i] = bt->hb[i].gmin_idx[2];
        L = z_layers(zmin, p->glo_num_idx[2], zl);
        // zl (layer of each z), then the layers' z bounds zs[0..L]
        std::vector<int> tbl(zl);
        for (int l = 0, z = 0; l <= L; ++l)
        {
            while (z < (int)zl.size() && zl[z] < l) ++z;
            tbl.push_back(z);
        }
        cudaError_t e;
        d_zl = (int*)pool_get(ctx, SLOT_ZLAYER, sizeof(int) * tbl.size(), &e);
        CK(e);
        CK(cudaMemcpyAsync(d_zl, tbl.data(), sizeof(int) * tbl.size(), cudaMemcpyHostToDevice, s));
        if (p->alg == TESSGPU_DENSE_DTFE)
        {
            target = (float*)pool_get(ctx, SLOT_GRID3, sizeof(float) * G, &e);
            CK(e);
        }
        else
            g.zlayer = d_zl;
    }
    const long long Gout = p->project ? area * L : G;
    const long long Gtarget = target == d_grid ? Gout : G;
    ctx->nmarks = 0;
    ctx->nsev = 0;
    ctx->spans.clear();
    mark(ctx, "start");
    // the brick rasteriser writes every point of the blocks' boxes (zeros
    // included); the grid needs zeroing only where the boxes leave gaps
    if (!bricks || !boxes_tile(bt->hb, p->glo_num_idx))
    {
        CK(cudaMemsetAsync(target, 0, sizeof(float) * Gtarget, s));
        mark(ctx, "grid_zero");
    }
    bt->last_alg = p->alg;

    if (p->alg == TESSGPU_DENSE_TESS)
    {
        if (!bt->cc_ok)
        {
            if (!bt->cc || bt->pooled)
                BALLOC(SLOT_CC, sizeof(float4) * bt->T, bt->cc);
            launch_circumcenters(bt->pos, bt->tv, (int)bt->T, bt->cc, s);
            ctx->launches += bt->T ? 1 : 0;
            bt->cc_ok = !bt->pooled;
            mark(ctx, "circumcenters");
        }
        int* counts = nullptr;
        if (bt->keep_debug)
        {
            if (!bt->d_cell_counts || bt->pooled)
                BALLOC(SLOT_CELLS, sizeof(int) * (bt->C ? bt->C : 1), bt->d_cell_counts);
            counts = bt->d_cell_counts;
        }
        launch_cells(CELL_DENSE_TESS, bt->d_blocks, bt->d_c_off, nb, (int)bt->C, bt->pos, bt->tv, bt->tn, bt->v2t,
                     bt->cc, nullptr, g, target, nullptr, nullptr, nullptr, nullptr, counts, ctx->d_status, s);
        ctx->launches += bt->C ? 1 : 0;
        mark(ctx, "cells_dense_tess");
    }
    else if (p->alg == TESSGPU_DENSE_CIC)
    {
        launch_cic(bt->d_blocks, bt->d_c_off, nb, (int)bt->C, bt->pos, g, target, ctx->d_status, s);
        ctx->launches += bt->C ? 1 : 0;
        mark(ctx, "cic");
    }
    else
    {
        if (bricks)
            return dtfe_batch_bricks(ctx, bt, p, g, gmax, target, d_grid, d_zl, L, Gout, bvar, nbricks, info);
        if (!bt->W || bt->pooled)
        {
            BALLOC(SLOT_W, sizeof(StarSum) * (bt->N ? bt->N : 1), bt->W);
            BALLOC(SLOT_RHO32, sizeof(float) * (bt->N ? bt->N : 1), bt->rho32);
            BALLOC(SLOT_RHO64, sizeof(double) * (bt->N ? bt->N : 1), bt->rho64);
            BALLOC(SLOT_FIX, sizeof(int) * (bt->T ? bt->T : 1), bt->fix_list);
            BALLOC(SLOT_FIXN, sizeof(int) * 2 * (nb + 1), bt->fix_count);
        }
        int* owner = nullptr;
        if (bt->keep_debug)
        {
            if (!bt->d_owner || bt->owner_n < G || bt->pooled)
                BALLOC(SLOT_OUT, sizeof(int) * G, bt->d_owner);
            CK(cudaMemsetAsync(bt->d_owner, 0xff, sizeof(int) * G, s));
            bt->owner_n = G;
            owner = bt->d_owner;
        }
        CK(cudaMemsetAsync(bt->W, 0, sizeof(StarSum) * bt->N, s));
        // fix_count: the FP64 fix-up list length per block, then the
        // rasteriser's chunk counter per block (persistent launches)
        int* next = bt->fix_count + (nb + 1);
        CK(cudaMemsetAsync(bt->fix_count, 0, sizeof(int) * 2 * (nb + 1), s));
        // fixed-point scale of the star-volume sums: any star volume is below
        // the volume of the particles' bounding box; allow 8x the data box
        const double scale = star_sum_scale(dmin, dmax, p->mode == TESSGPU_MODE_FP64);
        // TESSGPU_BATCH_OVERLAP=1: once the launch variant is known, blocks run
        // their stages on two streams in turn, so one block's star volumes
        // overlap another's rasteriser.  Off by default: the rasteriser's
        // persistent launches fill every SM, and two of them side by side
        // (4.49 ms a step at 2M -> 512^3) lose to each stage over all blocks
        // in one launch (4.37 ms).
        {
            const char* ov = getenv("TESSGPU_BATCH_OVERLAP");
            const char* oenv = getenv("TESSGPU_RASTER_ORDER");
            int known = bt->raster_variant[p->mode] >= 0 ? bt->raster_variant[p->mode] : ctx->raster_variant[p->mode];
            if ((ov && *ov && atoi(ov) == 1) && known >= 0 && !(oenv && atoi(oenv) == 1) && !p->project)
            {
                bt->raster_variant[p->mode] = known;
                if (!ctx->cs2) CK(cudaStreamCreateWithFlags(&ctx->cs2, cudaStreamNonBlocking));
                while ((int)ctx->pipe_ev.size() < 2 * nb + 2)
                {
                    cudaEvent_t e;
                    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
                    ctx->pipe_ev.push_back(e);
                }
                CK(cudaEventRecord(ctx->pipe_ev[2 * nb + 1], s));
                CK(cudaStreamWaitEvent(ctx->cs2, ctx->pipe_ev[2 * nb + 1], 0));
                for (int k = 0; k < nb; ++k)
                {
                    const BlockDesc& d = bt->hb[k];
                    cudaStream_t sk = (k & 1) ? ctx->cs2 : s;
                    const int t0 = smark(ctx, sk);
                    if (d.nt)
                        launch_star_volumes(p->mode, d.nt, bt->pos, bt->tv + d.t_off, (StarSum*)bt->W, scale,
                                            kTau, ctx->d_status, sk);
                    const int t1 = smark(ctx, sk);
                    if (d.np)
                        launch_densities((const StarSum*)bt->W + d.p_off, d.np, p->mass, 1.0 / scale,
                                         bt->rho32 + d.p_off, bt->rho64 + d.p_off, ctx->d_status, sk);
                    const int t2 = smark(ctx, sk);
                    int t3 = -1, t4 = -1;
                    if (d.nt)
                    {
                        launch_raster(p->mode, known, bt->d_blocks, nb, d.nt, bt->pos, bt->tv, bt->rho32, bt->rho64,
                                      g, kTau, target, owner, bt->fix_list + d.t_off, bt->fix_count + k,
                                      ctx->d_status, sk, nullptr, nullptr, d.t_off, false, next + k);
                        t3 = smark(ctx, sk);
                        if (p->mode != TESSGPU_MODE_FP64)
                        {
                            launch_raster_fix(bt->d_blocks, nb, d.nt, bt->pos, bt->tv, bt->rho32, bt->rho64, g, target,
                                              owner, bt->fix_list + d.t_off, bt->fix_count + k, ctx->d_status, sk);
                            t4 = smark(ctx, sk);
                        }
                    }
                    span(ctx, "star_volumes", t0, t1);
                    span(ctx, "densities", t1, t2);
                    span(ctx, "raster", t2, t3);
                    span(ctx, "raster_fp64_fixup", t3, t4);
                    ctx->launches += (d.nt ? (p->mode == TESSGPU_MODE_FP64 ? 2 : 3) : 0) + (d.np ? 1 : 0);
                    CK(cudaEventRecord(ctx->pipe_ev[nb + k], sk));
                }
                for (int k = nb - 1; k >= 0; --k)
                    if (k & 1)
                    {
                        CK(cudaStreamWaitEvent(s, ctx->pipe_ev[nb + k], 0));
                        break;
                    }
                mark(ctx, "dtfe_blocks");
                goto dtfe_done;
            }
        }
        launch_star_volumes(p->mode, (int)bt->T, bt->pos, bt->tv, (StarSum*)bt->W, scale, kTau,
                            ctx->d_status, s);
        mark(ctx, "star_volumes");
        launch_densities((const StarSum*)bt->W, (int)bt->N, p->mass, 1.0 / scale, bt->rho32, bt->rho64,
                         ctx->d_status, s);
        mark(ctx, "densities");
        // TESSGPU_RASTER_ORDER=1 rasterises the tets brick by brick (kept with a
        // device-resident batch while the grid stays the same).  It cuts the
        // rasteriser's HBM traffic by a third but not its time, which is set by
        // instruction issue, so the tets' own order is the default.
        const int* order = nullptr;
        const int* order_n = nullptr;
        const char* oenv = getenv("TESSGPU_RASTER_ORDER");
        if (bt->T && oenv && atoi(oenv) == 1)
        {
            const float okey[6] = { g.gmin[0], g.gmin[1], g.gmin[2], g.step[0], g.step[1], g.step[2] };
            const bool same = bt->order_ok && !std::memcmp(okey, bt->order_grid, sizeof(okey)) &&
                              !std::memcmp(g.n, bt->order_dims, sizeof(bt->order_dims));
            if (!same)
            {
                int nbx, nby, nbz;
                order_bricks(g, &nbx, &nby, &nbz);
                if (!bt->order || bt->pooled)
                {
                    BALLOC(SLOT_ORDER, sizeof(int) * bt->T, bt->order);
                    BALLOC(SLOT_OKEY, sizeof(int) * bt->T, bt->order_key);
                    BALLOC(SLOT_OCNT, sizeof(int), bt->order_n);
                }
                BALLOC(SLOT_OHIST, sizeof(int) * (size_t)nbx * nby * nbz, bt->order_hist);
                const int tn = (int)bt->T;
                CK(cudaMemcpyAsync(bt->order_n, &tn, sizeof(int), cudaMemcpyHostToDevice, s));
                CK(cudaStreamSynchronize(s));   // tn lives on this stack frame
                launch_tet_order(bt->pos, bt->tv, tn, g, bt->order_key, bt->order_hist, bt->order, s);
                ctx->launches += 3;
                bt->order_ok = !bt->pooled;
                std::memcpy(bt->order_grid, okey, sizeof(okey));
                std::memcpy(bt->order_dims, g.n, sizeof(bt->order_dims));
                mark(ctx, "tet_order");
            }
            order = bt->order;
            order_n = bt->order_n;
        }
        int& var = bt->raster_variant[p->mode];
        if (var < 0)
            var = ctx->raster_variant[p->mode];   // a choice made on an earlier batch of this context
        if (var < 0)
        {
            // TESSGPU_RASTER_VARIANT fixes the choice (tuning runs); otherwise
            // autotune: time each launch-bound variant twice on this batch (the
            // first launch of a kernel also pays its module load) and keep the
            // fastest; the grid is rewritten by every run, the fix list is reset
            const char* env = getenv("TESSGPU_RASTER_VARIANT");
            if (env && *env)
            {
                var = std::min(std::max(atoi(env), 0), raster_variants() - 1);
                ctx->raster_variant[p->mode] = var;
            }
        }
        if (var < 0)
        {
            // the tuning launches count into the status; keep what the stages
            // before the rasteriser counted (star volumes' FP64 tets, errors)
            // and put it back afterwards
            Status saved;
            CK(cudaMemcpyAsync(&saved, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            float best = 1e30f;
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            for (int v = 0; v < raster_variants(); ++v)
            {
                float vbest = 1e30f;
                for (int rep = 0; rep < 2; ++rep)
                {
                    CK(cudaMemsetAsync(bt->fix_count, 0, sizeof(int), s));
                    CK(cudaMemsetAsync(next, 0, sizeof(int), s));
                    cudaEventRecord(e0, s);
                    launch_raster(p->mode, v, bt->d_blocks, nb, (int)bt->T, bt->pos, bt->tv, bt->rho32, bt->rho64, g,
                                  kTau, target, owner, bt->fix_list, bt->fix_count, ctx->d_status, s, order, order_n,
                                  0, false, next);
                    cudaEventRecord(e1, s);
                    ctx->launches++;
                    CK(cudaEventSynchronize(e1));
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    vbest = std::min(vbest, ms);
                }
                if (v < 8) ctx->tune_ms[p->mode][v] = vbest;
                if (vbest < best) { best = vbest; var = v; }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            ctx->raster_variant[p->mode] = var;
            CK(cudaMemsetAsync(bt->fix_count, 0, sizeof(int), s));
            CK(cudaMemsetAsync(next, 0, sizeof(int), s));
            CK(cudaMemcpyAsync(ctx->d_status, &saved, sizeof(Status), cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
            CK(cudaMemsetAsync(target, 0, sizeof(float) * G, s));
            if (owner) CK(cudaMemsetAsync(owner, 0xff, sizeof(int) * G, s));
        }
        launch_raster(p->mode, var, bt->d_blocks, nb, (int)bt->T, bt->pos, bt->tv, bt->rho32, bt->rho64, g, kTau,
                      target, owner, bt->fix_list, bt->fix_count, ctx->d_status, s, order, order_n, 0, false, next);
        mark(ctx, "raster");
        if (p->mode != TESSGPU_MODE_FP64)
        {
            launch_raster_fix(bt->d_blocks, nb, (int)bt->T, bt->pos, bt->tv, bt->rho32, bt->rho64, g, target, owner,
                              bt->fix_list, bt->fix_count, ctx->d_status, s);
            mark(ctx, "raster_fp64_fixup");
        }
        ctx->launches += (bt->T ? (p->mode == TESSGPU_MODE_FP64 ? 2 : 3) : 0) + (bt->N ? 1 : 0);
        if (p->project)
        {
            // surface density: the column integral of rho over each layer's z range
            launch_project_layers(target, p->glo_num_idx[0], p->glo_num_idx[1], d_zl + p->glo_num_idx[2], L, step[2],
                                  d_grid, s);
            ctx->launches++;
            mark(ctx, "project_layers");
        }
    }
dtfe_done:
    double max_dense = 0.0;
    if (info || p->alg != TESSGPU_DENSE_DTFE)
    {
        CK(cudaMemsetAsync(ctx->d_max, 0, sizeof(float), s));
        launch_grid_max(d_grid, Gout, ctx->d_max, s);
        ctx->launches++;
        mark(ctx, "grid_max");
    }
    tessgpu_status st = finish_status(ctx);
    if (info)
    {
        float mx = 0.0f;
        CK(cudaMemcpy(&mx, ctx->d_max, sizeof(float), cudaMemcpyDeviceToHost));
        max_dense = mx;
        std::memset(info, 0, sizeof(*info));
        for (int i = 0; i < 3; ++i)
        {
            info->data_mins[i] = dmin[i]; info->data_maxs[i] = dmax[i];
            info->grid_phys_mins[i] = gmin[i]; info->grid_phys_maxs[i] = gmax[i]; info->grid_step_size[i] = step[i];
        }
        info->max_dense = max_dense;
        info->tot_mass = ctx->h_status->tot_mass;
        info->check_mass = (double)ctx->h_status->check_mass;
        info->grid_pts_assigned = (long long)ctx->h_status->assigned;
        info->fp64_tets = (long long)ctx->h_status->fp64_tets;
        info->exact_tests = (long long)ctx->h_status->exact_tests;
        info->rows_visited = (long long)ctx->h_status->rows;
        info->points_tested = (long long)ctx->h_status->candidates;
        info->raster_variant = bt->raster_variant[p->mode];
        for (int v = 0; v < 8; ++v)
            info->raster_variant_ms[v] = ctx->tune_ms[p->mode][v];
        info->grid_layers = L;
        info->grid_floats = Gout;
        info->cell_probes = (long long)ctx->h_status->probes;
        info->face_tests = (long long)ctx->h_status->face_tests;
    }
    return st;
}

// DTFE on a device batch with the brick rasteriser.  Stages: bin the tets
// into bricks, star volumes, densities, rasterise (FP64 values of the
// ill-conditioned tets inline).  Once the brick shape is known (autotuned on
// the first call per context and mode) the blocks alternate between two
// streams, each block its own segment of the bins; TESSGPU_BATCH_OVERLAP=0
// runs each stage over all blocks in one launch instead.
static tessgpu_status dtfe_batch_bricks(tessgpu_ctx* ctx, tessgpu_batch* bt, const tessgpu_dense_params* p,
                                        const GridDesc& g, const float* gmax, float* target, float* d_grid,
                                        const int* d_zl, int L, long long Gout, int var, long long nbricks,
                                        tessgpu_dense_info* info)
{
    cudaStream_t s = ctx->stream;
    const int nb = bt->nb;
    const long long G = (long long)p->glo_num_idx[0] * p->glo_num_idx[1] * p->glo_num_idx[2];
    if (!bt->W || bt->pooled)
    {
        BALLOC(SLOT_W, sizeof(StarSum) * (bt->N ? bt->N : 1), bt->W);
        BALLOC(SLOT_RHO32, sizeof(float) * (bt->N ? bt->N : 1), bt->rho32);
        BALLOC(SLOT_RHO64, sizeof(double) * (bt->N ? bt->N : 1), bt->rho64);
    }
    int* owner = nullptr;
    if (bt->keep_debug)
    {
        if (!bt->d_owner || bt->owner_n < G || bt->pooled)
            BALLOC(SLOT_OUT, sizeof(int) * G, bt->d_owner);
        CK(cudaMemsetAsync(bt->d_owner, 0xff, sizeof(int) * G, s));
        bt->owner_n = G;
        owner = bt->d_owner;
    }
    const double scale = star_sum_scale(g.dmin, g.dmax, p->mode == TESSGPU_MODE_FP64);
    StarSum* W = (StarSum*)bt->W;
    BrickBins bins;
    tessgpu_status st;
    if ((st = brick_bins(ctx, nbricks, nb, bt->T, &bins)) != TESSGPU_OK)
        return st;
    CK(cudaMemsetAsync(bins.pair_cursor, 0, sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(W, 0, sizeof(StarSum) * (bt->N ? bt->N : 1), s));
    const char* ov = getenv("TESSGPU_BATCH_OVERLAP");
    const bool overlap = var >= 0 && !(ov && *ov && atoi(ov) == 0) && !p->project && nb > 1;
    if (overlap)
    {
        if (!ctx->cs2) CK(cudaStreamCreateWithFlags(&ctx->cs2, cudaStreamNonBlocking));
        while ((int)ctx->pipe_ev.size() < 2 * nb + 2)
        {
            cudaEvent_t e;
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            ctx->pipe_ev.push_back(e);
        }
        CK(cudaEventRecord(ctx->pipe_ev[2 * nb + 1], s));
        CK(cudaStreamWaitEvent(ctx->cs2, ctx->pipe_ev[2 * nb + 1], 0));
        for (int k = 0; k < nb; ++k)
        {
            const BlockDesc& d = bt->hb[k];
            cudaStream_t sk = (k & 1) ? ctx->cs2 : s;
            const int e0 = smark(ctx, sk);
            bricks_reset(ctx, bt->hb, k, k + 1, nbricks, bins, sk);
            bricks_star(ctx, p->mode, var, bt->d_blocks, nb, d.t_off, d.nt, bt->pos, bt->tv, W, scale, g, bins, sk);
            const int e1 = smark(ctx, sk);
            bricks_place(ctx, var, bt->d_blocks, bt->hb, k, k + 1, nbricks, bins, bt->pos, bt->tv, g, target, sk);
            const int e2 = smark(ctx, sk);
            if (d.np)
            {
                launch_densities(W + d.p_off, d.np, p->mass, 1.0 / scale, bt->rho32 + d.p_off, bt->rho64 + d.p_off,
                                 ctx->d_status, sk);
                ctx->launches++;
            }
            const int e3 = smark(ctx, sk);
            bricks_raster(ctx, p->mode, var, bt->d_blocks, bt->hb, k, k + 1, nbricks, bins, bt->pos, bt->tv,
                          bt->rho32, bt->rho64, g, target, owner, sk);
            const int e4 = smark(ctx, sk);
            span(ctx, "star_volumes_bin_count", e0, e1);
            span(ctx, "bin_place", e1, e2);
            span(ctx, "densities", e2, e3);
            span(ctx, "raster", e3, e4);
            CK(cudaEventRecord(ctx->pipe_ev[nb + k], sk));
        }
        for (int k = nb - 1; k >= 0; --k)
            if (k & 1)
            {
                CK(cudaStreamWaitEvent(s, ctx->pipe_ev[nb + k], 0));
                break;
            }
        mark(ctx, "dtfe_blocks");
    }
    else
    {
        if (var >= 0)
        {
            bricks_reset(ctx, bt->hb, 0, nb, nbricks, bins, s);
            bricks_star(ctx, p->mode, var, bt->d_blocks, nb, 0, bt->T, bt->pos, bt->tv, W, scale, g, bins, s);
            mark(ctx, "star_volumes_bin_count");
            bricks_place(ctx, var, bt->d_blocks, bt->hb, 0, nb, nbricks, bins, bt->pos, bt->tv, g, target, s);
            mark(ctx, "bin_place");
        }
        else
        {
            launch_star_volumes(p->mode, (int)bt->T, bt->pos, bt->tv, W, scale, kTau, ctx->d_status, s);
            ctx->launches += bt->T ? 1 : 0;
            mark(ctx, "star_volumes");
        }
        launch_densities(W, (int)bt->N, p->mass, 1.0 / scale, bt->rho32, bt->rho64, ctx->d_status, s);
        mark(ctx, "densities");
        ctx->launches += bt->N ? 1 : 0;
        if (var < 0)
        {
            // autotune the brick shape: bin and rasterise with each, twice (the
            // first launch of a kernel also pays its module load); keep the fastest
            float best = 1e30f;
            cudaEvent_t e0, e1;
            CK(cudaEventCreate(&e0));
            CK(cudaEventCreate(&e1));
            for (int v = 0; v < brick_variants(); ++v)
            {
                const long long nbv = assign_bricks(bt->hb, v);
                CK(cudaMemcpyAsync(bt->d_blocks, bt->hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
                if ((st = brick_bins(ctx, nbv, nb, bt->T, &bins)) != TESSGPU_OK)
                    return st;
                float vbest = 1e30f;
                for (int rep = 0; rep < 2; ++rep)
                {
                    CK(cudaMemsetAsync(bins.pair_cursor, 0, sizeof(unsigned long long), s));
                    CK(cudaEventRecord(e0, s));
                    bricks_bin(ctx, v, bt->d_blocks, bt->hb, 0, nb, nbv, bins, bt->pos, bt->tv, g, target, s);
                    bricks_raster(ctx, p->mode, v, bt->d_blocks, bt->hb, 0, nb, nbv, bins, bt->pos, bt->tv,
                                  bt->rho32, bt->rho64, g, target, owner, s);
                    CK(cudaEventRecord(e1, s));
                    CK(cudaEventSynchronize(e1));
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    vbest = std::min(vbest, ms);
                }
                if (v < 8) ctx->tune_ms[p->mode][v] = vbest;
                if (vbest < best) { best = vbest; var = v; }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            CK(cudaStreamSynchronize(s));
            const Status& hs = *ctx->h_status;
            CK(cudaMemcpy(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost));
            if (hs.code && hs.code != TESSGPU_ERR_CAPACITY)
                return finish_status(ctx);
            if (hs.code == TESSGPU_ERR_CAPACITY)
                grow_pairs(ctx);
            ctx->raster_variant[p->mode] = var;
            bt->raster_variant[p->mode] = var;
            // the run itself, with the chosen shape
            return tessgpu_batch_dense(ctx, bt, p, d_grid, info);
        }
        bricks_raster(ctx, p->mode, var, bt->d_blocks, bt->hb, 0, nb, nbricks, bins, bt->pos, bt->tv, bt->rho32,
                      bt->rho64, g, target, owner, s);
        mark(ctx, "raster");
    }
    bt->raster_variant[p->mode] = var;
    if (p->project)
    {
        // surface density: the column integral of rho over each layer's z range
        launch_project_layers(target, p->glo_num_idx[0], p->glo_num_idx[1], d_zl + p->glo_num_idx[2], L, g.step[2],
                              d_grid, s);
        ctx->launches++;
        mark(ctx, "project_layers");
    }
    if (info)
    {
        CK(cudaMemsetAsync(ctx->d_max, 0, sizeof(float), s));
        launch_grid_max(d_grid, Gout, ctx->d_max, s);
        ctx->launches++;
        mark(ctx, "grid_max");
    }
    st = finish_status(ctx);
    if (st == TESSGPU_ERR_CAPACITY && !ctx->in_retry)
    {
        // the pair list was too small: size it for this call and run again
        grow_pairs(ctx);
        ctx->in_retry = true;
        st = tessgpu_batch_dense(ctx, bt, p, d_grid, info);
        ctx->in_retry = false;
        return st;
    }
    if (st != TESSGPU_OK || !info)
        return st;
    float mx = 0.0f;
    CK(cudaMemcpy(&mx, ctx->d_max, sizeof(float), cudaMemcpyDeviceToHost));
    std::memset(info, 0, sizeof(*info));
    for (int i = 0; i < 3; ++i)
    {
        info->data_mins[i] = g.dmin[i]; info->data_maxs[i] = g.dmax[i];
        info->grid_phys_mins[i] = g.gmin[i]; info->grid_phys_maxs[i] = gmax[i]; info->grid_step_size[i] = g.step[i];
    }
    const Status& hs = *ctx->h_status;
    info->max_dense = mx;
    info->tot_mass = hs.tot_mass;
    info->grid_pts_assigned = (long long)hs.assigned;
    info->fp64_tets = (long long)hs.fp64_tets;
    info->exact_tests = (long long)hs.exact_tests;
    info->rows_visited = (long long)hs.rows;
    info->points_tested = (long long)hs.candidates;
    info->raster_variant = var;
    for (int v = 0; v < 8; ++v)
        info->raster_variant_ms[v] = ctx->tune_ms[p->mode][v];
    info->grid_layers = L;
    info->grid_floats = Gout;
    unsigned long long pairs = 0;
    CK(cudaMemcpy(&pairs, bins.pair_cursor, sizeof(pairs), cudaMemcpyDeviceToHost));
    info->brick_pairs = (long long)pairs;
    return TESSGPU_OK;
}

// ---------------------------------------------------------------------------
// independent particle sets, each block with its own grid
// ---------------------------------------------------------------------------
extern "C" long long tessgpu_sets_grid_floats(int nsets, const int* glo_num_idx, long long* offsets)
{
    if (nsets <= 0 || !glo_num_idx) return -1;
    long long tot = 0;
    for (int b = 0; b < nsets; ++b)
    {
        if (offsets) offsets[b] = tot;
        long long n = 1;
        for (int k = 0; k < 3; ++k)
        {
            if (glo_num_idx[3 * b + k] < 2) return -1;
            n *= glo_num_idx[3 * b + k];
        }
        tot += n;
    }
    return tot;
}

// The independent sets on the row rasteriser: star volumes, densities, grid
// zeroing, one rasteriser launch over every set's tets and its FP64 fix-up
// pass (the block descriptors carry each set's grid); recorded into a CUDA
// graph when asked, as the brick path is.
static tessgpu_status dense_sets_rows(tessgpu_ctx* ctx, tessgpu_batch* bt, const int* glo_num_idx, float mass,
                                      float eps, int mode, float* d_out, int graph, tessgpu_dense_info* info,
                                      double scale, const GridDesc& g0, long long Gtot)
{
    cudaStream_t s = ctx->stream;
    const int nb = bt->nb;
    if (!bt->W || bt->pooled)
    {
        BALLOC(SLOT_W, sizeof(StarSum) * (bt->N ? bt->N : 1), bt->W);
        BALLOC(SLOT_RHO32, sizeof(float) * (bt->N ? bt->N : 1), bt->rho32);
        BALLOC(SLOT_RHO64, sizeof(double) * (bt->N ? bt->N : 1), bt->rho64);
    }
    if (!bt->fix_list || bt->pooled)
    {
        BALLOC(SLOT_FIX, sizeof(int) * (bt->T ? bt->T : 1), bt->fix_list);
        BALLOC(SLOT_FIXN, sizeof(int) * 2 * (nb + 1), bt->fix_count);
    }
    StarSum* W = bt->W;
    CK(cudaMemcpyAsync(bt->d_blocks, bt->hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
    const int var = 1;   // the per-block-grid row kernel has one launch configuration
    auto densities = [&](cudaStream_t rs) {
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), rs));
        CK(cudaMemsetAsync(W, 0, sizeof(StarSum) * (bt->N ? bt->N : 1), rs));
        launch_star_volumes(mode, (int)bt->T, bt->pos, bt->tv, W, scale, kTau, ctx->d_status, rs);
        launch_densities(W, (int)bt->N, mass, 1.0 / scale, bt->rho32, bt->rho64, ctx->d_status, rs);
        ctx->launches += (bt->T ? 1 : 0) + (bt->N ? 1 : 0);
        return TESSGPU_OK;
    };
    auto raster = [&](cudaStream_t rs, int v) {
        CK(cudaMemsetAsync(d_out, 0, sizeof(float) * Gtot, rs));
        CK(cudaMemsetAsync(bt->fix_count, 0, sizeof(int), rs));
        int* next = bt->fix_count + (nb + 1);   // the persistent rasteriser's chunk counter
        CK(cudaMemsetAsync(next, 0, sizeof(int), rs));
        launch_raster(mode, v, bt->d_blocks, nb, (int)bt->T, bt->pos, bt->tv, bt->rho32, bt->rho64, g0, kTau,
                      d_out, nullptr, bt->fix_list, bt->fix_count, ctx->d_status, rs, nullptr, nullptr, 0, true,
                      next);
        ctx->launches += bt->T ? 1 : 0;
        if (mode != TESSGPU_MODE_FP64)
        {
            launch_raster_fix(bt->d_blocks, nb, (int)bt->T, bt->pos, bt->tv, bt->rho32, bt->rho64, g0, d_out,
                              nullptr, bt->fix_list, bt->fix_count, ctx->d_status, rs, true);
            ctx->launches += bt->T ? 1 : 0;
        }
        return TESSGPU_OK;
    };
    tessgpu_status st;
    std::vector<long long> key = { 1000 + (long long)mode, (long long)var, (long long)(size_t)d_out,
                                   (long long)(size_t)bt->W, (long long)(size_t)bt->fix_list };
    for (int i = 0; i < 3 * nb; ++i) key.push_back(glo_num_idx[i]);
    long long mbits = 0, ebits = 0;
    std::memcpy(&mbits, &mass, sizeof(float));
    std::memcpy(&ebits, &eps, sizeof(float));
    key.push_back(mbits);
    key.push_back(ebits);
    auto record = [&](cudaStream_t rs) {
        tessgpu_status r = densities(rs);
        return r != TESSGPU_OK ? r : raster(rs, var);
    };
    const long long launches0 = ctx->launches;
    if (graph)
    {
        if (!bt->sets_exec || bt->sets_key != key)
        {
            if (bt->sets_exec) { cudaGraphExecDestroy(bt->sets_exec); bt->sets_exec = nullptr; }
            if (bt->sets_graph) { cudaGraphDestroy(bt->sets_graph); bt->sets_graph = nullptr; }
            if (!ctx->cap) CK(cudaStreamCreateWithFlags(&ctx->cap, cudaStreamNonBlocking));
            CK(cudaStreamSynchronize(s));
            CK(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal));
            tessgpu_status rs = record(ctx->cap);
            cudaGraph_t gr = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(ctx->cap, &gr);
            if (rs != TESSGPU_OK) { if (gr) cudaGraphDestroy(gr); return rs; }
            CK(ce);
            bt->sets_graph = gr;
            CK(cudaGraphInstantiate(&bt->sets_exec, gr, 0));
            bt->sets_key = key;
        }
        ctx->launches = launches0;
        CK(cudaGraphLaunch(bt->sets_exec, s));
        ctx->launches += bt->T ? (mode == TESSGPU_MODE_FP64 ? 3 : 4) : 1;
    }
    else if ((st = record(s)) != TESSGPU_OK)
        return st;
    if ((st = finish_status(ctx)) != TESSGPU_OK || !info)
        return st;
    std::memset(info, 0, sizeof(*info));
    const Status& hs = *ctx->h_status;
    info->grid_pts_assigned = (long long)hs.assigned;
    info->fp64_tets = (long long)hs.fp64_tets;
    info->exact_tests = (long long)hs.exact_tests;
    info->rows_visited = (long long)hs.rows;
    info->points_tested = (long long)hs.candidates;
    info->raster_variant = var;
    for (int v = 0; v < 8; ++v)
        info->raster_variant_ms[v] = ctx->tune_ms[mode][v];
    info->grid_floats = Gtot;
    return TESSGPU_OK;
}

// DTFE of every block of the batch as an independent set: block b is
// dense() over that one block onto its own glo_num_idx[3b..3b+2] grid, at
// d_out + offset b (tessgpu_sets_grid_floats).  Stages over all sets at once:
// star volumes with the brick pair counts, densities, the bins' scan and
// scatter, one persistent rasteriser launch whose CTAs take (brick, chunk)
// items of every set from one device counter.  graph != 0 records the step
// into a CUDA graph on the first call with these sets and replays it after
// (the brick shape is autotuned first, without the graph).
extern "C" tessgpu_status tessgpu_batch_dense_sets(tessgpu_ctx* ctx, tessgpu_batch* bt, const int* glo_num_idx,
                                                   float mass, float eps, int mode, float* d_out, int graph,
                                                   tessgpu_dense_info* info)
{
    if (!ctx || !bt || !glo_num_idx || !d_out || (mode != TESSGPU_MODE_MIXED && mode != TESSGPU_MODE_FP64))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad dense_sets arguments");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int nb = bt->nb;
    std::vector<long long> off(nb);
    const long long Gtot = tessgpu_sets_grid_floats(nb, glo_num_idx, off.data());
    if (Gtot < 0)
        return set_err(ctx, TESSGPU_ERR_INVALID, "a set's grid has fewer than 2 points on an axis");
    // each set's grid: dense() over its one block (DataBounds = its bounds)
    float umin[3] = { 0, 0, 0 }, umax[3] = { 0, 0, 0 };
    for (int b = 0; b < nb; ++b)
    {
        tessgpu_dense_params p;
        std::memset(&p, 0, sizeof(p));
        p.alg = TESSGPU_DENSE_DTFE;
        p.mode = mode;
        p.mass = mass;
        p.eps = eps;
        for (int k = 0; k < 3; ++k) p.glo_num_idx[k] = glo_num_idx[3 * b + k];
        float dmin[3], dmax[3], gmin[3], gmax[3], step[3];
        data_bounds(1, &bt->blocks[b], &p, dmin, dmax);
        grid_step_params(&p, dmin, dmax, gmin, gmax, step);
        BlockDesc& d = bt->hb[b];
        block_grid_params(bt->blocks[b], gmin, step, eps, dmin, dmax, p.glo_num_idx, d.gmin_idx, d.gmax_idx,
                          d.gnum_idx);
        for (int k = 0; k < 3; ++k)
        {
            d.gmin_idx[k] = std::max(d.gmin_idx[k], 0);
            d.gmax_idx[k] = std::min(d.gmax_idx[k], p.glo_num_idx[k] - 1);
            d.grid.gmin[k] = gmin[k];
            d.grid.step[k] = step[k];
            d.grid.inv_step[k] = 1.0f / step[k];
            d.grid.n[k] = p.glo_num_idx[k];
            if (b == 0 || dmin[k] < umin[k]) umin[k] = dmin[k];
            if (b == 0 || dmax[k] > umax[k]) umax[k] = dmax[k];
        }
        d.grid.off = off[b];
    }
    // one fixed-point scale for every set (the largest box): sums stay exact
    const double scale = star_sum_scale(umin, umax, mode == TESSGPU_MODE_FP64);
    GridDesc g0;
    std::memset(&g0, 0, sizeof(g0));
    for (int k = 0; k < 3; ++k)
    {
        g0.dmin[k] = umin[k];
        g0.dmax[k] = umax[k];
    }
    if (ctx->rows)
        return dense_sets_rows(ctx, bt, glo_num_idx, mass, eps, mode, d_out, graph, info, scale, g0, Gtot);
    int var = ctx->sets_variant[mode];
    const char* env = getenv("TESSGPU_RASTER_VARIANT");
    if (var < 0 && env && *env)
        var = ctx->sets_variant[mode] = std::min(std::max(atoi(env), 0), brick_variants() - 1);
    if (!bt->W || bt->pooled)
    {
        BALLOC(SLOT_W, sizeof(StarSum) * (bt->N ? bt->N : 1), bt->W);
        BALLOC(SLOT_RHO32, sizeof(float) * (bt->N ? bt->N : 1), bt->rho32);
        BALLOC(SLOT_RHO64, sizeof(double) * (bt->N ? bt->N : 1), bt->rho64);
    }
    StarSum* W = (StarSum*)bt->W;
    BrickBins bins;
    tessgpu_status st;
    if (var < 0)
    {
        // autotune the brick shape on these sets (bin + rasterise, twice each)
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), s));
        CK(cudaMemsetAsync(W, 0, sizeof(StarSum) * (bt->N ? bt->N : 1), s));
        launch_star_volumes(mode, (int)bt->T, bt->pos, bt->tv, W, scale, kTau, ctx->d_status, s);
        launch_densities(W, (int)bt->N, mass, 1.0 / scale, bt->rho32, bt->rho64, ctx->d_status, s);
        ctx->launches += 2;
        float best = 1e30f;
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        for (int v = 0; v < brick_variants(); ++v)
        {
            const long long nbv = assign_bricks(bt->hb, v);
            CK(cudaMemcpyAsync(bt->d_blocks, bt->hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
            if ((st = brick_bins(ctx, nbv, nb, bt->T, &bins)) != TESSGPU_OK)
                return st;
            float vbest = 1e30f;
            for (int rep = 0; rep < 2; ++rep)
            {
                CK(cudaMemsetAsync(bins.pair_cursor, 0, sizeof(unsigned long long), s));
                CK(cudaEventRecord(e0, s));
                bricks_bin(ctx, v, bt->d_blocks, bt->hb, 0, nb, nbv, bins, bt->pos, bt->tv, g0, d_out, s);
                bricks_raster(ctx, mode, v, bt->d_blocks, bt->hb, 0, nb, nbv, bins, bt->pos, bt->tv, bt->rho32,
                              bt->rho64, g0, d_out, nullptr, s);
                CK(cudaEventRecord(e1, s));
                CK(cudaEventSynchronize(e1));
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                vbest = std::min(vbest, ms);
            }
            if (v < 8) ctx->tune_ms[mode][v] = vbest;
            if (vbest < best) { best = vbest; var = v; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        CK(cudaMemcpy(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost));
        if (ctx->h_status->code == TESSGPU_ERR_CAPACITY)
            grow_pairs(ctx);
        else if (ctx->h_status->code)
            return finish_status(ctx);
        ctx->sets_variant[mode] = var;
    }
    const long long nbricks = assign_bricks(bt->hb, var);
    if ((st = brick_bins(ctx, nbricks, nb, bt->T, &bins)) != TESSGPU_OK)
        return st;
    // what a recorded step depends on: the sets' grids, the mode, the shape and the scratch
    std::vector<long long> key = { (long long)mode, (long long)var, (long long)(size_t)d_out,
                                   (long long)(size_t)bins.pairs, bins.pair_cap,
                                   (long long)(size_t)bins.cnt, (long long)(size_t)bt->W };
    for (int i = 0; i < 3 * nb; ++i) key.push_back(glo_num_idx[i]);
    long long mbits = 0, ebits = 0;
    std::memcpy(&mbits, &mass, sizeof(float));
    std::memcpy(&ebits, &eps, sizeof(float));
    key.push_back(mbits);
    key.push_back(ebits);
    // the descriptors go up before the step (a graph cannot hold a copy from pageable memory)
    CK(cudaMemcpyAsync(bt->d_blocks, bt->hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
    auto record = [&](cudaStream_t rs) {
        CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), rs));
        CK(cudaMemsetAsync(bins.pair_cursor, 0, sizeof(unsigned long long), rs));
        CK(cudaMemsetAsync(W, 0, sizeof(StarSum) * (bt->N ? bt->N : 1), rs));
        bricks_reset(ctx, bt->hb, 0, nb, nbricks, bins, rs);
        bricks_star(ctx, mode, var, bt->d_blocks, nb, 0, bt->T, bt->pos, bt->tv, W, scale, g0, bins, rs);
        bricks_place(ctx, var, bt->d_blocks, bt->hb, 0, nb, nbricks, bins, bt->pos, bt->tv, g0, d_out, rs);
        launch_densities(W, (int)bt->N, mass, 1.0 / scale, bt->rho32, bt->rho64, ctx->d_status, rs);
        ctx->launches += bt->N ? 1 : 0;
        bricks_raster(ctx, mode, var, bt->d_blocks, bt->hb, 0, nb, nbricks, bins, bt->pos, bt->tv, bt->rho32,
                      bt->rho64, g0, d_out, nullptr, rs);
        return TESSGPU_OK;
    };
    const long long launches0 = ctx->launches;
    if (graph)
    {
        if (!bt->sets_exec || bt->sets_key != key)
        {
            if (bt->sets_exec) { cudaGraphExecDestroy(bt->sets_exec); bt->sets_exec = nullptr; }
            if (bt->sets_graph) { cudaGraphDestroy(bt->sets_graph); bt->sets_graph = nullptr; }
            // recorded on the context's own capture stream (the legacy default
            // stream cannot be captured), launched on the context's stream
            if (!ctx->cap) CK(cudaStreamCreateWithFlags(&ctx->cap, cudaStreamNonBlocking));
            CK(cudaStreamSynchronize(s));
            CK(cudaStreamBeginCapture(ctx->cap, cudaStreamCaptureModeThreadLocal));
            tessgpu_status rs = record(ctx->cap);
            cudaGraph_t gr = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(ctx->cap, &gr);
            if (rs != TESSGPU_OK) { if (gr) cudaGraphDestroy(gr); return rs; }
            CK(ce);
            bt->sets_graph = gr;
            CK(cudaGraphInstantiate(&bt->sets_exec, gr, 0));
            bt->sets_key = key;
        }
        ctx->launches = launches0;   // counted per replay below
        CK(cudaGraphLaunch(bt->sets_exec, s));
        ctx->launches += bt->T ? 6 : 2;
    }
    else if ((st = record(s)) != TESSGPU_OK)
        return st;
    st = finish_status(ctx);
    if (st == TESSGPU_ERR_CAPACITY && !ctx->in_retry)
    {
        grow_pairs(ctx);
        ctx->in_retry = true;
        st = tessgpu_batch_dense_sets(ctx, bt, glo_num_idx, mass, eps, mode, d_out, graph, info);
        ctx->in_retry = false;
        return st;
    }
    if (st != TESSGPU_OK || !info)
        return st;
    std::memset(info, 0, sizeof(*info));
    const Status& hs = *ctx->h_status;
    info->grid_pts_assigned = (long long)hs.assigned;
    info->fp64_tets = (long long)hs.fp64_tets;
    info->exact_tests = (long long)hs.exact_tests;
    info->rows_visited = (long long)hs.rows;
    info->points_tested = (long long)hs.candidates;
    info->raster_variant = var;
    for (int v = 0; v < 8; ++v)
        info->raster_variant_ms[v] = ctx->tune_ms[mode][v];
    info->grid_floats = Gtot;
    unsigned long long pairs = 0;
    CK(cudaMemcpy(&pairs, bins.pair_cursor, sizeof(pairs), cudaMemcpyDeviceToHost));
    info->brick_pairs = (long long)pairs;
    return TESSGPU_OK;
}

extern "C" tessgpu_status tessgpu_batch_debug_outputs(tessgpu_ctx* ctx, tessgpu_batch* bt, int* cell_counts,
                                                      int* owner, float* rho)
{
    if (!ctx || !bt) return TESSGPU_ERR_INVALID;
    if (cell_counts)
    {
        if (!bt->d_cell_counts) return set_err(ctx, TESSGPU_ERR_INVALID, "no DENSE_TESS debug output kept");
        CK(cudaMemcpy(cell_counts, bt->d_cell_counts, sizeof(int) * bt->C, cudaMemcpyDeviceToHost));
    }
    if (owner)
    {
        if (!bt->d_owner) return set_err(ctx, TESSGPU_ERR_INVALID, "no DTFE debug output kept");
        CK(cudaMemcpy(owner, bt->d_owner, sizeof(int) * bt->owner_n, cudaMemcpyDeviceToHost));
    }
    if (rho)
    {
        if (!bt->rho32) return set_err(ctx, TESSGPU_ERR_INVALID, "no DTFE run on this batch");
        CK(cudaMemcpy(rho, bt->rho32, sizeof(float) * bt->N, cudaMemcpyDeviceToHost));
    }
    return TESSGPU_OK;
}

// ---------------------------------------------------------------------------
// host-buffer entry points
// ---------------------------------------------------------------------------
static tessgpu_block single_block(const float* particles, int np, const int* tets, int nt, const int* v2t)
{
    tessgpu_block b;
    std::memset(&b, 0, sizeof(b));
    b.num_orig_particles = np;
    b.num_particles = np;
    b.particles = particles;
    b.num_tets = nt;
    b.tets = tets;
    b.vert_to_tet = v2t;
    for (int i = 0; i < 3; ++i) { b.bounds_max[i] = 1; b.data_max[i] = 1; }
    return b;
}

extern "C" tessgpu_status tessgpu_fill_vert_to_tet(tessgpu_ctx* ctx, int num_particles, const int* tets, int num_tets,
                                                   int* vert_to_tet)
{
    if (!ctx || num_particles < 0 || num_tets < 0 || (num_particles && !vert_to_tet) || (num_tets && !tets))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    if (!num_particles) return TESSGPU_OK;
    // particles are not read by this call; a zero stand-in keeps the batch layout
    std::vector<float> zero(3 * (size_t)num_particles, 0.0f);
    tessgpu_block b = single_block(zero.data(), num_particles, tets, num_tets, nullptr);
    tessgpu_batch* bt = nullptr;
    tessgpu_status s = batch_build(ctx, 1, &b, false, true, &bt);
    if (s == TESSGPU_OK)
        s = cuda_check(ctx, cudaMemcpy(vert_to_tet, bt->v2t, sizeof(int) * num_particles, cudaMemcpyDeviceToHost),
                       "cudaMemcpy");
    tessgpu_batch_free(bt);
    return s;
}

extern "C" tessgpu_status tessgpu_fill_circumcenters(tessgpu_ctx* ctx, const float* particles, int num_particles,
                                                     const int* tets, int num_tets, float* out)
{
    if (!ctx || num_particles < 0 || num_tets < 0 || (num_tets && (!tets || !out || !particles)))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    if (!num_tets) return TESSGPU_OK;
    std::vector<int> none(num_particles ? num_particles : 1, -1);
    tessgpu_block b = single_block(particles, num_particles, tets, num_tets, none.data());
    tessgpu_batch* bt = nullptr;
    tessgpu_status s = batch_build(ctx, 1, &b, false, true, &bt);
    if (s == TESSGPU_OK)
    {
        cudaError_t e;
        float4* cc = (float4*)pool_get(ctx, SLOT_CC, sizeof(float4) * num_tets, &e);
        s = cuda_check(ctx, e, "cudaMalloc");
        if (s == TESSGPU_OK)
        {
            launch_circumcenters(bt->pos, bt->tv, num_tets, cc, ctx->stream);
            ctx->launches++;
            // float4 -> 3 floats per tet
            s = cuda_check(ctx, cudaMemcpy2D(out, 3 * sizeof(float), cc, sizeof(float4), 3 * sizeof(float), num_tets,
                                             cudaMemcpyDeviceToHost), "cudaMemcpy2D");
        }
    }
    tessgpu_batch_free(bt);
    return s;
}

static tessgpu_status cells_call(tessgpu_ctx* ctx, int mode, const float* particles, int num_particles,
                                 const int* tets, int num_tets, const int* v2t, int n, int* out_i, float* out_f,
                                 float* out_area, double* out_d)
{
    if (!ctx || n < 0 || n > num_particles || num_tets < 0 || (num_tets && !tets) || (num_particles && !particles))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    if (!n) return TESSGPU_OK;
    tessgpu_block b = single_block(particles, num_particles, tets, num_tets, v2t);
    b.num_orig_particles = n;
    tessgpu_batch* bt = nullptr;
    tessgpu_status s = batch_build(ctx, 1, &b, false, true, &bt);
    if (s != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
    cudaError_t e = cudaSuccess;
    void* d_out = pool_get(ctx, SLOT_OUT, sizeof(double) * n, &e);
    void* d_area = out_area ? pool_get(ctx, SLOT_OUT2, sizeof(float) * n, &e) : nullptr;
    if ((s = cuda_check(ctx, e, "cudaMalloc")) != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
    GridDesc g;
    std::memset(&g, 0, sizeof(g));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), ctx->stream));
    if (mode == CELL_VOLUME || mode == CELL_DENSE_TESS)
    {
        float4* cc = (float4*)pool_get(ctx, SLOT_CC, sizeof(float4) * (num_tets ? num_tets : 1), &e);
        if ((s = cuda_check(ctx, e, "cudaMalloc")) != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
        launch_circumcenters(bt->pos, bt->tv, num_tets, cc, ctx->stream);
        bt->cc = cc;
        ctx->launches++;
    }
    if (mode == CELL_VOLUME_F64)
    {
        double* cc64 = (double*)pool_get(ctx, SLOT_CC64, sizeof(double) * 3 * (num_tets ? num_tets : 1), &e);
        if ((s = cuda_check(ctx, e, "cudaMalloc")) != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
        launch_circumcenters_f64(bt->pos, bt->tv, num_tets, cc64, ctx->stream);
        bt->cc64 = cc64;
        ctx->launches++;
    }
    launch_cells(mode, bt->d_blocks, bt->d_c_off, 1, n, bt->pos, bt->tv, bt->tn, bt->v2t, bt->cc, bt->cc64, g,
                 nullptr, (int*)d_out, (float*)d_out, (float*)d_area, (double*)d_out, nullptr, ctx->d_status,
                 ctx->stream);
    ctx->launches++;
    s = finish_status(ctx);
    if (s == TESSGPU_OK)
    {
        size_t bytes = mode == CELL_VOLUME_F64 ? sizeof(double) * n : sizeof(int) * n;
        void* host = mode == CELL_COMPLETE ? (void*)out_i : mode == CELL_VOLUME ? (void*)out_f : (void*)out_d;
        s = cuda_check(ctx, cudaMemcpy(host, d_out, bytes, cudaMemcpyDeviceToHost), "cudaMemcpy");
        if (s == TESSGPU_OK && out_area)
            s = cuda_check(ctx, cudaMemcpy(out_area, d_area, sizeof(float) * n, cudaMemcpyDeviceToHost), "cudaMemcpy");
    }
    tessgpu_batch_free(bt);
    return s;
}

extern "C" tessgpu_status tessgpu_complete_all(tessgpu_ctx* ctx, const float* particles, int num_particles,
                                               const int* tets, int num_tets, const int* v2t, int n, int* out)
{
    if (n && !out) return set_err(ctx, TESSGPU_ERR_INVALID, "null output");
    return cells_call(ctx, CELL_COMPLETE, particles, num_particles, tets, num_tets, v2t, n, out, nullptr, nullptr,
                      nullptr);
}

extern "C" tessgpu_status tessgpu_volumes(tessgpu_ctx* ctx, const float* particles, int num_particles, const int* tets,
                                          int num_tets, const int* v2t, int n, float* volumes, float* areas)
{
    if (n && !volumes) return set_err(ctx, TESSGPU_ERR_INVALID, "null output");
    return cells_call(ctx, CELL_VOLUME, particles, num_particles, tets, num_tets, v2t, n, nullptr, volumes, areas,
                      nullptr);
}

extern "C" tessgpu_status tessgpu_volumes_f64(tessgpu_ctx* ctx, const float* particles, int num_particles,
                                              const int* tets, int num_tets, const int* v2t, int n, double* volumes)
{
    if (n && !volumes) return set_err(ctx, TESSGPU_ERR_INVALID, "null output");
    return cells_call(ctx, CELL_VOLUME_F64, particles, num_particles, tets, num_tets, v2t, n, nullptr, nullptr,
                      nullptr, volumes);
}

__global__ void k_extract_box(const float* grid, int nx, int ny, const int* mn, const int* num, float* out)
{
    const long long n = (long long)num[0] * num[1] * num[2];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    {
        const int x = (int)(i % num[0]);
        const int y = (int)((i / num[0]) % num[1]);
        const int z = (int)(i / ((long long)num[0] * num[1]));
        out[i] = grid[((size_t)(mn[2] + z) * ny + (mn[1] + y)) * nx + (mn[0] + x)];
    }
}

// ---------------------------------------------------------------------------
// DTFE through host buffers, pipelined per block
// ---------------------------------------------------------------------------
// one block's particles: xyz -> float4
__global__ void k_pack_block(const float* raw, int np, float4* pos)
{
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        pos[p] = make_float4(raw[3 * (size_t)p], raw[3 * (size_t)p + 1], raw[3 * (size_t)p + 2], 0.0f);
}

// A box of the global grid (x fastest, nx * ny per z plane) into the same box of a host array
// the device addresses directly (pageable memory on a host whose GPU shares its page tables):
// one CTA per row of the box
__global__ void k_store_box(const float* __restrict__ grid, float* host, int nx, int ny, int x0, int y0, int z0,
                            int bx, int by, int bz)
{
    const long long rows = (long long)by * bz;
    // 16-byte accesses when every row starts on a 16-byte boundary at both ends
    const bool v4 = ((x0 | bx | nx) & 3) == 0 && (((size_t)host | (size_t)grid) & 15) == 0;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x)
    {
        const int y = y0 + (int)(r % by), z = z0 + (int)(r / by);
        const size_t base = ((size_t)z * ny + y) * nx + x0;
        if (v4)
        {
            const float4* src = reinterpret_cast<const float4*>(grid + base);
            float4* dst = reinterpret_cast<float4*>(host + base);
            for (int x = threadIdx.x; x < (bx >> 2); x += blockDim.x) dst[x] = __ldg(src + x);
        }
        else
            for (int x = threadIdx.x; x < bx; x += blockDim.x) host[base + x] = grid[base + x];
    }
}

// n floats into a host array the device addresses directly
__global__ void k_store_run(const float* __restrict__ src, float* dst, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if ((((size_t)src | (size_t)dst) & 15) == 0)
    {
        const size_t n4 = n >> 2;
        for (size_t i = i0; i < n4; i += stride)
            reinterpret_cast<float4*>(dst)[i] = __ldg(reinterpret_cast<const float4*>(src) + i);
        i0 += n4 << 2;
    }
    for (size_t i = i0; i < n; i += stride)
        dst[i] = src[i];
}

// CTAs of a kernel that reads or writes host memory directly: each waits on
// the host link for most of its life, so a few keep the link busy and leave
// the SMs to the compute streams (TESSGPU_HOSTIO_CTAS overrides).  At 2M ->
// 512^3 from pageable arrays: 304 CTAs 8.2 ms a call, 192 7.3-7.5, 128
// 7.3-7.4, 96 7.5, 64 8.9 (the download then waits on the link).
static int hostio_ctas()
{
    const char* e = getenv("TESSGPU_HOSTIO_CTAS");
    const int n = e && *e ? atoi(e) : 0;
    return n > 0 ? n : 128;
}

// one block's tet_t vertices -> batch-wide particle indices, checked
__global__ void k_ingest_verts(const int4* raw, int nt, int np, int p_off, int4* tv, Status* st)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x)
    {
        int4 v = raw[2 * (size_t)t];   // verts; raw[2t + 1] holds the neighbours
        if ((unsigned)v.x >= (unsigned)np || (unsigned)v.y >= (unsigned)np || (unsigned)v.z >= (unsigned)np ||
            (unsigned)v.w >= (unsigned)np)
        {
            fail(st, TESSGPU_ERR_BAD_MESH, t);
            v = make_int4(0, 0, 0, 0);
        }
        tv[t] = make_int4(v.x + p_off, v.y + p_off, v.z + p_off, v.w + p_off);
    }
}

// The host-buffer DTFE call with its copies overlapped: block b's particles
// and tets go up on one copy stream while the compute stream works on the
// blocks before it (ingest, star volumes, densities, rasteriser and its FP64
// fix-up, block by block), and each z-slab of the grid goes down on another
// copy stream as soon as the last block that writes into it is done.  Same
// kernels and results as the batch path; it needs the rasteriser's launch
// variant chosen already.
// true when the device reads and writes pageable host memory directly (its page tables shared with
// the host's); asked once per context
static bool pageable_access(tessgpu_ctx* ctx)
{
    if (ctx->pageable_access < 0)
    {
        int a = 0;
        if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, ctx->device) != cudaSuccess) a = 0;
        cudaGetLastError();
        ctx->pageable_access = a ? 1 : 0;
    }
    return ctx->pageable_access == 1;
}

// host memory that is neither pinned nor registered with CUDA
static bool is_pageable(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return true;
    }
    return a.type == cudaMemoryTypeUnregistered;
}

static tessgpu_status dense_dtfe_pipelined(tessgpu_ctx* ctx, int nb, const tessgpu_block* blocks,
                                           const tessgpu_dense_params* p, int variant, float* host_grid,
                                           tessgpu_dense_info* info, float** d_grid_out)
{
    CK(cudaSetDevice(ctx->device));
    for (int i = 0; i < nb; ++i)
        if (blocks[i].num_particles < 0 || blocks[i].num_tets < 0 || blocks[i].num_orig_particles < 0 ||
            blocks[i].num_orig_particles > blocks[i].num_particles ||
            (blocks[i].num_particles && !blocks[i].particles) || (blocks[i].num_tets && !blocks[i].tets))
            return set_err(ctx, TESSGPU_ERR_INVALID, "block " + std::to_string(i) + " is malformed");
    if (!ctx->h2d) CK(cudaStreamCreateWithFlags(&ctx->h2d, cudaStreamNonBlocking));
    if (!ctx->d2h) CK(cudaStreamCreateWithFlags(&ctx->d2h, cudaStreamNonBlocking));
    if (!ctx->cs2) CK(cudaStreamCreateWithFlags(&ctx->cs2, cudaStreamNonBlocking));
    while ((int)ctx->pipe_ev.size() < 2 * nb + 2)
    {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->pipe_ev.push_back(e);
    }
    cudaStream_t s = ctx->stream;
    // descriptors and grid
    float dmin[3], dmax[3], gmin[3], gmax[3], step[3];
    data_bounds(nb, blocks, p, dmin, dmax);
    grid_step_params(p, dmin, dmax, gmin, gmax, step);
    GridDesc g;
    std::memset(&g, 0, sizeof(g));
    for (int i = 0; i < 3; ++i)
    {
        g.gmin[i] = gmin[i]; g.step[i] = step[i]; g.dmin[i] = dmin[i]; g.dmax[i] = dmax[i];
        g.n[i] = p->glo_num_idx[i];
        g.inv_step[i] = 1.0f / step[i];
    }
    g.eps = p->eps;
    g.mass = p->mass;
    g.div = step[0] * step[1] * step[2];
    std::vector<BlockDesc> hb(nb);
    long long N = 0, T = 0, C = 0;
    for (int i = 0; i < nb; ++i)
    {
        BlockDesc& d = hb[i];
        std::memset(&d, 0, sizeof(d));
        d.gid = blocks[i].gid;
        for (int k = 0; k < 3; ++k) { d.bmin[k] = blocks[i].bounds_min[k]; d.bmax[k] = blocks[i].bounds_max[k]; }
        d.p_off = (int)N; d.np = blocks[i].num_particles; d.norig = blocks[i].num_orig_particles;
        d.t_off = (int)T; d.nt = blocks[i].num_tets; d.c_off = (int)C;
        N += d.np; T += d.nt; C += d.norig;
        block_grid_params(blocks[i], gmin, step, p->eps, dmin, dmax, p->glo_num_idx, d.gmin_idx, d.gmax_idx,
                          d.gnum_idx);
        for (int k = 0; k < 3; ++k)
        {
            d.gmin_idx[k] = std::max(d.gmin_idx[k], 0);
            d.gmax_idx[k] = std::min(d.gmax_idx[k], p->glo_num_idx[k] - 1);
        }
    }
    if (N >= (1LL << 31) || T >= (1LL << 31))
        return set_err(ctx, TESSGPU_ERR_INVALID, "batch larger than 2^31 particles or tets");
    const long long area = (long long)p->glo_num_idx[0] * p->glo_num_idx[1];
    const long long G = area * p->glo_num_idx[2];
    set_block_grids(hb, g);
    const bool bricks = !ctx->rows;
    const long long nbricks = bricks ? assign_bricks(hb, variant) : 0;
    BrickBins bins;
    std::memset(&bins, 0, sizeof(bins));
    if (bricks)
    {
        tessgpu_status bs = brick_bins(ctx, nbricks, nb, T, &bins);
        if (bs != TESSGPU_OK) return bs;
    }
    cudaError_t e = cudaSuccess;
    auto get = [&](int slot, size_t bytes) { cudaError_t ee; void* q = pool_get(ctx, slot, bytes, &ee);
                                             if (ee != cudaSuccess) e = ee; return q; };
    BlockDesc* d_blocks = (BlockDesc*)get(SLOT_BLOCKS, sizeof(BlockDesc) * nb);
    float4* pos = (float4*)get(SLOT_POS, sizeof(float4) * std::max(N, 1LL));
    int4* tv = (int4*)get(SLOT_TV, sizeof(int4) * std::max(T, 1LL));
    char* stage = (char*)get(SLOT_STAGE, 32 * (size_t)T + 12 * (size_t)N + 16);
    StarSum* W = (StarSum*)get(SLOT_W, sizeof(StarSum) * std::max(N, 1LL));
    float* rho32 = (float*)get(SLOT_RHO32, sizeof(float) * std::max(N, 1LL));
    double* rho64 = (double*)get(SLOT_RHO64, sizeof(double) * std::max(N, 1LL));
    int* fix = bricks ? nullptr : (int*)get(SLOT_FIX, sizeof(int) * std::max(T, 1LL));
    // per block: the FP64 fix-up list length, then the rasteriser's chunk counter
    int* fixn = (int*)get(SLOT_FIXN, sizeof(int) * 2 * nb);
    float* grid = (float*)get(SLOT_GRID, sizeof(float) * G);
    CK(e);
    *d_grid_out = grid;
    int4* stage_tets = (int4*)stage;                     // 32 B per tet, first: 16-byte aligned
    float* stage_xyz = (float*)(stage + 32 * (size_t)T);

    // processing order: by first z index of the block's grid box; slab l of
    // the grid (between consecutive distinct first z indices) goes down after
    // the last block whose box reaches into it
    std::vector<int> order(nb);
    for (int i = 0; i < nb; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return hb[a].gmin_idx[2] < hb[b].gmin_idx[2]; });
    std::vector<int> zmin(nb), zl;
    for (int i = 0; i < nb; ++i) zmin[i] = hb[i].gmin_idx[2];
    const int L = z_layers(zmin, p->glo_num_idx[2], zl);
    std::vector<int> slab_lo(L, -1), slab_hi(L, -1), slab_ready(L, -1);
    for (int z = 0; z < p->glo_num_idx[2]; ++z)
    {
        if (slab_lo[zl[z]] < 0) slab_lo[zl[z]] = z;
        slab_hi[zl[z]] = z;
    }
    for (int k = 0; k < nb; ++k)
    {
        const BlockDesc& d = hb[order[k]];
        for (int l = 0; l < L; ++l)
            if (d.gmax_idx[2] >= slab_lo[l] && d.gmin_idx[2] <= slab_hi[l])
                slab_ready[l] = k;
    }
    // when the blocks' grid boxes tile the grid (the usual case), each box
    // goes down as soon as its block is done, so only the last box trails
    const bool tiles = boxes_tile(hb, p->glo_num_idx);
    // pageable host arrays on a device that addresses them: the ingest kernels read the caller's
    // particles and tets in place, and the grid boxes are stored into the caller's array by a kernel on
    // the download stream (a copy from or to pageable memory would wait on the host thread, stalling
    // the pipeline); pinned or registered arrays go through the copy engines
    bool direct_in = pageable_access(ctx);
    for (int i = 0; i < nb && direct_in; ++i)
        if ((blocks[i].num_particles && !is_pageable(blocks[i].particles)) ||
            (blocks[i].num_tets && !is_pageable(blocks[i].tets)) ||
            (blocks[i].num_tets && ((uintptr_t)blocks[i].tets & 15)))
            direct_in = false;
    const bool direct_out = host_grid && pageable_access(ctx) && is_pageable(host_grid);

    const double scale = star_sum_scale(dmin, dmax, p->mode == TESSGPU_MODE_FP64);

    ctx->nmarks = 0;
    ctx->nsev = 0;
    ctx->spans.clear();
    mark(ctx, "start");
    // the status word is zeroed first: the upload stream's ingest kernels may
    // report into it (pageable arrays read in place)
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), s));
    // the copy streams start after whatever the compute stream was doing with the pool
    cudaEvent_t ev0 = ctx->pipe_ev[2 * nb];
    CK(cudaEventRecord(ev0, s));
    CK(cudaStreamWaitEvent(ctx->h2d, ev0, 0));
    CK(cudaStreamWaitEvent(ctx->d2h, ev0, 0));
    // the first block goes up in quarters (particles first), so its ingest and
    // star volumes start after a quarter of its upload rather than all of it
    constexpr int kFirstParts = 4;
    for (int i = 0; i < 1 + kFirstParts; ++i)
        if (!ctx->first_ev[i]) CK(cudaEventCreateWithFlags(&ctx->first_ev[i], cudaEventDisableTiming));
    auto part = [&](const BlockDesc& d, int i) { return (long long)d.nt * i / kFirstParts; };
    for (int k = 0; k < nb; ++k)
    {
        const int b = order[k];
        const BlockDesc& d = hb[b];
        const int eu0 = smark(ctx, ctx->h2d);
        if (direct_in)
        {
            // the block's arrays are read where they lie, by kernels on this
            // stream (the copy engines' place when the arrays are pinned), so
            // they run ahead of the compute streams as the copies do; few CTAs,
            // since each mostly waits on the host link
            if (d.np)
            {
                k_pack_block<<<std::min(grid_small(d.np), hostio_ctas()), 256, 0, ctx->h2d>>>(blocks[b].particles,
                                                                                               d.np, pos + d.p_off);
                ctx->launches++;
            }
            if (k == 0)
                CK(cudaEventRecord(ctx->first_ev[0], ctx->h2d));
            for (int i = 0; i < (k == 0 ? kFirstParts : 1); ++i)
            {
                const long long t0 = k == 0 ? part(d, i) : 0, t1 = k == 0 ? part(d, i + 1) : d.nt;
                if (t1 > t0)
                {
                    k_ingest_verts<<<std::min(grid_small(t1 - t0), hostio_ctas()), 256, 0, ctx->h2d>>>(
                        reinterpret_cast<const int4*>(blocks[b].tets) + 2 * (size_t)t0, (int)(t1 - t0), d.np, d.p_off,
                        tv + d.t_off + t0, ctx->d_status);
                    ctx->launches++;
                }
                if (k == 0)
                    CK(cudaEventRecord(ctx->first_ev[1 + i], ctx->h2d));
            }
            CK(cudaEventRecord(ctx->pipe_ev[k], ctx->h2d));
            span(ctx, "upload", eu0, smark(ctx, ctx->h2d));
            continue;
        }
        if (k == 0)
        {
            if (d.np)
                CK(cudaMemcpyAsync(stage_xyz + 3 * (size_t)d.p_off, blocks[b].particles, 12 * (size_t)d.np,
                                   cudaMemcpyHostToDevice, ctx->h2d));
            CK(cudaEventRecord(ctx->first_ev[0], ctx->h2d));
            for (int i = 0; i < kFirstParts; ++i)
            {
                const long long t0 = part(d, i), t1 = part(d, i + 1);
                if (t1 > t0)
                    CK(cudaMemcpyAsync(stage_tets + 2 * ((size_t)d.t_off + t0), blocks[b].tets + 8 * t0,
                                       32 * (size_t)(t1 - t0), cudaMemcpyHostToDevice, ctx->h2d));
                CK(cudaEventRecord(ctx->first_ev[1 + i], ctx->h2d));
            }
            CK(cudaEventRecord(ctx->pipe_ev[k], ctx->h2d));
            span(ctx, "upload", eu0, smark(ctx, ctx->h2d));
            continue;
        }
        if (d.nt)
            CK(cudaMemcpyAsync(stage_tets + 2 * (size_t)d.t_off, blocks[b].tets, 32 * (size_t)d.nt,
                               cudaMemcpyHostToDevice, ctx->h2d));
        if (d.np)
            CK(cudaMemcpyAsync(stage_xyz + 3 * (size_t)d.p_off, blocks[b].particles, 12 * (size_t)d.np,
                               cudaMemcpyHostToDevice, ctx->h2d));
        CK(cudaEventRecord(ctx->pipe_ev[k], ctx->h2d));
        span(ctx, "upload", eu0, smark(ctx, ctx->h2d));
    }
    CK(cudaMemcpyAsync(d_blocks, hb.data(), sizeof(BlockDesc) * nb, cudaMemcpyHostToDevice, s));
    // the brick rasteriser writes every point of the blocks' boxes
    if (!bricks || !tiles)
        CK(cudaMemsetAsync(grid, 0, sizeof(float) * G, s));
    CK(cudaMemsetAsync(fixn, 0, sizeof(int) * 2 * nb, s));
    if (bricks)
        CK(cudaMemsetAsync(bins.pair_cursor, 0, sizeof(unsigned long long), s));
    // blocks alternate between two compute streams, so one block's launches
    // fill the SMs the previous block's last waves leave idle; they share
    // nothing but read-only descriptors, the status word (atomics) and the grid,
    // where each writes only its own box
    cudaEvent_t ev_setup = ctx->pipe_ev[2 * nb + 1];
    CK(cudaEventRecord(ev_setup, s));
    CK(cudaStreamWaitEvent(ctx->cs2, ev_setup, 0));
    const bool mixed = p->mode != TESSGPU_MODE_FP64;
    // TESSGPU_PIPELINE_STREAMS=1: every block's compute on one stream
    const char* psenv = getenv("TESSGPU_PIPELINE_STREAMS");
    const bool two_streams = !(psenv && *psenv && atoi(psenv) == 1);
    for (int k = 0; k < nb; ++k)
    {
        const int b = order[k];
        const BlockDesc& d = hb[b];
        cudaStream_t s = (two_streams && (k & 1)) ? ctx->cs2 : ctx->stream;
        CK(cudaStreamWaitEvent(s, k == 0 ? ctx->first_ev[0] : ctx->pipe_ev[k], 0));
        const int ec0 = smark(ctx, s);
        if (d.np)
        {
            if (!direct_in)   // (direct: packed on the upload stream)
            {
                k_pack_block<<<grid_small(d.np), 256, 0, s>>>(stage_xyz + 3 * (size_t)d.p_off, d.np, pos + d.p_off);
                ctx->launches++;
            }
            CK(cudaMemsetAsync(W + d.p_off, 0, sizeof(StarSum) * d.np, s));
        }
        if (bricks)
            bricks_reset(ctx, hb, b, b + 1, nbricks, bins, s);
        for (int i = 0; i < (k == 0 ? kFirstParts : 1); ++i)
        {
            // the tets in the parts they came up in (one part after the first block)
            const long long t0 = k == 0 ? part(d, i) : 0, t1 = k == 0 ? part(d, i + 1) : d.nt;
            if (k == 0)
                CK(cudaStreamWaitEvent(s, ctx->first_ev[1 + i], 0));
            if (t1 <= t0) continue;
            if (!direct_in)   // (direct: ingested on the upload stream)
            {
                k_ingest_verts<<<grid_small(t1 - t0), 256, 0, s>>>(stage_tets + 2 * ((size_t)d.t_off + t0),
                                                                    (int)(t1 - t0), d.np, d.p_off, tv + d.t_off + t0,
                                                                    ctx->d_status);
                ctx->launches++;
            }
            if (bricks)
                bricks_star(ctx, p->mode, variant, d_blocks, nb, d.t_off + t0, t1 - t0, pos, tv, W, scale, g, bins, s);
            else
            {
                launch_star_volumes(p->mode, (int)(t1 - t0), pos, tv + d.t_off + t0, W, scale, kTau, ctx->d_status,
                                    s);
                ctx->launches++;
            }
        }
        if (bricks)
            bricks_place(ctx, variant, d_blocks, hb, b, b + 1, nbricks, bins, pos, tv, g, grid, s);
        if (d.np)
        {
            launch_densities(W + d.p_off, d.np, p->mass, 1.0 / scale, rho32 + d.p_off, rho64 + d.p_off,
                             ctx->d_status, s);
            ctx->launches++;
        }
        if (bricks)
            bricks_raster(ctx, p->mode, variant, d_blocks, hb, b, b + 1, nbricks, bins, pos, tv, rho32, rho64, g,
                          grid, nullptr, s);
        else if (d.nt)
        {
            // the block's FP64 fix-up list: its own segment of the list buffer
            launch_raster(p->mode, variant, d_blocks, nb, d.nt, pos, tv, rho32, rho64, g, kTau, grid, nullptr,
                          fix + d.t_off, fixn + k, ctx->d_status, s, nullptr, nullptr, d.t_off, false,
                          fixn + nb + k);
            ctx->launches++;
            if (mixed)
            {
                launch_raster_fix(d_blocks, nb, d.nt, pos, tv, rho32, rho64, g, grid, nullptr, fix + d.t_off,
                                  fixn + k, ctx->d_status, s);
                ctx->launches++;
            }
        }
        CK(cudaEventRecord(ctx->pipe_ev[nb + k], s));
        span(ctx, "compute", ec0, smark(ctx, s));
        if (tiles && host_grid)
        {
            CK(cudaStreamWaitEvent(ctx->d2h, ctx->pipe_ev[nb + k], 0));
            cudaMemcpy3DParms prm;
            std::memset(&prm, 0, sizeof(prm));
            const int nx = p->glo_num_idx[0], ny = p->glo_num_idx[1];
            prm.srcPtr = make_cudaPitchedPtr(grid, sizeof(float) * nx, nx, ny);
            prm.dstPtr = make_cudaPitchedPtr(host_grid, sizeof(float) * nx, nx, ny);
            prm.srcPos = make_cudaPos(sizeof(float) * d.gmin_idx[0], d.gmin_idx[1], d.gmin_idx[2]);
            prm.dstPos = prm.srcPos;
            prm.extent = make_cudaExtent(sizeof(float) * (d.gmax_idx[0] - d.gmin_idx[0] + 1),
                                         d.gmax_idx[1] - d.gmin_idx[1] + 1, d.gmax_idx[2] - d.gmin_idx[2] + 1);
            prm.kind = cudaMemcpyDeviceToHost;
            const int e0 = smark(ctx, ctx->d2h);
            if (direct_out)
            {
                const int bx = d.gmax_idx[0] - d.gmin_idx[0] + 1, by = d.gmax_idx[1] - d.gmin_idx[1] + 1,
                          bz = d.gmax_idx[2] - d.gmin_idx[2] + 1;
                const long long rows = (long long)by * bz;
                if (rows > 0 && bx > 0)
                {
                    k_store_box<<<(unsigned)std::min(rows, (long long)hostio_ctas()), 256, 0, ctx->d2h>>>(
                        grid, host_grid, nx, ny, d.gmin_idx[0], d.gmin_idx[1], d.gmin_idx[2], bx, by, bz);
                    ctx->launches++;
                }
            }
            else
                CK(cudaMemcpy3DAsync(&prm, ctx->d2h));
            span(ctx, "download", e0, smark(ctx, ctx->d2h));
        }
        for (int l = 0; l < L && !tiles; ++l)
            if (slab_ready[l] == k && host_grid)
            {
                for (int kk = std::max(0, k - 1); kk <= k; ++kk)   // this block and the one on the other stream
                    CK(cudaStreamWaitEvent(ctx->d2h, ctx->pipe_ev[nb + kk], 0));
                const size_t off = (size_t)slab_lo[l] * area, n = (size_t)(slab_hi[l] - slab_lo[l] + 1) * area;
                if (direct_out)
                {
                    k_store_run<<<hostio_ctas(), 256, 0, ctx->d2h>>>(grid + off, host_grid + off, n);
                    ctx->launches++;
                }
                else
                    CK(cudaMemcpyAsync(host_grid + off, grid + off, sizeof(float) * n, cudaMemcpyDeviceToHost,
                                       ctx->d2h));
            }
    }
    // the second compute stream's last block, before the statistics
    for (int k = nb - 1; k >= 0; --k)
        if (k & 1)
        {
            CK(cudaStreamWaitEvent(s, ctx->pipe_ev[nb + k], 0));
            break;
        }
    mark(ctx, "blocks_done");
    if (host_grid)
    {
        // the last download, on the context's stream's timeline
        CK(cudaEventRecord(ctx->pipe_ev[2 * nb], ctx->d2h));
        CK(cudaStreamWaitEvent(s, ctx->pipe_ev[2 * nb], 0));
        mark(ctx, "downloads_done");
    }
    if (info)
    {
        CK(cudaMemsetAsync(ctx->d_max, 0, sizeof(float), s));
        launch_grid_max(grid, G, ctx->d_max, s);
        ctx->launches++;
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(Status), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(ctx->d2h));
    CK(cudaStreamSynchronize(s));
    const Status& st = *ctx->h_status;
    if (st.code)
        return set_err(ctx, (tessgpu_status)st.code, "DTFE failed at item " + std::to_string(st.detail));
    if (info)
    {
        float mx = 0.0f;
        CK(cudaMemcpy(&mx, ctx->d_max, sizeof(float), cudaMemcpyDeviceToHost));
        std::memset(info, 0, sizeof(*info));
        for (int i = 0; i < 3; ++i)
        {
            info->data_mins[i] = dmin[i]; info->data_maxs[i] = dmax[i];
            info->grid_phys_mins[i] = gmin[i]; info->grid_phys_maxs[i] = gmax[i]; info->grid_step_size[i] = step[i];
        }
        info->max_dense = mx;
        info->grid_pts_assigned = (long long)st.assigned;
        info->fp64_tets = (long long)st.fp64_tets;
        info->exact_tests = (long long)st.exact_tests;
        info->rows_visited = (long long)st.rows;
        info->points_tested = (long long)st.candidates;
        info->raster_variant = variant;
        for (int v = 0; v < 8; ++v)
            info->raster_variant_ms[v] = ctx->tune_ms[p->mode][v];
        info->grid_layers = 0;
        info->grid_floats = G;
        if (bricks)
        {
            unsigned long long pairs = 0;
            CK(cudaMemcpy(&pairs, bins.pair_cursor, sizeof(pairs), cudaMemcpyDeviceToHost));
            info->brick_pairs = (long long)pairs;
        }
    }
    return TESSGPU_OK;
}

extern "C" tessgpu_status tessgpu_dense(tessgpu_ctx* ctx, int nblocks, const tessgpu_block* blocks,
                                        const tessgpu_dense_params* p, float* global_grid, float** block_density,
                                        tessgpu_dense_info* info)
{
    if (!ctx || nblocks <= 0 || !blocks || !valid_params(p))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad dense arguments");
    ctx->last_grid = nullptr;
    ctx->last_grid_floats = 0;
    if (p->alg == TESSGPU_DENSE_DTFE && !p->project && !block_density && ctx->raster_variant[p->mode] >= 0)
    {
        const char* oenv = getenv("TESSGPU_RASTER_ORDER");
        const char* penv = getenv("TESSGPU_PIPELINE");
        if (!(oenv && atoi(oenv) == 1) && !(penv && *penv && atoi(penv) == 0))
        {
            float* d_grid = nullptr;
            tessgpu_status s = dense_dtfe_pipelined(ctx, nblocks, blocks, p, ctx->raster_variant[p->mode],
                                                    global_grid, info, &d_grid);
            if (s == TESSGPU_ERR_CAPACITY && !ctx->in_retry)
            {
                // the brick pair list was too small: size it for this call and run again
                grow_pairs(ctx);
                ctx->in_retry = true;
                s = dense_dtfe_pipelined(ctx, nblocks, blocks, p, ctx->raster_variant[p->mode], global_grid, info,
                                         &d_grid);
                ctx->in_retry = false;
            }
            if (s == TESSGPU_OK)
            {
                ctx->last_grid = d_grid;
                ctx->last_grid_floats = (long long)p->glo_num_idx[0] * p->glo_num_idx[1] * p->glo_num_idx[2];
            }
            return s;
        }
    }
    tessgpu_batch* bt = nullptr;
    tessgpu_status s = batch_build(ctx, nblocks, blocks, false, true, &bt);
    if (s != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
    const long long area = (long long)p->glo_num_idx[0] * p->glo_num_idx[1];
    int L = 0;
    const long long Gout = tessgpu_dense_grid_floats(nblocks, blocks, p, &L);
    cudaError_t e;
    float* d_grid = (float*)pool_get(ctx, SLOT_GRID, sizeof(float) * Gout, &e);
    if ((s = cuda_check(ctx, e, "cudaMalloc")) != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
    s = tessgpu_batch_dense(ctx, bt, p, d_grid, info);
    // the global grid WriteGrid writes: 3-D, or the layers summed (ProjectGrid)
    const float* d_global = d_grid;
    long long Gglobal = Gout;
    if (s == TESSGPU_OK && p->project)
    {
        float* d_proj = (float*)pool_get(ctx, SLOT_PROJ, sizeof(float) * area, &e);
        if ((s = cuda_check(ctx, e, "cudaMalloc")) == TESSGPU_OK)
            s = tessgpu_project_grid(ctx, d_grid, L, area, d_proj);
        d_global = d_proj;
        Gglobal = area;
    }
    if (s == TESSGPU_OK && global_grid)
        s = cuda_check(ctx, cudaMemcpyAsync(global_grid, d_global, sizeof(float) * Gglobal, cudaMemcpyDeviceToHost,
                                            ctx->stream), "cudaMemcpy");
    std::vector<int> zl;
    if (s == TESSGPU_OK && block_density && p->project)
    {
        std::vector<int> zmin(nblocks);
        for (int i = 0; i < nblocks; ++i)
        {
            int out9[9];
            tessgpu_block_grid_points(nblocks, blocks, i, p, out9);
            zmin[i] = out9[2];
        }
        z_layers(zmin, p->glo_num_idx[2], zl);
    }
    if (s == TESSGPU_OK && block_density)
    {
        for (int i = 0; i < nblocks && s == TESSGPU_OK; ++i)
        {
            if (!block_density[i]) continue;
            int out9[9];
            long long n = tessgpu_block_grid_points(nblocks, blocks, i, p, out9);
            if (n <= 0) continue;
            bool inside = true;
            for (int k = 0; k < 3; ++k)
                if (out9[k] < 0 || out9[3 + k] >= p->glo_num_idx[k]) inside = false;
            if (!inside)
            {
                s = set_err(ctx, TESSGPU_ERR_UNSUPPORTED,
                            "block " + std::to_string(i) + "'s grid box reaches outside the grid");
                break;
            }
            int* d_box = (int*)pool_get(ctx, SLOT_COUNT, sizeof(int) * 9, &e);
            float* d_tmp = (float*)pool_get(ctx, SLOT_OUT2, sizeof(float) * n, &e);
            if ((s = cuda_check(ctx, e, "cudaMalloc")) != TESSGPU_OK) break;
            int box[6] = { out9[0], out9[1], out9[2], out9[6], out9[7], out9[8] };
            if (p->project)
            {
                // the block's 2-D array is its layer's rectangle
                box[2] = layer_of(zl, out9[2]);
                box[5] = 1;
            }
            CK(cudaMemcpyAsync(d_box, box, sizeof(box), cudaMemcpyHostToDevice, ctx->stream));
            k_extract_box<<<grid_small(n), 256, 0, ctx->stream>>>(d_grid, p->glo_num_idx[0], p->glo_num_idx[1], d_box,
                                                                  d_box + 3, d_tmp);
            ctx->launches++;
            s = cuda_check(ctx, cudaMemcpyAsync(block_density[i], d_tmp, sizeof(float) * n, cudaMemcpyDeviceToHost,
                                                ctx->stream), "cudaMemcpy");
            if (s == TESSGPU_OK)
                s = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        }
    }
    if (s == TESSGPU_OK)
        s = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (s == TESSGPU_OK)
    {
        ctx->last_grid = d_global;
        ctx->last_grid_floats = Gglobal;
    }
    tessgpu_batch_free(bt);
    return s;
}

// ---------------------------------------------------------------------------
// ProjectGrid and WriteGrid
// ---------------------------------------------------------------------------
extern "C" tessgpu_status tessgpu_project_grid(tessgpu_ctx* ctx, const float* d_layers, int num_layers,
                                               long long layer_floats, float* d_out)
{
    if (!ctx || num_layers < 1 || layer_floats < 0 || (layer_floats && (!d_layers || !d_out)))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    if (!layer_floats) return TESSGPU_OK;
    CK(cudaSetDevice(ctx->device));
    launch_sum_layers(d_layers, num_layers, layer_floats, d_out, ctx->stream);
    ctx->launches++;
    mark(ctx, "project_grid");
    CK(cudaGetLastError());
    return TESSGPU_OK;
}

static const size_t kStageBytes = 32u << 20;   // one pinned staging chunk

extern "C" tessgpu_status tessgpu_write_grid(tessgpu_ctx* ctx, const float* d_grid, long long num_floats,
                                             const char* path)
{
    if (!ctx || !path || num_floats < 0 || (num_floats && !d_grid))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    for (int i = 0; i < 2; ++i)
    {
        if (!ctx->h_stage[i]) CK(cudaMallocHost(&ctx->h_stage[i], kStageBytes));
        if (!ctx->stage_ev[i]) CK(cudaEventCreateWithFlags(&ctx->stage_ev[i], cudaEventDisableTiming));
    }
    FILE* f = std::fopen(path, "wb");   // truncates, as WriteGrid's MPI_File_set_size(fd, 0)
    if (!f) return set_err(ctx, TESSGPU_ERR_IO, std::string("cannot open ") + path);
    const size_t total = sizeof(float) * (size_t)num_floats;
    const size_t nchunks = (total + kStageBytes - 1) / kStageBytes;
    auto issue = [&](size_t c) -> cudaError_t {
        const size_t off = c * kStageBytes, n = std::min(kStageBytes, total - off);
        cudaError_t e = cudaMemcpyAsync(ctx->h_stage[c & 1], (const char*)d_grid + off, n, cudaMemcpyDeviceToHost,
                                        ctx->stream);
        return e != cudaSuccess ? e : cudaEventRecord(ctx->stage_ev[c & 1], ctx->stream);
    };
    tessgpu_status s = TESSGPU_OK;
    if (nchunks) s = cuda_check(ctx, issue(0), "cudaMemcpyAsync");
    for (size_t c = 0; c < nchunks && s == TESSGPU_OK; ++c)
    {
        // the next chunk's copy runs while this one is written
        if (c + 1 < nchunks && (s = cuda_check(ctx, issue(c + 1), "cudaMemcpyAsync")) != TESSGPU_OK) break;
        if ((s = cuda_check(ctx, cudaEventSynchronize(ctx->stage_ev[c & 1]), "cudaEventSynchronize")) != TESSGPU_OK)
            break;
        const size_t n = std::min(kStageBytes, total - c * kStageBytes);
        if (std::fwrite(ctx->h_stage[c & 1], 1, n, f) != n)
            s = set_err(ctx, TESSGPU_ERR_IO, std::string("short write to ") + path);
    }
    if (s != TESSGPU_OK) cudaStreamSynchronize(ctx->stream);   // no copy may land in a reused buffer later
    if (std::fclose(f) != 0 && s == TESSGPU_OK)
        s = set_err(ctx, TESSGPU_ERR_IO, std::string("cannot close ") + path);
    return s;
}

extern "C" tessgpu_status tessgpu_write_last_grid(tessgpu_ctx* ctx, const char* path)
{
    if (!ctx) return TESSGPU_ERR_INVALID;
    if (!ctx->last_grid) return set_err(ctx, TESSGPU_ERR_INVALID, "no tessgpu_dense call has finished on this context");
    return tessgpu_write_grid(ctx, ctx->last_grid, ctx->last_grid_floats, path);
}

// ---------------------------------------------------------------------------
// incomplete_cells
// ---------------------------------------------------------------------------
extern "C" tessgpu_status tessgpu_batch_incomplete_cells(tessgpu_ctx* ctx, tessgpu_batch* bt, const int* link_offsets,
                                                         const tessgpu_link* links, const int* last_neighbor,
                                                         unsigned long long* d_send_mask, long long* enqueued)
{
    if (!ctx || !bt || !link_offsets || (!links && link_offsets[bt->nb]) || (bt->C && !d_send_mask))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    const int nb = bt->nb;
    if (link_offsets[0] != 0) return set_err(ctx, TESSGPU_ERR_INVALID, "link_offsets[0] must be 0");
    for (int b = 0; b < nb; ++b)
    {
        const int n = link_offsets[b + 1] - link_offsets[b];
        const int f = last_neighbor ? last_neighbor[b] : 0;
        if (n < 0 || n > 64 || f < 0)
            return set_err(ctx, n > 64 ? TESSGPU_ERR_UNSUPPORTED : TESSGPU_ERR_INVALID,
                           "block " + std::to_string(b) + ": links must number 0..64 and last_neighbor be >= 0");
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int nl = link_offsets[nb];
    // wrap_bounds: a link across a periodic boundary sees its box shifted by
    // the wrap direction times the data extent (DBlock::data_bounds)
    std::vector<float> l6(6 * (size_t)std::max(nl, 1), 0.0f);
    std::vector<int> meta(2 * nb + 1);
    std::vector<unsigned long long> fill(nb, 0ull);
    for (int b = 0; b < nb; ++b)
    {
        const tessgpu_block& B = bt->blocks[b];
        for (int i = link_offsets[b]; i < link_offsets[b + 1]; ++i)
            for (int d = 0; d < 3; ++d)
            {
                const float ext = B.data_max[d] - B.data_min[d];
                l6[6 * i + d] = links[i].bounds_min[d] + links[i].wrap[d] * ext;
                l6[6 * i + 3 + d] = links[i].bounds_max[d] + links[i].wrap[d] * ext;
            }
        const int f = last_neighbor ? last_neighbor[b] : 0;
        for (int i = f; i < link_offsets[b + 1] - link_offsets[b]; ++i)
            fill[b] |= 1ull << i;
    }
    for (int b = 0; b <= nb; ++b) meta[b] = link_offsets[b];
    for (int b = 0; b < nb; ++b) meta[nb + 1 + b] = last_neighbor ? last_neighbor[b] : 0;
    cudaError_t e;
    float* d_l6 = (float*)pool_get(ctx, SLOT_LINKS, sizeof(float) * l6.size(), &e);
    CK(e);
    int* d_meta = (int*)pool_get(ctx, SLOT_LINKOFF, sizeof(int) * meta.size(), &e);
    CK(e);
    unsigned long long* d_aux =
        (unsigned long long*)pool_get(ctx, SLOT_SENDS, sizeof(unsigned long long) * 2 * nb, &e);
    CK(e);
    CK(cudaMemcpyAsync(d_l6, l6.data(), sizeof(float) * l6.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_meta, meta.data(), sizeof(int) * meta.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(d_aux, fill.data(), sizeof(unsigned long long) * nb, cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(d_aux + nb, 0, sizeof(unsigned long long) * nb, s));
    if (bt->C) CK(cudaMemsetAsync(d_send_mask, 0, sizeof(unsigned long long) * bt->C, s));
    ctx->nmarks = 0;
    ctx->nsev = 0;
    ctx->spans.clear();
    mark(ctx, "start");
    launch_incomplete_cells(bt->d_blocks, bt->d_c_off, nb, (int)bt->T, (int)bt->C, bt->pos, bt->tv, bt->tn, d_l6,
                            d_meta, d_meta + nb + 1, d_aux, d_send_mask, d_aux + nb, s);
    ctx->launches += (bt->C ? 2 : 0) + (bt->T ? 1 : 0);
    mark(ctx, "incomplete_cells");
    CK(cudaGetLastError());
    if (enqueued)
    {
        std::vector<unsigned long long> cnt(nb);
        CK(cudaMemcpyAsync(cnt.data(), d_aux + nb, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        for (int b = 0; b < nb; ++b) enqueued[b] = (long long)cnt[b];
    }
    return TESSGPU_OK;
}

extern "C" tessgpu_status tessgpu_incomplete_cells(tessgpu_ctx* ctx, const tessgpu_block* block, int num_links,
                                                   const tessgpu_link* links, int last_neighbor,
                                                   unsigned long long* send_mask, long long* enqueued)
{
    if (!ctx || !block || num_links < 0 || (num_links && !links) || last_neighbor < 0 ||
        (block->num_orig_particles && !send_mask))
        return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    tessgpu_batch* bt = nullptr;
    tessgpu_status s = batch_build(ctx, 1, block, false, true, &bt);
    if (s != TESSGPU_OK) { tessgpu_batch_free(bt); return s; }
    cudaError_t e;
    unsigned long long* d_mask =
        (unsigned long long*)pool_get(ctx, SLOT_MASK, sizeof(unsigned long long) * std::max<long long>(bt->C, 1), &e);
    if ((s = cuda_check(ctx, e, "cudaMalloc")) == TESSGPU_OK)
    {
        const int off[2] = { 0, num_links };
        long long enq = 0;
        s = tessgpu_batch_incomplete_cells(ctx, bt, off, links, &last_neighbor, d_mask, &enq);
        if (s == TESSGPU_OK && bt->C)
            s = cuda_check(ctx, cudaMemcpy(send_mask, d_mask, sizeof(unsigned long long) * bt->C,
                                           cudaMemcpyDeviceToHost), "cudaMemcpy");
        if (s == TESSGPU_OK && enqueued) *enqueued = enq;
    }
    tessgpu_batch_free(bt);
    return s;
}

// ---------------------------------------------------------------------------
// reorder_neighbors
// ---------------------------------------------------------------------------
extern "C" tessgpu_status tessgpu_reorder_neighbors_device(tessgpu_ctx* ctx, int* d_tets, int num_tets)
{
    if (!ctx || num_tets < 0 || (num_tets && !d_tets)) return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    if (!num_tets) return TESSGPU_OK;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(Status), ctx->stream));
    ctx->nmarks = 0;
    ctx->nsev = 0;
    ctx->spans.clear();
    mark(ctx, "start");
    launch_reorder_neighbors(d_tets, num_tets, ctx->d_status, ctx->stream);
    mark(ctx, "reorder_neighbors");
    ctx->launches++;
    return finish_status(ctx);
}

extern "C" tessgpu_status tessgpu_reorder_neighbors(tessgpu_ctx* ctx, int* tets, int num_tets)
{
    if (!ctx || num_tets < 0 || (num_tets && !tets)) return set_err(ctx, TESSGPU_ERR_INVALID, "bad arguments");
    if (!num_tets) return TESSGPU_OK;
    CK(cudaSetDevice(ctx->device));
    cudaError_t e;
    int* d = (int*)pool_get(ctx, SLOT_STAGE, sizeof(int) * 8 * (size_t)num_tets, &e);
    CK(e);
    CK(cudaMemcpyAsync(d, tets, sizeof(int) * 8 * (size_t)num_tets, cudaMemcpyHostToDevice, ctx->stream));
    tessgpu_status s = tessgpu_reorder_neighbors_device(ctx, d, num_tets);
    if (s != TESSGPU_OK) return s;
    CK(cudaMemcpy(tets, d, sizeof(int) * 8 * (size_t)num_tets, cudaMemcpyDeviceToHost));
    return TESSGPU_OK;
}
