"""GPU parity against the reference's golden vectors and the CPU oracle.

Everything here calls the C ABI of libtess2_gb300.so (through
tess2_gb300.api).  Bars:
  * circumcenters, complete flags, Voronoi volumes, per-cell DENSE_TESS
    grid-point counts: bit-identical to the reference;
  * DENSE_TESS / DENSE_CIC grids: within 1e-5 relative L2 of the reference
    (atomic float adds change the order of the rare multi-hit sums);
  * DTFE: point-to-tet owners bit-identical to the FP64 oracle; grid values
    within 1e-6 relative L2 of it (mixed) and 1e-12 (FP64 mode).
"""
import numpy as np
import pytest

from conftest import load_blocks, load_single, rel_l2, single_block

pytestmark = pytest.mark.gpu

SINGLE = ["c1_uniform4096_seed1", "mix2048_seed7"]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", SINGLE)
def test_circumcenters_bitexact(gpu_ctx, name):
    d = load_single(name)
    cc = gpu_ctx.fill_circumcenters(d["tets"], d["particles"])
    assert np.array_equal(bits(cc), bits(d["circumcenters"]))


@pytest.mark.parametrize("name", SINGLE)
def test_vert_to_tet_bitexact(gpu_ctx, name):
    d = load_single(name)
    v = gpu_ctx.fill_vert_to_tet(len(d["particles"]), d["tets"])
    assert np.array_equal(v, d["vert_to_tet"])


@pytest.mark.parametrize("name", SINGLE)
def test_complete_bitexact(gpu_ctx, name):
    d = load_single(name)
    c = gpu_ctx.complete(d["tets"], d["vert_to_tet"], d["particles"])
    assert np.array_equal(c, d["complete"])


@pytest.mark.parametrize("name", SINGLE)
def test_volumes_bitexact(gpu_ctx, name):
    d = load_single(name)
    v = gpu_ctx.volume(d["vert_to_tet"], d["tets"], d["particles"])
    assert np.array_equal(bits(v), bits(d["volumes"]))


@pytest.mark.parametrize("name", SINGLE)
def test_face_areas_bitexact(gpu_ctx, oracle, name):
    """tessgpu_volumes' areas output: each cell's face areas (volume()'s fan
    sums, src/volume.cpp:25-47) added in face order, against the oracle."""
    d = load_single(name)
    v, a = gpu_ctx.volume(d["vert_to_tet"], d["tets"], d["particles"], areas=True)
    rv, ra = oracle.volume_areas(d["particles"], d["tets"], d["vert_to_tet"])
    assert np.array_equal(bits(v), bits(rv))
    assert np.array_equal(bits(a), bits(ra))
    assert np.all(a[v > 0] > 0)


@pytest.mark.parametrize("name", SINGLE)
def test_volumes_f64_vs_oracle(gpu_ctx, oracle, name):
    d = load_single(name)
    v = gpu_ctx.volume_f64(d["vert_to_tet"], d["tets"], d["particles"])
    ref = oracle.volumes_f64(d["particles"], d["tets"], d["vert_to_tet"])
    fin = ref > 0
    assert np.array_equal(v < 0, ref < 0)
    assert np.max(np.abs(v[fin] - ref[fin]) / ref[fin]) < 1e-12
    # the FP32 reference volumes against FP64: the error the reference carries
    v32 = d["volumes"].astype(np.float64)
    assert rel_l2(v32[fin], ref[fin]) < 1e-4


@pytest.mark.parametrize("name", SINGLE)
@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
def test_dense_single_block(gpu_ctx, name, alg, tag):
    from tess2_gb300.api import Batch
    d = load_single(name)
    gni = [int(x) for x in d["glo_num_idx"]]
    r = gpu_ctx.dense(alg, single_block(d), gni)
    ref = d[f"{tag}_grid"]
    assert rel_l2(r["grid"], ref) < 1e-5
    # points hit by one cell match bit for bit; points hit by several differ
    # only by the order of their float additions (a few ulps)
    assert np.allclose(r["grid"], ref, rtol=4e-6, atol=0.0)
    st = d[f"{tag}_stats"]
    assert r["info"]["check_mass"] == st[2]
    assert abs(r["info"]["tot_mass"] - st[1]) <= 1e-6 * st[1]
    assert abs(r["info"]["max_dense"] - st[0]) <= 1e-5 * st[0]


@pytest.mark.parametrize("name", SINGLE)
def test_dense_tess_cell_counts_bitexact(gpu_ctx, name):
    import torch
    from tess2_gb300.api import DENSE_TESS
    d = load_single(name)
    gni = [int(x) for x in d["glo_num_idx"]]
    b = gpu_ctx.upload(single_block(d))
    b.keep_debug(True)
    grid = torch.zeros(gni[2], gni[1], gni[0], dtype=torch.float32, device="cuda")
    b.dense(DENSE_TESS, gni, grid.data_ptr())
    counts, _, _ = b.debug_outputs(cells=len(d["particles"]))
    assert np.array_equal(counts, d["tess_cell_counts"])
    assert rel_l2(grid.cpu().numpy(), d["tess_grid"]) < 1e-5


@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
def test_dense_multiblock(gpu_ctx, alg, tag):
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    r = gpu_ctx.dense(alg, blocks, gni, block_arrays=True)
    ref = d[f"{tag}_grid"]
    assert rel_l2(r["grid"], ref) < 1e-5
    st = d[f"{tag}_stats"]
    assert r["info"]["check_mass"] == st[2]
    assert abs(r["info"]["tot_mass"] - st[1]) <= 1e-6 * st[1]
    # per-block arrays are the block's BlockGridParams box of the global grid
    from tess2_gb300.api import lib, make_blocks, make_params
    import ctypes
    arr, keep = make_blocks(blocks)
    p = make_params(alg, gni)
    for i, ba in enumerate(r["blocks"]):
        o9 = (ctypes.c_int * 9)()
        lib().tessgpu_block_grid_points(len(blocks), arr, i, ctypes.byref(p), o9)
        mn, num = o9[0:3], o9[6:9]
        box = r["grid"][mn[2]:mn[2] + num[2], mn[1]:mn[1] + num[1], mn[0]:mn[0] + num[0]]
        assert np.array_equal(ba.reshape(num[2], num[1], num[0]), box)


def _dtfe_case(oracle, gpu_ctx, blocks, gni, mode):
    import torch
    from tess2_gb300.api import DENSE_DTFE
    ref = oracle.dtfe(blocks, gni)
    b = gpu_ctx.upload(blocks)
    b.keep_debug(True)
    grid = torch.zeros(gni[2], gni[1], gni[0], dtype=torch.float32, device="cuda")
    info = b.dense(DENSE_DTFE, gni, grid.data_ptr(), mode=mode)
    _, owner, _ = b.debug_outputs(grid_points=grid.numel())
    return ref, grid.cpu().numpy(), owner.reshape(grid.shape), info


@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 1e-12)])
@pytest.mark.parametrize("name", SINGLE)
def test_dtfe_single_block(gpu_ctx, oracle, name, mode, tol):
    d = load_single(name)
    gni = [int(x) for x in d["glo_num_idx"]]
    ref, grid, owner, info = _dtfe_case(oracle, gpu_ctx, single_block(d), gni, mode)
    assert np.array_equal(owner, ref["owner"])
    assert info["grid_pts_assigned"] == ref["assigned"]
    assert rel_l2(grid, ref["grid"]) < tol


@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 1e-12)])
def test_dtfe_multiblock(gpu_ctx, oracle, mode, tol):
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    ref, grid, owner, info = _dtfe_case(oracle, gpu_ctx, blocks, gni, mode)
    assert np.array_equal(owner, ref["owner"])
    assert rel_l2(grid, ref["grid"]) < tol


def test_dtfe_sharded_blocks_sum_to_whole(gpu_ctx):
    """Blocks split over two shares (as ranks would hold them), each run with
    the whole decomposition's data bounds: the grids add up to the one-batch
    grid bit for bit, since every grid point has one owner."""
    import torch
    from tess2_gb300 import host
    from tess2_gb300.api import DENSE_DTFE
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    whole = torch.zeros(gni[2], gni[1], gni[0], dtype=torch.float32, device="cuda")
    gpu_ctx.upload(blocks).dense(DENSE_DTFE, gni, whole.data_ptr())
    bounds = host.data_bounds_of(blocks)
    total = torch.zeros_like(whole)
    for r in range(2):
        part = torch.zeros_like(whole)
        gpu_ctx.upload(host.shard_blocks(blocks, r, 2)).dense(DENSE_DTFE, gni, part.data_ptr(), data_bounds=bounds)
        total += part
    assert torch.equal(total, whole)


@pytest.mark.parametrize("name", SINGLE)
def test_reorder_neighbors_bitexact(gpu_ctx, oracle, name):
    from test_oracle_golden import shuffled_neighbors
    d = load_single(name)
    shuf = shuffled_neighbors(d["tets"], 2)
    got = gpu_ctx.reorder_neighbors(shuf)
    assert np.array_equal(got, oracle.reorder_neighbors(shuf))
    assert np.array_equal(got, d["tets"])


# ---------------------------------------------------------------------------
# dense(project) + ProjectGrid + WriteGrid
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", ["c1_uniform4096_seed1", "mix2048_seed7", "blocks8_mix8192_seed3"])
@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
def test_dense_projected_vs_reference_writegrid(gpu_ctx, tmp_path, name, alg, tag):
    """Projected densities against the file the reference's WriteGrid wrote
    (after its ProjectGrid) and each block's array as dense() left it.  Column
    sums gather a deposit per z, so the atomic adds' order shows at the
    level of a few ulps of the sum: rtol 2e-5 (one grid point's share of a
    column is >1e-3 of it)."""
    from conftest import load_case_blocks, load_writegrid
    d, blocks, gni = load_case_blocks(name)
    w = load_writegrid()
    r = gpu_ctx.dense(alg, blocks, gni, project=True, block_arrays=True)
    f = w[f"{name}_{tag}_proj_file"].reshape(gni[1], gni[0])
    assert r["grid"].shape == f.shape
    np.testing.assert_allclose(r["grid"], f, rtol=2e-5, atol=0)
    assert np.array_equal(r["grid"] == 0, f == 0)
    got = np.concatenate(r["blocks"])
    ref = w[f"{name}_{tag}_proj_blocks"]
    assert got.size == ref.size
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=0)
    st = w[f"{name}_{tag}_proj_stats"]
    assert r["info"]["check_mass"] == st[2]
    assert np.isclose(r["info"]["tot_mass"], st[1], rtol=1e-12)
    assert np.isclose(r["info"]["max_dense"], st[0], rtol=2e-5)
    # WriteGrid after dense(): the file is the projected grid, byte for byte
    out = tmp_path / "proj.raw"
    gpu_ctx.write_last_grid(str(out))
    assert np.array_equal(np.fromfile(out, np.float32), r["grid"].ravel())


def test_write_grid_exact_bytes(gpu_ctx, tmp_path):
    """The writer's file is the device buffer byte for byte, over several
    staging chunks and a ragged last chunk; a zero-length write truncates."""
    import torch
    from tess2_gb300.api import TessGpuError
    n = 3 * (8 << 20) + 12345          # 3 x 32 MiB chunks of floats plus a tail
    g = torch.randn(n, device="cuda:0")
    torch.cuda.synchronize()
    out = tmp_path / "g.raw"
    out.write_bytes(b"x" * (4 * n + 100))   # longer old contents must go
    gpu_ctx.write_grid(g.data_ptr(), n, str(out))
    got = np.fromfile(out, np.float32)
    assert got.size == n and np.array_equal(got, g.cpu().numpy())
    gpu_ctx.write_grid(g.data_ptr(), 0, str(out))
    assert out.stat().st_size == 0
    with pytest.raises(TessGpuError) as e:
        gpu_ctx.write_grid(g.data_ptr(), 16, str(tmp_path / "no_such_dir" / "g.raw"))
    assert e.value.code == 9


def test_write_last_grid_3d(gpu_ctx, tmp_path):
    d = load_single("mix2048_seed7")
    gni = [int(x) for x in d["glo_num_idx"]]
    r = gpu_ctx.dense(0, single_block(d), gni)
    out = tmp_path / "g3.raw"
    gpu_ctx.write_last_grid(str(out))
    assert np.array_equal(np.fromfile(out, np.float32), r["grid"].ravel())


def test_project_grid_sums_layers_in_order(gpu_ctx, oracle):
    import torch
    gen = torch.Generator().manual_seed(5)
    lay = (torch.rand((3, 41, 37), generator=gen) * 1e3).to(torch.float32)
    d_l = lay.to("cuda:0")
    d_o = torch.empty((41, 37), device="cuda:0")
    gpu_ctx.project_grid(d_l.data_ptr(), 3, 41 * 37, d_o.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d_o.cpu().numpy(), oracle.sum_layers(lay.numpy()))


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 2, 2)])
def test_dtfe_projected(gpu_ctx, oracle, dims):
    """DTFE projected: each layer is the column integral (sum of rho * dz in
    ascending z) of the 3-D DTFE grid over the layer's z range -- bit for bit
    the projection of the GPU's own 3-D grid, and within 1e-6 relative L2 of
    the projection of the FP64 oracle's grid."""
    import ctypes
    import torch
    from tess2_gb300 import host
    from tess2_gb300.api import DENSE_DTFE, grid_floats, lib, make_blocks, make_params
    pts = host.mixture_particles(6000, 11, n_clumps=8, sigma=0.05)
    blocks = host.tessellate(host.decompose(pts, dims, 0.15), processes=1)
    gni = [36, 30, 33]
    nfl, L = grid_floats(blocks, DENSE_DTFE, gni, project=True)
    assert L == dims[2] and nfl == L * gni[0] * gni[1]
    batch = gpu_ctx.upload(blocks)
    g3 = torch.zeros(int(np.prod(gni)), device="cuda:0")
    info3 = batch.dense(DENSE_DTFE, gni, g3.data_ptr())
    gp = torch.zeros(nfl, device="cuda:0")
    info = batch.dense(DENSE_DTFE, gni, gp.data_ptr(), project=True)
    torch.cuda.synchronize()
    assert info["grid_layers"] == L and info["grid_floats"] == nfl
    grid3 = g3.cpu().numpy().reshape(gni[2], gni[1], gni[0])
    layers = gp.cpu().numpy().reshape(L, gni[1], gni[0])
    zmin = []
    arr, keep = make_blocks(blocks)
    prm = make_params(DENSE_DTFE, gni, project=True)
    for i in range(len(blocks)):
        o9 = np.zeros(9, np.int32)
        lib().tessgpu_block_grid_points(len(blocks), arr, i, ctypes.byref(prm), o9.ctypes.data)
        zmin.append(int(o9[2]))
    zl, nl = oracle.z_layers(zmin, gni[2])
    assert nl == L
    dz = info3["grid_step_size"][2]
    assert np.array_equal(layers, oracle.project_layers(grid3, zl, dz))
    ref = oracle.dtfe(blocks, gni, want_owner=False, want_rho=False)["grid"]
    assert rel_l2(layers, oracle.project_layers(ref, zl, dz)) < 1e-6
    # max over the layers, as dense() reports it before ProjectGrid
    assert np.isclose(info["max_dense"], layers.max(), rtol=0)


# ---------------------------------------------------------------------------
# incomplete_cells
# ---------------------------------------------------------------------------
def _links_of(blocks, bi):
    return np.array([np.concatenate([o["bounds_min"], o["bounds_max"]]) for k, o in enumerate(blocks) if k != bi],
                    np.float32)


def test_incomplete_cells_batch_bitexact(gpu_ctx, oracle):
    """Every block of the 2x2x2 golden decomposition, all links from 0: the
    send masks bit for bit, and the per-block counts."""
    import torch
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    batch = gpu_ctx.upload(blocks)
    C = sum(int(b["num_orig"]) for b in blocks)
    dm = torch.zeros(C, dtype=torch.int64, device="cuda:0")
    enq = batch.incomplete_cells([_links_of(blocks, i) for i in range(len(blocks))], dm.data_ptr())
    torch.cuda.synchronize()
    got = dm.cpu().numpy().view(np.uint64)
    off = 0
    for i, b in enumerate(blocks):
        m, n = oracle.incomplete_cells(b, _links_of(blocks, i))
        assert np.array_equal(got[off:off + b["num_orig"]], m), i
        assert enq[i] == n
        off += b["num_orig"]


@pytest.mark.parametrize("last", [0, 3])
def test_incomplete_cells_periodic_bitexact(gpu_ctx, oracle, last):
    from tess2_gb300 import host
    pts = host.mixture_particles(20000, 9, n_clumps=32, sigma=0.02)
    blocks = host.tessellate(host.decompose(pts, (3, 2, 2), 0.06), processes=1)
    b = blocks[4]
    l6 = _links_of(blocks, 4)
    w3 = np.zeros((len(l6), 3), np.int32)
    w3[::3, 0] = 1
    w3[1::4, 1] = -1
    m, n = gpu_ctx.incomplete_cells(b, l6, w3, last_neighbor=last)
    mo, no = oracle.incomplete_cells(b, l6, w3, last_neighbor=last)
    assert np.array_equal(m, mo) and n == no and n > 0


def test_incomplete_cells_without_tets_gpu(gpu_ctx, oracle):
    p = np.random.default_rng(1).random((4, 3), dtype=np.float32)
    b = dict(particles=p, tets=np.zeros((0, 8), np.int32), vert_to_tet=np.full(4, -1, np.int32), num_orig=3,
             bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
             data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))
    l6 = np.tile(np.array([0, 0, 0, 1, 1, 1], np.float32), (5, 1))
    m, n = gpu_ctx.incomplete_cells(b, l6, last_neighbor=2)
    assert list(m) == [0b11100] * 3 and n == 9


@pytest.mark.parametrize("dims", [(2, 2, 2), (1, 2, 3), "gap"])
def test_dtfe_host_pipeline_matches_batch(gpu_ctx, dims):
    """The host-buffer DTFE call (copies overlapped with the per-block
    kernels, each block's grid box -- or, when the boxes leave a gap, each
    z-slab -- copied back as it completes) against the device-resident batch
    path: the same grid bit for bit, and the same counts; TESSGPU_PIPELINE=0
    takes the unpipelined host path."""
    import os
    import torch
    from tess2_gb300 import host
    from tess2_gb300.api import DENSE_DTFE, MODE_FP64, MODE_MIXED
    pts = host.mixture_particles(30000, 21, n_clumps=16, sigma=0.02)
    if dims == "gap":
        blocks = host.tessellate(host.decompose(pts, (1, 1, 2), 0.08), processes=1)
        blocks[1]["bounds_min"] = np.array([0.0, 0.0, 0.6], np.float32)   # z in (0.5, 0.6): no block's box
    else:
        blocks = host.tessellate(host.decompose(pts, dims, 0.08), processes=1)
    gni = [48, 44, 52]
    for mode in (MODE_MIXED, MODE_FP64):
        batch = gpu_ctx.upload(blocks)
        g = torch.zeros(int(np.prod(gni)), device="cuda:0")
        ib = batch.dense(DENSE_DTFE, gni, g.data_ptr(), mode=mode)   # chooses the launch variant if not yet chosen
        torch.cuda.synchronize()
        ref = g.cpu().numpy().reshape(gni[2], gni[1], gni[0])
        batch.free()
        r1 = gpu_ctx.dense(DENSE_DTFE, blocks, gni, mode=mode)
        assert np.array_equal(r1["grid"], ref)
        for k in ("grid_pts_assigned", "fp64_tets", "exact_tests"):
            assert r1["info"][k] == ib[k], k
        assert r1["info"]["max_dense"] == ib["max_dense"]
        os.environ["TESSGPU_PIPELINE"] = "0"
        try:
            r0 = gpu_ctx.dense(DENSE_DTFE, blocks, gni, mode=mode)
        finally:
            del os.environ["TESSGPU_PIPELINE"]
        assert np.array_equal(r0["grid"], ref)
        os.environ["TESSGPU_PIPELINE_STREAMS"] = "1"   # every block's kernels on one stream
        try:
            r2 = gpu_ctx.dense(DENSE_DTFE, blocks, gni, mode=mode)
        finally:
            del os.environ["TESSGPU_PIPELINE_STREAMS"]
        assert np.array_equal(r2["grid"], ref)
        assert r2["info"]["fp64_tets"] == ib["fp64_tets"]
        # pinned host arrays go through the copy engines; pageable ones (above) are read and
        # written in place by the kernels where the device addresses pageable memory
        keep, pblocks = [], []
        for b in blocks:
            nb = dict(b)
            for k in ("particles", "tets"):
                a = np.ascontiguousarray(b[k])
                t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0]).dtype, pin_memory=True)
                t.numpy()[...] = a
                keep.append(t)
                nb[k] = t.numpy()
            pblocks.append(nb)
        out = torch.empty((gni[2], gni[1], gni[0]), dtype=torch.float32, pin_memory=True).numpy()
        gpu_ctx.dense(DENSE_DTFE, pblocks, gni, mode=mode, out=out)
        assert np.array_equal(out, ref)


def test_dtfe_brick_order_same_grid(gpu_ctx):
    """TESSGPU_RASTER_ORDER=1 (tets rasterised brick by brick) writes the
    same grid bit for bit: every grid point has exactly one owner tet."""
    import os
    import torch
    from tess2_gb300.api import DENSE_DTFE
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [56, 60, 52]
    out = []
    for env in (None, "1"):
        if env:
            os.environ["TESSGPU_RASTER_ORDER"] = env
        try:
            batch = gpu_ctx.upload(blocks)
            g = torch.zeros(int(np.prod(gni)), device="cuda:0")
            info = batch.dense(DENSE_DTFE, gni, g.data_ptr())
            torch.cuda.synchronize()
            out.append((g.cpu().numpy(), info["grid_pts_assigned"]))
            batch.free()
        finally:
            os.environ.pop("TESSGPU_RASTER_ORDER", None)
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_dtfe_batch_overlap_same_grid(gpu_ctx):
    """The batch path with blocks on two streams (TESSGPU_BATCH_OVERLAP=1, once
    the launch variant is known) and by default (stages one after the other
    over all blocks): the same grid bit for bit and the same counts."""
    import os
    import torch
    from tess2_gb300.api import DENSE_DTFE, MODE_FP64, MODE_MIXED
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [50, 46, 54]
    for mode in (MODE_MIXED, MODE_FP64):
        out = []
        for env in ("1", None):
            if env:
                os.environ["TESSGPU_BATCH_OVERLAP"] = env
            try:
                batch = gpu_ctx.upload(blocks)
                g = torch.zeros(int(np.prod(gni)), device="cuda:0")
                batch.dense(DENSE_DTFE, gni, g.data_ptr(), mode=mode)     # chooses the variant if needed
                info = batch.dense(DENSE_DTFE, gni, g.data_ptr(), mode=mode)
                torch.cuda.synchronize()
                out.append((g.cpu().numpy(), info))
                batch.free()
            finally:
                os.environ.pop("TESSGPU_BATCH_OVERLAP", None)
        assert np.array_equal(out[0][0], out[1][0])
        for k in ("grid_pts_assigned", "fp64_tets", "exact_tests", "max_dense"):
            assert out[0][1][k] == out[1][1][k], k


# ---------------------------------------------------------------------------
# error statuses (the kernels check their indices and report; nothing faults)
# ---------------------------------------------------------------------------
def test_error_statuses(gpu_ctx):
    from tess2_gb300.api import DENSE_DTFE, TessGpuError
    d = load_single("mix2048_seed7")
    bad = d["tets"].copy()
    bad[7, 5] = bad.shape[0] + 3          # a neighbour index past the tets
    with pytest.raises(TessGpuError) as e:
        gpu_ctx.reorder_neighbors(bad)
    assert e.value.code == 7
    b = single_block(d)[0]
    l6 = np.tile(np.array([0, 0, 0, 1, 1, 1], np.float32), (65, 1))
    with pytest.raises(TessGpuError) as e:
        gpu_ctx.incomplete_cells(b, l6)
    assert e.value.code == 8
    gni = [int(x) for x in d["glo_num_idx"]]
    badv = dict(b, tets=d["tets"].copy())
    badv["tets"][11, 2] = len(d["particles"]) + 5   # a vertex index past the particles
    for _ in range(2):   # twice: the first call may choose the launch variant, the second is pipelined
        with pytest.raises(TessGpuError) as e:
            gpu_ctx.dense(DENSE_DTFE, [badv], gni)
        assert e.value.code == 7
    # the context stays usable
    r = gpu_ctx.dense(DENSE_DTFE, [b], gni)
    assert r["info"]["grid_pts_assigned"] > 0


@pytest.mark.parametrize("given", [False, True])
def test_offset_domain_gpu(gpu_ctx, oracle, given):
    """Anisotropic, offset domain and given grid bounds: DENSE_TESS and
    DENSE_CIC against the restated reference, DTFE owners against the FP64
    oracle (exact) and values within 1e-6 relative L2."""
    import torch
    from test_oracle_golden import _shifted_blocks
    from tess2_gb300.api import DENSE_DTFE
    blocks, g = _shifted_blocks(given)
    gni = [36, 23, 28]
    for alg in (0, 1):
        r = gpu_ctx.dense(alg, blocks, gni, given=g)
        ref = oracle.dense(alg, blocks, gni, given=g)
        assert rel_l2(r["grid"], ref["grid"]) < 1e-5
        assert np.allclose(r["grid"], ref["grid"], rtol=4e-6, atol=0.0)
        assert r["info"]["check_mass"] == ref["check_mass"]
    batch = gpu_ctx.upload(blocks)
    batch.keep_debug(True)
    d = torch.zeros(int(np.prod(gni)), device="cuda:0")
    batch.dense(DENSE_DTFE, gni, d.data_ptr(), given=g)
    torch.cuda.synchronize()
    _, owner, _ = batch.debug_outputs(grid_points=int(np.prod(gni)))
    o = oracle.dtfe(blocks, gni, given=g)
    assert np.array_equal(owner, o["owner"].ravel())
    assert rel_l2(d.cpu().numpy(), o["grid"].ravel()) < 1e-6


# ---------------------------------------------------------------------------
# the brick rasteriser (default) against the row kernel and the oracle
# ---------------------------------------------------------------------------
def _fresh_ctx(env):
    """A context made with the given environment switches (the rasteriser
    kind and launch variant are fixed when a context is made or first used)."""
    import os
    from tess2_gb300.api import Context
    old = {k: os.environ.get(k) for k in env}
    os.environ.update({k: v for k, v in env.items() if v is not None})
    for k, v in env.items():
        if v is None:
            os.environ.pop(k, None)
    try:
        ctx = Context(0)
        return ctx, old
    except Exception:
        _restore(old)
        raise


def _restore(old):
    import os
    for k, v in old.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v


def _dtfe_batch(ctx, blocks, gni, mode, want_owner=True):
    """DTFE of a device batch on a fresh context: the first call picks the
    launch variant, the second is the one checked (grid preset to -7)."""
    import torch
    from tess2_gb300.api import DENSE_DTFE
    b = ctx.upload(blocks)
    b.keep_debug(want_owner)
    grid = torch.full((gni[2], gni[1], gni[0]), -7.0, dtype=torch.float32, device="cuda")
    b.dense(DENSE_DTFE, gni, grid.data_ptr(), mode=mode)
    grid.fill_(-7.0)
    info = b.dense(DENSE_DTFE, gni, grid.data_ptr(), mode=mode)
    owner = None
    if want_owner:
        _, owner, _ = b.debug_outputs(grid_points=grid.numel())
        owner = owner.reshape(grid.shape)
    g = grid.cpu().numpy()
    b.free()
    return g, owner, info


_ROW_VARIANT_GRIDS = {}


@pytest.mark.parametrize("variant", ["0", "1", "2", "3", "4", "5", "6", "7"])
@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 1e-12)])
def test_dtfe_row_variants_vs_oracle(oracle, variant, mode, tol):
    """Every launch variant of the row rasteriser the autotuner may pick
    (blocks per SM, compact, flat, with and without per-slice rows): owners
    equal to the FP64 oracle's, values within the mode's bound, and the same
    grid bits as variant 0."""
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    ref = oracle.dtfe(blocks, gni)
    ctx, old = _fresh_ctx({"TESSGPU_RASTER": "rows", "TESSGPU_RASTER_VARIANT": variant})
    try:
        g, owner, info = _dtfe_batch(ctx, blocks, gni, mode)
    finally:
        _restore(old)
    assert info["raster_variant"] == int(variant)
    assert np.array_equal(owner, ref["owner"])
    assert info["grid_pts_assigned"] == ref["assigned"]
    assert rel_l2(g, ref["grid"]) < tol
    assert np.all(g[ref["owner"] < 0] == 0)
    first = _ROW_VARIANT_GRIDS.setdefault(mode, g)
    assert np.array_equal(g.view(np.uint32), first.view(np.uint32))


@pytest.mark.parametrize("variant", ["0", "1", "2", "3"])
@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 1e-12)])
def test_dtfe_brick_variants_vs_oracle(oracle, variant, mode, tol):
    """Every brick shape the autotuner may pick (TESSGPU_RASTER=bricks): owners equal to the FP64
    oracle's, values within the mode's bound, every grid point written (the
    grid starts at -7 and the brick kernel writes zeros itself)."""
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    ref = oracle.dtfe(blocks, gni)
    ctx, old = _fresh_ctx({"TESSGPU_RASTER": "bricks", "TESSGPU_RASTER_VARIANT": variant})
    try:
        g, owner, info = _dtfe_batch(ctx, blocks, gni, mode)
    finally:
        _restore(old)
    assert info["raster_variant"] == int(variant)
    assert np.array_equal(owner, ref["owner"])
    assert info["grid_pts_assigned"] == ref["assigned"]
    assert rel_l2(g, ref["grid"]) < tol
    assert np.all(g[ref["owner"] < 0] == 0)


@pytest.mark.parametrize("mode", [0, 1])
def test_dtfe_bricks_match_row_kernel(mode):
    """The brick kernel and the per-tet row kernel (TESSGPU_RASTER=rows): the
    same owners and counts, and values within the mode's FP32 rounding of each
    other (the row kernel evaluates each tet along its own row axis, so the
    three-term dot products round in a different order)."""
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [61, 47, 55]
    out = []
    for env in ({"TESSGPU_RASTER": "rows", "TESSGPU_RASTER_VARIANT": None},
                {"TESSGPU_RASTER": "bricks", "TESSGPU_RASTER_VARIANT": None}):
        ctx, old = _fresh_ctx(env)
        try:
            out.append(_dtfe_batch(ctx, blocks, gni, mode))
        finally:
            _restore(old)
    (g0, o0, i0), (g1, o1, i1) = out
    assert np.array_equal(o0, o1)
    for k in ("grid_pts_assigned", "fp64_tets", "exact_tests"):
        assert i0[k] == i1[k], k
    assert rel_l2(g1, g0) < (1e-6 if mode == 0 else 1e-12)


@pytest.mark.parametrize("mode", [0, 1])
def test_dtfe_lattice_ties_gpu(oracle, mode):
    """Particles on a lattice whose points coincide with grid points, plus
    jittered ones: every shared-face, edge and vertex tie occurs, and the GPU
    must give each grid point the oracle's owner (the perturbation rule)."""
    from tess2_gb300 import host
    g1 = np.arange(5, dtype=np.float32) / 4
    lat = np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3)
    jit = host.uniform_particles(40, 5) * np.float32(0.9) + np.float32(0.05)
    for pts in (lat, np.concatenate([lat, jit])):
        tets = host.delaunay_tets(pts)
        blk = [dict(gid=0, particles=pts, tets=tets, vert_to_tet=host.vert_to_tet_host(len(pts), tets),
                    num_orig=len(pts), bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
                    data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))]
        gni = [17, 17, 17]   # step 1/16: the lattice is on grid points
        ref = oracle.dtfe(blk, gni)
        ctx, old = _fresh_ctx({"TESSGPU_RASTER": "bricks", "TESSGPU_RASTER_VARIANT": "3"})
        try:
            g, owner, info = _dtfe_batch(ctx, blk, gni, mode)
        finally:
            _restore(old)
        assert np.array_equal(owner, ref["owner"])
        assert rel_l2(g, ref["grid"]) < (1e-6 if mode == 0 else 1e-12)
        assert info["exact_tests"] > 0


def test_dtfe_split_bricks_and_pair_retry(oracle):
    """Two particles per grid point put tens of thousands of candidate tets
    into each brick, so every brick's work is split into items of 2048 (the
    regions zeroed first); a pair list sized far too small
    (TESSGPU_PAIR_CAP) makes the call retry with the size it needed."""
    from tess2_gb300 import host
    pts = host.uniform_particles(30000, 9)
    tets = host.delaunay_tets(pts)
    blk = [dict(gid=0, particles=pts, tets=tets, vert_to_tet=host.vert_to_tet_host(len(pts), tets),
                num_orig=len(pts), bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
                data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))]
    gni = [24, 24, 24]
    ref = oracle.dtfe(blk, gni)
    for env in ({"TESSGPU_RASTER_VARIANT": "0", "TESSGPU_PAIR_CAP": None},
                {"TESSGPU_RASTER_VARIANT": "0", "TESSGPU_PAIR_CAP": "1000"}):
        ctx, old = _fresh_ctx(dict(env, TESSGPU_RASTER="bricks"))
        try:
            g, owner, info = _dtfe_batch(ctx, blk, gni, 0)
            # and once more through the host-buffer call on the same context
            r = ctx.dense(2, blk, gni)
        finally:
            _restore(old)
        assert np.array_equal(owner, ref["owner"])
        assert rel_l2(g, ref["grid"]) < 1e-6
        assert np.array_equal(r["grid"], g)
