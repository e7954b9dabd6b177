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
