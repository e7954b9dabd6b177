"""Parity at a size the small golden cases do not reach: 262,144 particles of
the benchmark's mixture (50 % uniform, 50 % in 256 Gaussian clumps of sigma
0.01), 2x2x2 blocks with a 0.05 ghost zone, onto a 256^3 grid -- the same
particles per grid point as 2,097,152 particles onto 512^3.

The oracle recomputes a sample (oracle/parity.py): DTFE for every 16th tet of
each block in FP64 (owners point for point, values within 1e-6 relative L2
in mixed mode and 1e-12 in FP64 mode), and the reference estimator's
per-cell CellGridPts results for a seeded random sample of every block's
cells (uniform and clump cells alike), which must be bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GNI = [256, 256, 256]
STRIDE = 16


@pytest.fixture(scope="module")
def mix_blocks():
    from tess2_gb300 import host
    pts = host.mixture_particles(262144, 77, frac_uniform=0.5, n_clumps=256, sigma=0.01)
    return host.tessellate(host.decompose(pts, (2, 2, 2), 0.05))


@pytest.fixture(scope="module")
def dtfe_sample(mix_blocks):
    from oracle import parity
    return parity.dtfe_oracle_sample(mix_blocks, GNI, STRIDE)


@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 1e-12)])
def test_dtfe_sampled_vs_fp64_oracle(gpu_ctx, mix_blocks, dtfe_sample, mode, tol):
    import torch
    from oracle import parity
    from tess2_gb300.api import DENSE_DTFE
    b = gpu_ctx.upload(mix_blocks)
    b.keep_debug(True)
    g = torch.full((int(np.prod(GNI)),), -7.0, dtype=torch.float32, device="cuda")
    info = b.dense(DENSE_DTFE, GNI, g.data_ptr(), mode=mode)
    _, owner, _ = b.debug_outputs(grid_points=g.numel())
    grid = g.cpu().numpy()
    b.free()
    r = parity.dtfe_compare(grid, owner, dtfe_sample, STRIDE)
    assert r["points"] > 500000
    assert r["owners_equal"] and r["no_extra"], r
    assert r["rel_l2"] < tol, r
    # every grid point was written; points owned by no tet are zero
    assert np.all(grid[owner < 0] == 0)
    assert info["grid_pts_assigned"] == int(np.count_nonzero(owner >= 0))


def test_dense_tess_sampled_cell_counts(gpu_ctx, mix_blocks):
    import torch
    from oracle import parity
    from tess2_gb300.api import DENSE_TESS
    b = gpu_ctx.upload(mix_blocks)
    b.keep_debug(True)
    g = torch.zeros(int(np.prod(GNI)), dtype=torch.float32, device="cuda")
    b.dense(DENSE_TESS, GNI, g.data_ptr())
    total = sum(int(x["num_orig"]) for x in mix_blocks)
    counts, _, _ = b.debug_outputs(cells=total)
    b.free()
    cells = parity.tess_cell_sample(mix_blocks, 1500, seed=5)
    ref = parity.tess_counts_oracle(mix_blocks, GNI, cells)
    off = 0
    for blk, c, r in zip(mix_blocks, cells, ref):
        assert np.array_equal(counts[off + c], r)
        off += int(blk["num_orig"])


@pytest.mark.parametrize("mode", [0, 1])
def test_dtfe_star_sums_batch_vs_noalloc(gpu_ctx, mix_blocks, mode):
    """Vertex densities of the mixture, block by block: the batch path (all
    blocks' tets in one star-volume launch) against the allocation-free entry
    point (its own kernel, one block per call).  Both sum the star volumes as
    fixed-point integers at the scale of the same data bounds, so the
    densities agree bit for bit whatever order the atomics land in."""
    import ctypes
    import torch
    from tess2_gb300.api import DENSE_DTFE, lib
    b = gpu_ctx.upload(mix_blocks)
    b.keep_debug(True)
    g = torch.zeros(int(np.prod(GNI)), dtype=torch.float32, device="cuda")
    b.dense(DENSE_DTFE, GNI, g.data_ptr(), mode=mode)
    total = sum(len(x["particles"]) for x in mix_blocks)
    _, _, rho = b.debug_outputs(particles=total)
    b.free()
    mn = np.min([x["bounds_min"] for x in mix_blocks], axis=0)
    mx = np.max([x["bounds_max"] for x in mix_blocks], axis=0)
    bounds = (ctypes.c_float * 6)(*[float(v) for v in mn], *[float(v) for v in mx])
    off = 0
    for blk in mix_blocks:
        p = torch.from_numpy(np.ascontiguousarray(blk["particles"], np.float32)).cuda()
        t = torch.from_numpy(np.ascontiguousarray(blk["tets"], np.int32)).cuda()   # tet_t records
        assert t.dim() == 2 and t.shape[1] == 8
        out = torch.full((p.shape[0],), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        s = lib().tessgpu_dtfe_densities_noalloc(p.data_ptr(), p.shape[0], t.data_ptr(), t.shape[0], bounds, 1.0,
                                                 mode, out.data_ptr(), None)
        assert s == 0
        got = rho[off:off + p.shape[0]]
        assert np.array_equal(got.view(np.uint32), out.cpu().numpy().view(np.uint32))
        off += p.shape[0]
    assert off == total
