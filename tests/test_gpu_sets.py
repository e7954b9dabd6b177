"""Many independent particle sets in one call (tessgpu_batch_dense_sets): each
block is its own dense() over its own grid, all sets share every stage's
launch (one rasteriser launch over all of them, row or brick kernel); with
graph=True the step is recorded into a CUDA graph once and replayed.

Each set's grid must equal what a one-block tessgpu_batch_dense of that set
writes (bit for bit: same arithmetic, same fixed-point scale for sets in the
same box) and agree with the FP64 oracle within the mode's bound."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def make_sets(n, seed):
    from tess2_gb300 import host
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(1500), np.log(12000), n)).astype(int)
    sides = rng.choice([16, 24, 32, 40], n)
    blocks = []
    for i, c in enumerate(counts):
        pts = host.mixture_particles(int(c), seed * 100 + i, frac_uniform=0.5, n_clumps=8, sigma=0.03)
        blocks.append(dict(gid=i, particles=pts, num_orig=len(pts), bounds_min=np.zeros(3, np.float32),
                           bounds_max=np.ones(3, np.float32), data_min=np.zeros(3, np.float32),
                           data_max=np.ones(3, np.float32)))
    blocks = host.tessellate(blocks)
    gni = [[int(s), int(s) + 2 * (i % 2), int(s) - 2 * (i % 3 == 0)] for i, s in enumerate(sides)]
    return blocks, gni


def make_ctx(kind):
    """A context whose dense() rasteriser is kind ("rows" or "bricks")."""
    import os
    from tess2_gb300.api import Context
    old = os.environ.get("TESSGPU_RASTER")
    os.environ["TESSGPU_RASTER"] = kind
    try:
        return Context(0)
    finally:
        if old is None:
            os.environ.pop("TESSGPU_RASTER", None)
        else:
            os.environ["TESSGPU_RASTER"] = old


@pytest.mark.parametrize("kind", ["rows", "bricks"])
@pytest.mark.parametrize("mode,tol", [(0, 1e-6), (1, 1e-12)])
def test_sets_match_single_block_runs_and_oracle(oracle, kind, mode, tol):
    import torch
    from tess2_gb300.api import DENSE_DTFE, sets_offsets
    gpu_ctx = make_ctx(kind)
    blocks, gni = make_sets(7, 31)
    total, off = sets_offsets(gni)
    out = torch.full((total,), -7.0, dtype=torch.float32, device="cuda")
    b = gpu_ctx.upload(blocks)
    info = b.dense_sets(gni, out.data_ptr(), mode=mode)
    got = out.cpu().numpy()
    assert info["grid_floats"] == total and (info["brick_pairs"] > 0) == (kind == "bricks")
    assigned = 0
    for i, blk in enumerate(blocks):
        n = int(np.prod(gni[i]))
        mine = got[off[i]:off[i] + n].reshape(gni[i][2], gni[i][1], gni[i][0])
        one = gpu_ctx.upload([blk])
        g = torch.zeros(n, dtype=torch.float32, device="cuda")
        one.dense(DENSE_DTFE, gni[i], g.data_ptr(), mode=mode)
        one.free()
        assert np.array_equal(mine.ravel(), g.cpu().numpy()), i
        ref = oracle.dtfe([blk], gni[i], want_owner=True)
        assert rel_l2(mine, ref["grid"]) < tol
        assert np.count_nonzero(mine) <= ref["assigned"]
        assigned += ref["assigned"]
    assert info["grid_pts_assigned"] == assigned
    b.free()


@pytest.mark.parametrize("kind", ["rows", "bricks"])
def test_sets_graph_replay(kind):
    """The recorded step replays to the same grids, call after call, and a
    replay after the output was overwritten rewrites every point."""
    import torch
    from tess2_gb300.api import sets_offsets
    gpu_ctx = make_ctx(kind)
    blocks, gni = make_sets(5, 8)
    total, off = sets_offsets(gni)
    b = gpu_ctx.upload(blocks)
    ref = torch.zeros(total, dtype=torch.float32, device="cuda")
    b.dense_sets(gni, ref.data_ptr())
    out = torch.full((total,), 3.0, dtype=torch.float32, device="cuda")
    infos = []
    for k in range(3):
        out.fill_(float(k) - 5.0)
        infos.append(b.dense_sets(gni, out.data_ptr(), graph=True))
        torch.cuda.synchronize()
        assert torch.equal(out, ref), k
    for k in ("grid_pts_assigned", "exact_tests", "fp64_tets", "brick_pairs"):
        assert infos[0][k] == infos[1][k] == infos[2][k], k
    assert infos[0]["grid_pts_assigned"] > 0
    b.free()
