"""The allocation-free DTFE density entry point (tessgpu_dtfe_densities_noalloc).

It exists for callers that cannot allocate GPU memory when they need the
densities (in-situ analysis inside a simulation that owns the device's
memory, or code that must not let cudaMalloc/cudaFree synchronise the
device).  Its scratch is a static array in the library shared by every call,
so the test makes two calls in a row on different blocks (the second must not
see the first one's sums) and compares each with the densities the batch
DENSE_DTFE path computes for the same block.  The file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_single, single_block

pytestmark = pytest.mark.gpu


def batch_rho(ctx, d):
    import torch
    from tess2_gb300.api import DENSE_DTFE
    gni = [int(x) for x in d["glo_num_idx"]]
    b = ctx.upload(single_block(d))
    b.keep_debug(True)
    grid = torch.zeros(gni[2], gni[1], gni[0], dtype=torch.float32, device="cuda")
    b.dense(DENSE_DTFE, gni, grid.data_ptr())
    _, _, rho = b.debug_outputs(particles=len(d["particles"]))
    return rho


def noalloc_rho(d, blk, mode=0):
    import torch
    from tess2_gb300.api import lib
    p = torch.from_numpy(np.ascontiguousarray(d["particles"], np.float32)).cuda()
    t = torch.from_numpy(np.ascontiguousarray(d["tets"], np.int32)).cuda()
    rho = torch.full((p.shape[0],), -1.0, dtype=torch.float32, device="cuda")
    # the data bounds dense() derives for this one block: its own bounds
    bounds = (ctypes.c_float * 6)(*[float(x) for x in blk["data_min"]], *[float(x) for x in blk["data_max"]])
    torch.cuda.synchronize()
    s = lib().tessgpu_dtfe_densities_noalloc(p.data_ptr(), p.shape[0], t.data_ptr(), t.shape[0], bounds, 1.0, mode,
                                             rho.data_ptr(), None)
    assert s == 0
    return rho.cpu().numpy()


def test_noalloc_matches_batch_path_twice(gpu_ctx, oracle):
    # two calls in a row through the C ABI, on blocks of different sizes: the
    # same arithmetic and fixed-point sums as the batch path, so the same bits
    for name in ("c1_uniform4096_seed1", "mix2048_seed7"):
        d = load_single(name)
        blk = single_block(d)[0]
        ref = batch_rho(gpu_ctx, d)
        got = noalloc_rho(d, blk)
        assert np.all(np.isfinite(got))
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
        # and the FP64 oracle's densities, within FP32 rounding of the result
        orc = oracle.dtfe(single_block(d), [8, 8, 8], want_owner=False)["rho"]
        assert np.allclose(got, orc, rtol=2e-6, atol=0.0)


def test_noalloc_rejects_oversize():
    from tess2_gb300.api import lib
    from tess2_gb300 import build
    build.build()
    bounds = (ctypes.c_float * 6)(0, 0, 0, 1, 1, 1)
    n = (1 << 21) + 1
    s = lib().tessgpu_dtfe_densities_noalloc(1, n, 1, 1, bounds, 1.0, 0, 1, None)
    assert s == 1   # TESSGPU_ERR_INVALID, before any device work
