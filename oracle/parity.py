"""Sampled parity checks of a large GPU run against the CPU oracle.

Test infrastructure, like the rest of oracle/: tests/ and bench.py use it to
check the GPU's output at workload sizes the oracle cannot recompute whole in
seconds.  Blocks are checked in parallel worker processes (spawned, so a
parent that already holds a CUDA context is safe).

* DTFE: the FP64 oracle (orc_dtfe_f64_sample) rasterises every stride-th tet
  of each block, star volumes over all tets.  A grid point holds a value in
  the oracle's output exactly when its owner is one of those tets; the GPU's
  owner array (block-local tet indices) must agree there point for point, and
  its values must agree within the mode's relative L2 bound over those points.
* DENSE_TESS: per-cell CellGridPts results (the reference's own estimator,
  src/dense.cpp:1363-1458, restated bit-exactly) of a seeded random sample of
  every block's cells against the GPU's per-cell counts.
"""
import multiprocessing as mp

import numpy as np


def _dtfe_block(block, data6, gni, stride):
    from oracle.oracle import Restated
    r = Restated().dtfe([block], gni, want_rho=False, data6=data6, raster_stride=stride)
    own = r["owner"].ravel()
    idx = np.flatnonzero(own >= 0)
    return idx.astype(np.int64), own[idx].astype(np.int32), r["grid"].ravel()[idx]


def _data6(blocks):
    mn = np.min([b["bounds_min"] for b in blocks], axis=0)
    mx = np.max([b["bounds_max"] for b in blocks], axis=0)
    return np.concatenate([mn, mx]).astype(np.float32)


def dtfe_oracle_sample(blocks, gni, stride, processes=None):
    """The oracle's sampled DTFE of every block (in parallel): flat grid indices,
    block-local owner tets and FP64-oracle values (float32) of the points whose
    owner is a sampled tet (block-local index divisible by stride)."""
    d6 = _data6(blocks)
    procs = processes or min(len(blocks), mp.cpu_count() or 1)
    args = [(b, d6, list(gni), stride) for b in blocks]
    if procs > 1 and len(blocks) > 1:
        with mp.get_context("spawn").Pool(procs) as pool:
            parts = pool.starmap(_dtfe_block, args)
    else:
        parts = [_dtfe_block(*a) for a in args]
    idx = np.concatenate([p[0] for p in parts])
    own = np.concatenate([p[1] for p in parts])
    val = np.concatenate([p[2] for p in parts])
    return idx, own, val


def dtfe_compare(gpu_grid, gpu_owner, sample, stride):
    """Compare a GPU DTFE run (flat float32 grid, flat block-local owner array)
    with dtfe_oracle_sample's output.  Returns a dict of counts and errors; the
    owners agree when owners_equal and no_extra are both true."""
    idx, own, val = sample
    g_own = gpu_owner[idx]
    owners_equal = bool(np.array_equal(g_own, own))
    # the GPU must not give a sampled tet any point the oracle does not
    gpu_sampled = int(np.count_nonzero((gpu_owner >= 0) & (gpu_owner % stride == 0)))
    g = gpu_grid[idx].astype(np.float64)
    v = val.astype(np.float64)
    nv = np.linalg.norm(v)
    rel = float(np.linalg.norm(g - v) / (nv if nv > 0 else 1.0))
    nz = v != 0
    max_rel = float(np.max(np.abs(g[nz] - v[nz]) / np.abs(v[nz]))) if np.any(nz) else 0.0
    return dict(points=int(idx.size), owners_equal=owners_equal, no_extra=gpu_sampled == int(idx.size),
                rel_l2=rel, max_rel=max_rel, stride=stride)


def _tess_block(block, data6, gni, cells):
    from oracle.oracle import TessCells
    _, counts = TessCells(block, data6, gni).run(cells, counts=True)
    return counts


def tess_cell_sample(blocks, per_block, seed):
    """A seeded random sample of per_block cells of every block (uniform and
    clump cells alike): a list of int32 arrays of block-local cell indices."""
    rng = np.random.default_rng(seed)
    return [np.sort(rng.choice(b["num_orig"], size=min(per_block, b["num_orig"]), replace=False)).astype(np.int32)
            for b in blocks]


def tess_counts_oracle(blocks, gni, cells, processes=None):
    """The restated reference's CellGridPts result for the sampled cells of each block."""
    d6 = _data6(blocks)
    procs = processes or min(len(blocks), mp.cpu_count() or 1)
    args = [(b, d6, list(gni), c) for b, c in zip(blocks, cells)]
    if procs > 1 and len(blocks) > 1:
        with mp.get_context("spawn").Pool(procs) as pool:
            return pool.starmap(_tess_block, args)
    return [_tess_block(*a) for a in args]
