"""Host-side preparation of DIY-style blocks for the GPU path.

The Delaunay construction stays on the host, as in tess2: tess2 runs Qhull
(src/tess-qhull.c:46, options "qhull d Qt") or CGAL per block.  Here scipy's
bundled Qhull with "Qt" stands in for that engine.  Its simplices/neighbors
already follow tet_t's convention (include/tess/tet.h:4-7): neighbour i lies
opposite vertex i, -1 on the convex hull.

Also here: the seeded synthetic particle sets of the benchmark workloads and
a regular block decomposition with a ghost zone (tess2 instead grows ghosts
adaptively, src/tess.cpp:492-628; that is a host choice outside the GPU path).
"""
import multiprocessing as mp
import os

import numpy as np

TET_FIELDS = 8  # tet_t: int verts[4]; int tets[4]


def uniform_particles(n, seed):
    """n float32 points uniform in [0,1)^3 from a seed."""
    rng = np.random.default_rng(seed)
    return rng.random((n, 3), dtype=np.float32)


def mixture_particles(n, seed, frac_uniform=0.5, n_clumps=256, sigma=0.01, sigma_range=None):
    """Uniform background plus isotropic Gaussian clumps in [0,1)^3.

    Clump centres are uniform, clump weights Dirichlet(1); samples that fall
    outside the unit box are redrawn.  sigma_range=(lo, hi) draws each clump's
    sigma log-uniformly instead of using one sigma.
    """
    rng = np.random.default_rng(seed)
    n_uni = int(round(n * frac_uniform))
    n_cl = n - n_uni
    pts = [rng.random((n_uni, 3))]
    if n_cl > 0:
        centres = rng.random((n_clumps, 3))
        if sigma_range is not None:
            lo, hi = np.log(sigma_range[0]), np.log(sigma_range[1])
            sig = np.exp(rng.uniform(lo, hi, n_clumps))
        else:
            sig = np.full(n_clumps, sigma)
        w = rng.dirichlet(np.ones(n_clumps))
        counts = rng.multinomial(n_cl, w)
        cid = np.repeat(np.arange(n_clumps), counts)
        out = np.empty((n_cl, 3))
        todo = np.arange(n_cl)
        while todo.size:
            c = cid[todo]
            s = centres[c] + rng.standard_normal((todo.size, 3)) * sig[c, None]
            ok = np.all((s >= 0.0) & (s < 1.0), axis=1)
            out[todo[ok]] = s[ok]
            todo = todo[~ok]
        pts.append(out)
    p = np.concatenate(pts).astype(np.float32)
    # float32 rounding can land exactly on 1.0
    np.minimum(p, np.nextafter(np.float32(1.0), np.float32(0.0)), out=p)
    return p


def delaunay_tets(points):
    """Qhull Delaunay tets of float32 points as a (T, 8) int32 tet_t array."""
    from scipy.spatial import Delaunay
    pts = np.asarray(points, dtype=np.float32)
    if pts.shape[0] < 5:
        return np.zeros((0, TET_FIELDS), np.int32)
    d = Delaunay(pts.astype(np.float64), qhull_options="Qt")
    tets = np.empty((d.simplices.shape[0], TET_FIELDS), np.int32)
    tets[:, :4] = d.simplices
    tets[:, 4:] = d.neighbors
    return tets


def vert_to_tet_host(num_particles, tets):
    """fill_vert_to_tet (src/tess.cpp:767-787) on the host: the last tet wins."""
    v2t = np.full(num_particles, -1, np.int32)
    if tets.shape[0]:
        np.maximum.at(v2t, tets[:, :4].ravel(),
                      np.repeat(np.arange(tets.shape[0], dtype=np.int32), 4))
    return v2t


def decompose(points, dims=(1, 1, 1), ghost=0.0, domain_min=(0.0, 0.0, 0.0), domain_max=(1.0, 1.0, 1.0)):
    """Regular dims[0] x dims[1] x dims[2] blocks over the domain.

    Each block keeps its own points first (num_orig) followed by ghost points
    within `ghost` of its bounds, like a DIY block after the tess2 exchange.
    Block gid = i + dims[0] * (j + dims[1] * k).
    """
    pts = np.asarray(points, dtype=np.float32)
    dmin = np.asarray(domain_min, np.float32)
    dmax = np.asarray(domain_max, np.float32)
    dims = np.asarray(dims)
    ext = (dmax - dmin) / dims
    # owner block of every point (points exactly on dmax go to the last block)
    cell = np.floor((pts - dmin) / ext).astype(np.int64)
    cell = np.clip(cell, 0, dims - 1)
    owner = cell[:, 0] + dims[0] * (cell[:, 1] + dims[1] * cell[:, 2])
    blocks = []
    for k in range(dims[2]):
        for j in range(dims[1]):
            for i in range(dims[0]):
                gid = i + dims[0] * (j + dims[1] * k)
                bmin = (dmin + ext * np.array([i, j, k])).astype(np.float32)
                bmax = (dmin + ext * np.array([i + 1, j + 1, k + 1])).astype(np.float32)
                if i == dims[0] - 1:
                    bmax[0] = dmax[0]
                if j == dims[1] - 1:
                    bmax[1] = dmax[1]
                if k == dims[2] - 1:
                    bmax[2] = dmax[2]
                own = np.nonzero(owner == gid)[0]
                if ghost > 0:
                    near = np.all((pts >= bmin - ghost) & (pts <= bmax + ghost), axis=1)
                    near[own] = False
                    gh = np.nonzero(near)[0]
                else:
                    gh = np.zeros(0, np.int64)
                blocks.append(dict(gid=int(gid), particles=np.concatenate([pts[own], pts[gh]]),
                                   num_orig=int(own.size), global_ids=np.concatenate([own, gh]),
                                   bounds_min=bmin, bounds_max=bmax,
                                   data_min=dmin.copy(), data_max=dmax.copy()))
    return blocks


def _tess_one(p):
    return delaunay_tets(p)


def tessellate(blocks, processes=None):
    """Fill tets and vert_to_tet of every block (host Qhull, one process per block)."""
    work = [b["particles"] for b in blocks]
    if processes is None:
        processes = min(len(blocks), os.cpu_count() or 1)
    if processes > 1 and len(blocks) > 1:
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes) as pool:
            tets = pool.map(_tess_one, work)
    else:
        tets = [_tess_one(p) for p in work]
    for b, t in zip(blocks, tets):
        b["tets"] = t
        b["vert_to_tet"] = vert_to_tet_host(b["particles"].shape[0], t)
    return blocks


def shard_blocks(blocks, rank, world):
    """The blocks rank `rank` of `world` processes (round robin by position).

    Blocks are independent units of the density path: each writes only the
    grid points of its own BlockGridParams box, so ranks need no exchange on
    the data path; the data bounds all ranks must agree on are those of the
    whole decomposition (data_bounds_of(blocks)).
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return blocks[rank::world]


def data_bounds_of(blocks):
    """DataBounds over all blocks (src/dense.cpp:1221-1275): min/max of block bounds."""
    mn = np.min([b["bounds_min"] for b in blocks], axis=0).astype(np.float32)
    mx = np.max([b["bounds_max"] for b in blocks], axis=0).astype(np.float32)
    return mn, mx
