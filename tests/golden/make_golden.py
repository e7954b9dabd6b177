"""Generates the golden vectors in tests/golden/ from the reference itself.

The reference's own src/tet.cpp, src/volume.cpp and src/dense.cpp, compiled
unmodified by `make -C oracle ref` (g++ -O2 -ffp-contract=off, flags recorded
in each file), compute every output stored here.  Inputs are seeded
synthetic particle sets; their Delaunay tets come from scipy's Qhull ("Qt"),
the stand-in for tess2's host Qhull engine, and are stored with the outputs
so that no machine has to reproduce Qhull's numbering.

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py             (everything)
    python tests/golden/make_golden.py writegrid   (only writegrid.npz, from the stored inputs)
Each dense() call runs in a fresh process: the reference keeps its
max_dense / tot_mass / check_mass statistics in process-global variables
(src/dense.cpp:25-27).
"""
import json
import multiprocessing as mp
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
OUT = os.path.dirname(os.path.abspath(__file__))


def _dense_in_child(args):
    alg, blocks, gni = args
    from oracle.oracle import Oracle
    r = Oracle("ref").dense(alg, blocks, gni)
    return r


def dense_fresh(alg, blocks, gni):
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        return pool.map(_dense_in_child, [(alg, blocks, gni)])[0]


def _write_in_child(args):
    alg, blocks, gni, project, path = args
    from oracle.oracle import Oracle
    return Oracle("ref").dense_write(alg, blocks, gni, path, project=project)


def dense_write_fresh(alg, blocks, gni, project):
    """dense() + WriteGrid of the reference in a fresh process; returns (result, file contents)."""
    import tempfile
    fd, path = tempfile.mkstemp(suffix=".raw")
    os.close(fd)
    try:
        ctx = mp.get_context("spawn")
        with ctx.Pool(1) as pool:
            r = pool.map(_write_in_child, [(alg, blocks, gni, project, path)])[0]
        return r, np.fromfile(path, np.float32)
    finally:
        os.remove(path)


def flags():
    with open(os.path.join(ROOT, "oracle", "_ref", "FLAGS.txt")) as f:
        return f.read().strip()


def case_single(name, pts, gni):
    from oracle.oracle import Oracle
    from tess2_gb300 import host
    R = Oracle("ref")
    blocks = host.tessellate(host.decompose(pts))
    b = blocks[0]
    p, t, v = b["particles"], b["tets"], b["vert_to_tet"]
    cc = R.fill_circumcenters(p, t)
    comp = R.complete_all(t, v)
    vol = R.volumes(p, t, v)
    out = dict(particles=p, tets=t, vert_to_tet=v, circumcenters=cc, complete=comp, volumes=vol,
               glo_num_idx=np.array(gni, np.int32))
    for alg, tag in ((0, "tess"), (1, "cic")):
        r = dense_fresh(alg, blocks, gni)
        out[f"{tag}_grid"] = r["grid"]
        out[f"{tag}_stats"] = np.array([r["max_dense"], r["tot_mass"], r["check_mass"]])
        out["grid_min"], out["grid_step"] = r["grid_min"], r["grid_step"]
    # per-cell CellGridPts results of the reference (count, or -1 skipped, 0 outside)
    counts = np.empty(len(p), np.int32)
    for c in range(len(p)):
        n, _, _, _ = R.cell_grid_pts(b, c, r["data_min"], r["data_max"], r["grid_min"], r["grid_step"])
        counts[c] = n
    out["tess_cell_counts"] = counts
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
    return dict(name=name, n=int(len(p)), tets=int(len(t)), grid=list(gni), cells_deposited=int((counts > 0).sum()))


def case_blocks(name, pts, dims, ghost, gni):
    from tess2_gb300 import host
    blocks = host.tessellate(host.decompose(pts, dims, ghost))
    out = dict(glo_num_idx=np.array(gni, np.int32), nblocks=np.int32(len(blocks)))
    for i, b in enumerate(blocks):
        for k in ("particles", "tets", "vert_to_tet", "bounds_min", "bounds_max", "data_min", "data_max"):
            out[f"b{i}_{k}"] = b[k]
        out[f"b{i}_num_orig"] = np.int32(b["num_orig"])
        out[f"b{i}_gid"] = np.int32(b["gid"])
    for alg, tag in ((0, "tess"), (1, "cic")):
        r = dense_fresh(alg, blocks, gni)
        out[f"{tag}_grid"] = r["grid"]
        out[f"{tag}_stats"] = np.array([r["max_dense"], r["tot_mass"], r["check_mass"]])
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
    return dict(name=name, blocks=len(blocks), dims=list(dims), ghost=ghost, grid=list(gni))


def case_writegrid():
    """WriteGrid files (src/dense.cpp:751-870) written by the reference's own
    WriteGrid through oracle/ref_shim's MPI-IO, for the stored inputs above:
    projected (ProjectGrid) for every case, and a check that the 3-D file is
    the stored global grid.  Inputs are read back from the fixtures, not
    re-tessellated."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from conftest import load_blocks, load_single, single_block
    out = {}
    cases = []
    for name in ("c1_uniform4096_seed1", "mix2048_seed7"):
        d = load_single(name)
        cases.append((name, single_block(d), [int(x) for x in d["glo_num_idx"]], d))
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    cases.append(("blocks8_mix8192_seed3", blocks, [int(x) for x in d["glo_num_idx"]], d))
    for name, blocks, gni, d in cases:
        for alg, tag in ((0, "tess"), (1, "cic")):
            r3, f3 = dense_write_fresh(alg, blocks, gni, False)
            assert np.array_equal(f3.view(np.uint32), d[f"{tag}_grid"].ravel().view(np.uint32)), name
            r, f = dense_write_fresh(alg, blocks, gni, True)
            out[f"{name}_{tag}_proj_file"] = f
            out[f"{name}_{tag}_proj_blocks"] = np.concatenate(r["blocks"])
            out[f"{name}_{tag}_proj_block_sizes"] = np.array([len(b) for b in r["blocks"]], np.int32)
            out[f"{name}_{tag}_proj_stats"] = np.array([r["max_dense"], r["tot_mass"], r["check_mass"]])
    np.savez_compressed(os.path.join(OUT, "writegrid.npz"), **out)
    return dict(name="writegrid", files=sorted(k for k in out if k.endswith("_file")))


def main():
    if sys.argv[1:] == ["writegrid"]:
        meta = json.load(open(os.path.join(OUT, "golden.json")))
        meta["cases"] = [c for c in meta["cases"] if c["name"] != "writegrid"] + [case_writegrid()]
        with open(os.path.join(OUT, "golden.json"), "w") as f:
            json.dump(meta, f, indent=1)
        return
    from tess2_gb300 import host
    meta = dict(reference_build=flags(), delaunay="scipy.spatial.Delaunay(qhull_options='Qt')",
                mass=1.0, eps=1e-4, cases=[])
    # the small plain-method workload: 4096 uniform particles, one block, 64^3
    meta["cases"].append(case_single("c1_uniform4096_seed1", host.uniform_particles(4096, 1), [64, 64, 64]))
    # clumpy particles on a grid that is not a power of two
    meta["cases"].append(case_single("mix2048_seed7", host.mixture_particles(2048, 7, n_clumps=16, sigma=0.03),
                                     [33, 40, 29]))
    # 2x2x2 blocks with ghosts: cross-block deposits through the exchange
    meta["cases"].append(case_blocks("blocks8_mix8192_seed3", host.mixture_particles(8192, 3), (2, 2, 2), 0.1,
                                     [40, 40, 40]))
    # WriteGrid / ProjectGrid output of the cases above
    meta["cases"].append(case_writegrid())
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
