"""The restated oracle (oracle/tess_oracle.c) against the reference's golden
vectors (tests/golden/, produced by the reference's own sources).  Bit-exact:
every float compared by its bits."""
import numpy as np
import pytest

from conftest import load_blocks, load_single, single_block

SINGLE = ["c1_uniform4096_seed1", "mix2048_seed7"]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", SINGLE)
def test_vert_to_tet(oracle, name):
    d = load_single(name)
    assert np.array_equal(oracle.fill_vert_to_tet(len(d["particles"]), d["tets"]), d["vert_to_tet"])


@pytest.mark.parametrize("name", SINGLE)
def test_circumcenters(oracle, name):
    d = load_single(name)
    assert np.array_equal(bits(oracle.fill_circumcenters(d["particles"], d["tets"])), bits(d["circumcenters"]))


@pytest.mark.parametrize("name", SINGLE)
def test_complete(oracle, name):
    d = load_single(name)
    assert np.array_equal(oracle.complete_all(d["tets"], d["vert_to_tet"]), d["complete"])


@pytest.mark.parametrize("name", SINGLE)
def test_volumes(oracle, name):
    d = load_single(name)
    v = oracle.volumes(d["particles"], d["tets"], d["vert_to_tet"])
    assert np.array_equal(bits(v), bits(d["volumes"]))


@pytest.mark.parametrize("name", SINGLE)
@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
def test_dense_single(oracle, name, alg, tag):
    d = load_single(name)
    r = oracle.dense(alg, single_block(d), [int(x) for x in d["glo_num_idx"]], cell_counts=True)
    assert np.array_equal(bits(r["grid"]), bits(d[f"{tag}_grid"]))
    st = d[f"{tag}_stats"]
    assert (r["max_dense"], r["tot_mass"], r["check_mass"]) == (st[0], st[1], st[2])
    assert r["lost"] == 0
    if alg == 0:
        assert np.array_equal(r["cell_counts"], d["tess_cell_counts"])


@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
def test_dense_blocks(oracle, alg, tag):
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    r = oracle.dense(alg, blocks, [int(x) for x in d["glo_num_idx"]])
    assert np.array_equal(bits(r["grid"]), bits(d[f"{tag}_grid"]))
    st = d[f"{tag}_stats"]
    # tot_mass / check_mass are per call here; the golden run was a fresh process
    assert (r["max_dense"], r["tot_mass"], r["check_mass"]) == (st[0], st[1], st[2])


def test_cell_grid_pts_matches_counts(oracle):
    d = load_single("mix2048_seed7")
    b = single_block(d)[0]
    r = oracle.dense(0, [b], [int(x) for x in d["glo_num_idx"]])
    for c in range(0, len(d["particles"]), 97):
        n, idx, m, _ = oracle.cell_grid_pts(b, c, r["data_min"], r["data_max"], r["grid_min"], r["grid_step"])
        assert n == d["tess_cell_counts"][c]
        if n > 0:
            assert idx.shape == (n, 3)
            assert np.isclose(m.sum(), 1.0, rtol=1e-5)


def test_empty_and_tiny_blocks(oracle):
    """Degenerate inputs the reference loops over without work: no particles,
    and four particles without tets."""
    empty = dict(particles=np.zeros((0, 3), np.float32), tets=np.zeros((0, 8), np.int32),
                 vert_to_tet=np.zeros(0, np.int32), num_orig=0, bounds_min=np.zeros(3, np.float32),
                 bounds_max=np.ones(3, np.float32), data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))
    r = oracle.dense(0, [empty], [8, 8, 8])
    assert r["grid"].sum() == 0 and r["check_mass"] == 0
    four = dict(empty, particles=np.random.default_rng(0).random((4, 3), dtype=np.float32),
                vert_to_tet=np.full(4, -1, np.int32), num_orig=4)
    r = oracle.dense(0, [four], [8, 8, 8])
    assert r["grid"].sum() == 0
    r = oracle.dense(1, [four], [8, 8, 8])
    assert r["check_mass"] == 4


def shuffled_neighbors(tets, seed):
    """tet_t records with each tet's neighbour list permuted (Qhull's order)."""
    rng = np.random.default_rng(seed)
    t = tets.copy()
    perm = np.argsort(rng.random((t.shape[0], 4)), axis=1)
    t[:, 4:] = np.take_along_axis(t[:, 4:], perm, axis=1)
    return t


@pytest.mark.parametrize("name", SINGLE)
def test_reorder_neighbors(oracle, name):
    d = load_single(name)
    got = oracle.reorder_neighbors(shuffled_neighbors(d["tets"], 1))
    assert np.array_equal(got, d["tets"])


@pytest.mark.parametrize("name", ["c1_uniform4096_seed1", "mix2048_seed7", "blocks8_mix8192_seed3"])
@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
def test_projected_writegrid(oracle, name, alg, tag):
    """dense(project) + ProjectGrid + WriteGrid: the restated oracle against
    the file the reference's own WriteGrid wrote, and every block's array."""
    from conftest import load_case_blocks, load_writegrid
    d, blocks, gni = load_case_blocks(name)
    w = load_writegrid()
    r = oracle.dense(alg, blocks, gni, project=True, block_arrays=True)
    f = w[f"{name}_{tag}_proj_file"]
    assert f.size == gni[0] * gni[1]
    assert np.array_equal(bits(r["grid"].ravel()), bits(f))
    sizes = w[f"{name}_{tag}_proj_block_sizes"]
    ref_blocks = w[f"{name}_{tag}_proj_blocks"]
    assert np.array_equal(bits(r["block_concat"][:sizes.sum()]), bits(ref_blocks))
    st = w[f"{name}_{tag}_proj_stats"]
    assert (r["max_dense"], r["tot_mass"], r["check_mass"]) == (st[0], st[1], st[2])


def test_project_helpers(oracle):
    """z layers from block starts, and the float32 z-projection order."""
    zl, n = oracle.z_layers([0, 20, 20, 0], 40)
    assert n == 2 and zl[19] == 0 and zl[20] == 1 and zl[-1] == 1
    zl1, n1 = oracle.z_layers([5], 8)
    assert n1 == 1 and not zl1.any()
    g = np.arange(2 * 3 * 4, dtype=np.float32).reshape(2, 3, 4)
    lay = oracle.project_layers(g, np.array([0, 1], np.int32), 0.5)
    assert np.array_equal(lay[0], g[0] * np.float32(0.5)) and np.array_equal(lay[1], g[1] * np.float32(0.5))
    assert np.array_equal(oracle.sum_layers(lay), lay[0] + lay[1])


def test_side_of_plane_and_distance_pinned():
    """side_of_plane and distance of the restated oracle against the
    reference's own src/tet.cpp (oracle/_ref), on random and coplanar tets."""
    import os
    from oracle.oracle import REF_SO, Oracle, Restated
    if not os.path.exists(REF_SO):
        pytest.skip("reference build not present")
    R, O = Oracle("ref"), Restated()
    rng = np.random.default_rng(3)
    tet = np.array([0, 1, 2, 3, -1, -1, -1, -1], np.int32)
    for it in range(2000):
        P = rng.random((4, 3), dtype=np.float32)
        if it % 5 == 0:   # vertex 3 on the plane of 0, 1, 2 (up to rounding)
            w = rng.random(2).astype(np.float32)
            P[3] = P[0] + w[0] * (P[1] - P[0]) + w[1] * (P[2] - P[0])
        lo = (rng.random(3, dtype=np.float32) * 2 - 0.5).astype(np.float32)
        box = np.concatenate([lo, lo + rng.random(3, dtype=np.float32)]).astype(np.float32)
        for j in range(4):
            assert R.side_of_plane(box, tet, P, j) == O.side_of_plane(box, tet, P, j)
        assert R.distance(P[0], P[1]).view(np.uint32) == O.distance(P[0], P[1]).view(np.uint32)


def _incomplete_cells_loops(O, b, links6, wrap3, last):
    """incomplete_cells (src/tess.cpp:492-628) once more, in Python loops over
    the oracle's pinned primitives, as an independent check of the C oracle's
    control flow."""
    f32 = np.float32
    norig = int(b["num_orig"])
    P, T = b["particles"], b["tets"]
    ext = (b["data_max"] - b["data_min"]).astype(f32)
    boxes = []
    for i, l6 in enumerate(links6):
        w = wrap3[i] if wrap3 is not None else np.zeros(3, np.int32)
        sh = np.array([f32(w[d]) * ext[d] for d in range(3)], f32)
        boxes.append(np.concatenate([(l6[:3] + sh).astype(f32), (l6[3:] + sh).astype(f32)]))
    cc = O.fill_circumcenters(P, T)
    masks = [0] * norig
    for t in range(len(T)):
        verts, nbrs = T[t, :4], T[t, 4:]
        if not any(v < norig for v in verts):
            continue
        c = cc[t]
        rad = O.distance(c, P[verts[0]])
        for j in range(4):
            if nbrs[j] != -1 or not any(verts[k] < norig for k in range(4) if k != j):
                continue
            for i in range(last, len(boxes)):
                if O.side_of_plane(boxes[i], T[t], P, j):
                    for k in range(4):
                        if k != j and verts[k] < norig:
                            masks[verts[k]] |= 1 << i
        deep = all(c[d] - b["bounds_min"][d] > rad and b["bounds_max"][d] - c[d] > rad for d in range(3))
        if deep:
            continue
        for i in range(last, len(boxes)):
            if O.box_distance(boxes[i], c) <= rad:
                for v in verts:
                    if v < norig:
                        masks[v] |= 1 << i
    return np.array(masks, np.uint64)


@pytest.mark.parametrize("periodic", [False, True])
def test_incomplete_cells_restated_twice(oracle, periodic):
    from tess2_gb300 import host
    pts = host.mixture_particles(1200, 5, n_clumps=4, sigma=0.05)
    blocks = host.tessellate(host.decompose(pts, (2, 2, 2), 0.08), processes=1)
    b = blocks[5]
    links6 = np.array([np.concatenate([o["bounds_min"], o["bounds_max"]]) for k, o in enumerate(blocks) if k != 5],
                      np.float32)
    wrap3 = None
    if periodic:
        wrap3 = np.zeros((len(links6), 3), np.int32)
        wrap3[::2, 0] = 1
        wrap3[1::3, 2] = -1
    m, enq = oracle.incomplete_cells(b, links6, wrap3, last_neighbor=1)
    ref = _incomplete_cells_loops(oracle, b, links6, wrap3, 1)
    assert np.array_equal(m, ref)
    assert enq == sum(bin(int(x)).count("1") for x in m)
    assert enq > 0 and not (m & np.uint64(1)).any()   # link 0 is below last_neighbor


def test_incomplete_cells_without_tets(oracle):
    """A block with fewer than five particles has no tets: every original
    particle goes to every tested link."""
    p = np.random.default_rng(1).random((4, 3), dtype=np.float32)
    b = dict(particles=p, tets=np.zeros((0, 8), np.int32), vert_to_tet=np.full(4, -1, np.int32), num_orig=3,
             bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
             data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))
    links6 = np.tile(np.array([0, 0, 0, 1, 1, 1], np.float32), (5, 1))
    m, enq = oracle.incomplete_cells(b, links6, last_neighbor=2)
    assert list(m) == [0b11100] * 3 and enq == 9


def _shifted_blocks(given):
    """2x1x2 blocks over an anisotropic, offset domain, for the given-bounds path."""
    from tess2_gb300 import host
    p = host.mixture_particles(3000, 17, n_clumps=6, sigma=0.05)
    scale = np.array([8.0, 1.0, 2.0], np.float32)
    off = np.array([-3.0, 10.0, 0.0], np.float32)
    pts = (p * scale + off).astype(np.float32)
    blocks = host.tessellate(host.decompose(pts, (2, 1, 2), 0.4, domain_min=off, domain_max=off + scale),
                             processes=1)
    # grid sizes and given bounds are chosen so that no grid point lies on the
    # blocks' shared faces (x = 1, z = 1): there the reference's inclusive
    # bounds test and its trimmed block boxes disagree (src/dense.cpp:279-284
    # against :615-626) and its deposit lands outside the block's array
    g = (off - np.array([0.3, 0.1, 0.35], np.float32), off + scale + np.array([0.5, 0.05, 0.2], np.float32)) \
        if given else None
    return blocks, g


@pytest.mark.parametrize("given", [False, True])
@pytest.mark.parametrize("alg", [0, 1])
def test_offset_domain_matches_reference(oracle, given, alg):
    """GridStepParams' cube-ified bounds (anisotropic, offset domain) and the
    given-bounds override: the restated oracle against the reference build."""
    import os
    from oracle.oracle import REF_SO, Oracle
    if not os.path.exists(REF_SO):
        pytest.skip("reference build not present")
    blocks, g = _shifted_blocks(given)
    gni = [36, 23, 28]
    r = oracle.dense(alg, blocks, gni, given=g)
    ref = Oracle("ref").dense(alg, blocks, gni, given=g)
    # deposits at grid points outside every block's bounds are dropped by both
    # (the cube-ified grid reaches past the data in y)
    assert np.array_equal(bits(r["grid"]), bits(ref["grid"]))
    assert np.array_equal(r["grid_step"], ref["grid_step"]) and np.array_equal(r["grid_min"], ref["grid_min"])
    assert r["grid"].sum() > 0


def test_sampled_parity_helpers_against_full_oracle(oracle):
    """oracle/parity.py: the sampled DTFE (every 4th tet) agrees with the full
    FP64 oracle's owners restricted to those tets, and the cell-list DENSE_TESS
    gives the reference's golden per-cell counts."""
    from conftest import load_blocks, load_single, single_block
    from oracle import parity
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    full = oracle.dtfe(blocks, gni)
    smp = parity.dtfe_oracle_sample(blocks, gni, 4, processes=1)
    r = parity.dtfe_compare(full["grid"].ravel(), full["owner"].ravel(), smp, 4)
    assert r["points"] > 0 and r["owners_equal"] and r["no_extra"] and r["rel_l2"] == 0.0
    s = load_single("mix2048_seed7")
    blk = single_block(s)
    cells = parity.tess_cell_sample(blk, 500, seed=3)
    cnt = parity.tess_counts_oracle(blk, [int(x) for x in s["glo_num_idx"]], cells, processes=1)
    assert np.array_equal(cnt[0], s["tess_cell_counts"][cells[0]])
