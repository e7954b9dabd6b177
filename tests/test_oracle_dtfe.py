"""The FP64 DTFE oracle and its exact predicates.

Parity for DTFE is anchored here, since the reference has no DTFE: the
orientation predicate against exact rational arithmetic (fractions), the
point-to-tet assignment against a brute-force exact search, and the field
against known answers (mass conservation, vertex values, linear interpolation).
"""
from fractions import Fraction

import numpy as np
import pytest

from conftest import load_single, single_block


def orient_fraction(a, b, c, d):
    A = [Fraction(float(x)) for x in a]
    B = [Fraction(float(x)) for x in b]
    C = [Fraction(float(x)) for x in c]
    D = [Fraction(float(x)) for x in d]
    u = [B[i] - A[i] for i in range(3)]
    v = [C[i] - A[i] for i in range(3)]
    w = [D[i] - A[i] for i in range(3)]
    det = (u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) +
           u[2] * (v[0] * w[1] - v[1] * w[0]))
    return (det > 0) - (det < 0)


def test_orient_exact_random(oracle):
    rng = np.random.default_rng(5)
    for _ in range(300):
        p = rng.random((4, 3), dtype=np.float32)
        assert oracle.orient3d_exact(*p) == orient_fraction(*p)


def test_orient_exact_near_degenerate(oracle):
    """Points nudged off a plane by one ulp: double evaluation is unreliable
    here, the exact predicate is not."""
    rng = np.random.default_rng(6)
    for _ in range(300):
        a, b, c = rng.random((3, 3), dtype=np.float32)
        s, t = rng.random(2)
        d = (a + np.float32(s) * (b - a) + np.float32(t) * (c - a)).astype(np.float32)
        d = np.nextafter(d, d + rng.choice([-1, 1], 3).astype(np.float32))
        assert oracle.orient3d_exact(a, b, c, d) == orient_fraction(a, b, c, d)
        assert oracle.orient3d_exact(a, b, c, a) == 0


def test_orient_exact_wide_exponents(oracle):
    rng = np.random.default_rng(7)
    for _ in range(200):
        p = (rng.random((4, 3)) * 10.0 ** rng.integers(-30, 5, (4, 3))).astype(np.float32)
        assert oracle.orient3d_exact(*p) == orient_fraction(*p)


def test_assignment_is_exact_partition(oracle):
    """Every grid point inside the hull belongs to exactly one tet, found by
    brute force with the exact predicate; grid points on shared faces, edges
    and vertices of a regular lattice exercise the perturbation tie-break."""
    from tess2_gb300 import host
    # lattice points coincide with grid points: every tie case occurs
    g = np.arange(4, dtype=np.float32) / 3
    lat = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    jit = host.uniform_particles(30, 3) * np.float32(0.9) + np.float32(0.05)
    for pts in (lat, np.concatenate([lat, jit])):
        tets = host.delaunay_tets(pts)
        v2t = host.vert_to_tet_host(len(pts), tets)
        blk = [dict(gid=0, particles=pts, tets=tets, vert_to_tet=v2t, num_orig=len(pts),
                    bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
                    data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))]
        r = oracle.dtfe(blk, [10, 10, 10])
        step = r["grid_step"]
        owner = r["owner"]
        for z in range(10):
            for y in range(10):
                for x in range(10):
                    p = (np.arange(3) * 0 + np.array([x, y, z])).astype(np.int32)
                    pos = np.array([np.float32(p[i]) * step[i] + r["grid_min"][i] for i in range(3)], np.float32)
                    hits = [t for t in range(len(tets)) if oracle.tet_contains(pts, tets[t], pos)]
                    assert len(hits) <= 1
                    assert owner[z, y, x] == (hits[0] if hits else -1)
                    # the convex hull is the unit cube; the perturbation moves points on
                    # its upper faces (coordinate 1.0) outside, every other point is owned
                    if max(x, y, z) < 9:
                        assert hits


def test_dtfe_known_answers(oracle):
    d = load_single("c1_uniform4096_seed1")
    r = oracle.dtfe(single_block(d), [64, 64, 64])
    p = d["particles"].astype(np.float64)
    t = d["tets"][:, :4]
    V = np.abs(np.linalg.det(p[t[:, 1:]] - p[t[:, :1]])) / 6
    # star volumes: rho_v = 4 m / sum of incident tet volumes
    W = np.zeros(len(p))
    np.add.at(W, t.ravel(), np.repeat(V, 4))
    assert np.allclose(r["rho"], 4.0 / W, rtol=1e-12)
    # the linear field integrates to the total mass exactly
    assert np.isclose((V * r["rho"][t].mean(axis=1)).sum(), len(p), rtol=1e-12)
    # every grid point is owned by at most one tet and holds its interpolated value
    own = r["owner"]
    assert r["assigned"] == np.count_nonzero(own >= 0)
    assert np.all(r["grid"][own < 0] == 0)
    rng = np.random.default_rng(1)
    idx = np.argwhere(own >= 0)
    for z, y, x in idx[rng.choice(len(idx), 50, replace=False)]:
        tt = t[own[z, y, x]]
        q = np.array([x, y, z], np.float32) * r["grid_step"] + r["grid_min"]
        A = np.vstack([p[tt].T, np.ones(4)])
        lam = np.linalg.solve(A, np.append(q.astype(np.float64), 1.0))
        assert np.all(lam >= -1e-9)
        assert np.isclose(r["grid"][z, y, x], lam @ r["rho"][tt], rtol=1e-6)
