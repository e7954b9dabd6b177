"""The surrogate's kernels against the FP64 CPU oracle (oracle/surrogate_oracle.py),
and a short training run on fields the plain DTFE path makes."""
import numpy as np
import pytest

from conftest import rel_l2


def _bf16(a):
    """float32 values exactly representable in bf16 (round to nearest even)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def test_oracle_gradients_finite_differences():
    """The oracle's data and weight gradients against finite differences."""
    from oracle.surrogate_oracle import conv3d, conv3d_dgrad, conv3d_wgrad
    rng = np.random.default_rng(0)
    x = rng.standard_normal((3, 4, 5, 2))
    w = rng.standard_normal((27, 3, 2))
    b = rng.standard_normal(3)
    dy = rng.standard_normal((3, 4, 5, 3))
    f = lambda xx, ww, bb: float((dy * conv3d(xx, ww, bb)).sum())
    dx = conv3d_dgrad(dy, w)
    dw, db = conv3d_wgrad(x, dy)
    h = 1e-6
    for idx in [(0, 0, 0, 0), (1, 2, 3, 1), (2, 3, 4, 0)]:
        e = np.zeros_like(x); e[idx] = h
        assert abs((f(x + e, w, b) - f(x - e, w, b)) / (2 * h) - dx[idx]) < 1e-6
    for idx in [(0, 0, 0), (13, 2, 1), (26, 1, 0)]:
        e = np.zeros_like(w); e[idx] = h
        assert abs((f(x, w + e, b) - f(x, w - e, b)) / (2 * h) - dw[idx]) < 1e-6
    e = np.zeros_like(b); e[1] = h
    assert abs((f(x, w, b + e) - f(x, w, b - e)) / (2 * h) - db[1]) < 1e-6


def test_planar_layout_helpers():
    """to_planar / from_planar: channel c of voxel v at [c // 8, v, c % 8], and back."""
    from tess2_gb300 import surrogate as S
    a = np.arange(5 * 32).reshape(5, 32)
    p = S.to_planar(a)
    assert p.shape == S.planar_shape(5, 32) == (4, 5, 8)
    for v in range(5):
        for c in range(32):
            assert p[c // 8, v, c % 8] == a[v, c]
    assert np.array_equal(S.from_planar(p), a)


def _slab(x, x0, y, z, n):
    """Positions x0 - 1 .. x0 - 2 + n of input row (y, z), zero outside the grid (x: Z, Y, X, C)."""
    Z, Y, X, C = x.shape
    out = np.zeros((n, C))
    if 0 <= y < Y and 0 <= z < Z:
        lo, hi = max(x0 - 1, 0), min(x0 - 1 + n, X)
        if hi > lo:
            out[lo - (x0 - 1):hi - (x0 - 1)] = x[z, y, lo:hi]
    return out


@pytest.mark.parametrize("shape", [(3, 6, 16), (2, 5, 140), (1, 1, 16)])
def test_tcgen05_forward_decomposition(shape):
    """The tcgen05 forward's decomposition, restated on the CPU: groups of four
    tiles of 128 voxels on consecutive y rows; per dz the group's rows
    y0 - 1 .. y0 + Tg are one slab each; tile t, tap (dz, dy, dx) reads slab
    row t + dy + 1 from position dx + 1 on.  Equals the FP64 convolution."""
    from oracle.surrogate_oracle import conv3d
    rng = np.random.default_rng(11)
    x = rng.standard_normal(shape + (16,))
    w = rng.standard_normal((27, 8, 16))
    Z, Y, X = shape
    y = np.full((Z, Y, X, 8), np.nan)
    per_row, T = (X + 127) // 128, 4
    for q in range(per_row * ((Y + T - 1) // T) * Z):
        xt, yb, z = q % per_row, (q // per_row) % ((Y + T - 1) // T), q // (per_row * ((Y + T - 1) // T))
        Tg, x0, y0 = min(T, Y - yb * T), xt * 128, yb * T
        slabs = {(dz, rho): _slab(x, x0, y0 - 1 + rho, z + dz, 130) for dz in (-1, 0, 1) for rho in range(Tg + 2)}
        for t in range(Tg):
            acc = np.zeros((128, 8))
            for g in range(9):
                dz, dy = g // 3 - 1, g % 3 - 1
                for sh in range(3):
                    acc += slabs[(dz, t + dy + 1)][sh:sh + 128] @ w[g * 3 + sh].T
            n = min(128, X - x0)
            y[z, y0 + t, x0:x0 + n] = acc[:n]
    assert np.abs(y - conv3d(x, w)).max() < 1e-9


@pytest.mark.parametrize("shape", [(3, 4, 16), (2, 3, 140)])
def test_tcgen05_wgrad_decomposition(shape):
    """The tcgen05 weight gradient's decomposition, restated on the CPU: one
    accumulator per tap of a dz, D[co][ci] += dyT^T slab[r + dx + 1] over the
    tiles of 128 voxels (dy zero past X).  Equals the FP64 weight gradient."""
    from oracle.surrogate_oracle import conv3d_wgrad
    rng = np.random.default_rng(12)
    x = rng.standard_normal(shape + (16,))
    dyv = rng.standard_normal(shape + (8,))
    Z, Y, X = shape
    dw = np.zeros((27, 8, 16))
    per_row = (X + 127) // 128
    for dz in (-1, 0, 1):
        for t in range(per_row * Y * Z):
            r = t // per_row
            x0, yy, zz = (t % per_row) * 128, r % Y, r // Y
            A = np.zeros((128, 8))
            n = min(128, X - x0)
            A[:n] = dyv[zz, yy, x0:x0 + n]
            for d in range(3):
                slab = _slab(x, x0, yy + d - 1, zz + dz, 130)
                for sh in range(3):
                    dw[(dz + 1) * 9 + d * 3 + sh] += A.T @ slab[sh:sh + 128]
    ref, _ = conv3d_wgrad(x, dyv)
    assert np.abs(dw - ref).max() < 1e-9


@pytest.fixture
def engine(request):
    from tess2_gb300 import surrogate as S
    S.set_engine(request.param)
    yield request.param
    S.check()
    S.set_engine(S.ENGINE_TCGEN05)


# shapes: tiles of 128 x-padded positions that cross x rows; a ragged last
# tile; a grid smaller than one tile
SHAPES = [(5, 6, 32), (3, 7, 48), (1, 2, 16)]


@pytest.mark.gpu
@pytest.mark.parametrize("engine", [0, 1], ids=["tcgen05", "mma_sync"], indirect=True)
@pytest.mark.parametrize("shape", SHAPES, ids=["5x6x32", "3x7x48", "1x2x16"])
@pytest.mark.parametrize("cin,cout", [(16, 16), (16, 32), (32, 16), (32, 32)])
def test_conv3d_kernels_vs_oracle(gpu_ctx, engine, shape, cin, cout):
    import torch
    from oracle.surrogate_oracle import conv3d, conv3d_dgrad, conv3d_wgrad
    from tess2_gb300 import surrogate as S
    rng = np.random.default_rng(cin * 100 + cout)
    Z, Y, X = shape
    x = _bf16(rng.standard_normal((Z, Y, X, cin)).astype(np.float32))
    w = (rng.standard_normal((27, cout, cin)) * 0.2).astype(np.float32)
    wq = _bf16(w)
    b = rng.standard_normal(cout).astype(np.float32)
    dy = _bf16(rng.standard_normal((Z, Y, X, cout)).astype(np.float32))
    dev = "cuda:0"
    V = Z * Y * X
    # the kernels' chunk-planar layout; the oracle's is channels-last
    tx = torch.from_numpy(S.to_planar(x.reshape(V, cin))).to(dev).to(torch.bfloat16)
    tw = torch.from_numpy(w).to(dev)
    wb = torch.empty((27, cout, cin), dtype=torch.bfloat16, device=dev)
    wt = torch.empty((27, cin, cout), dtype=torch.bfloat16, device=dev)
    S.prepare_weights(tw, cout, cin, wb, wt)
    tb = torch.from_numpy(b).to(dev)
    y32 = torch.empty(S.planar_shape(V, cout), device=dev)
    S.conv3d_fwd(tx, (Z, Y, X), cin, cout, wb, tb, relu=False, y_f32=y32)
    ref = conv3d(x, wq, b)
    torch.cuda.synchronize()
    assert rel_l2(S.from_planar(y32.cpu().numpy()), ref.reshape(-1, cout)) < 1e-5
    # relu and bf16 output
    yb = torch.empty(S.planar_shape(V, cout), dtype=torch.bfloat16, device=dev)
    S.conv3d_fwd(tx, (Z, Y, X), cin, cout, wb, tb, relu=True, y_bf16=yb)
    assert rel_l2(S.from_planar(yb.float().cpu().numpy()), np.maximum(ref, 0).reshape(-1, cout)) < 1e-2
    # data gradient through the flipped weights
    tdy = torch.from_numpy(S.to_planar(dy.reshape(V, cout))).to(dev).to(torch.bfloat16)
    dx = torch.empty(S.planar_shape(V, cin), device=dev)
    S.conv3d_fwd(tdy, (Z, Y, X), cout, cin, wt, None, relu=False, y_f32=dx)
    assert rel_l2(S.from_planar(dx.cpu().numpy()), conv3d_dgrad(dy, wq).reshape(-1, cin)) < 1e-5
    # weight and bias gradient
    dw = torch.zeros((27, cout, cin), device=dev)
    db = torch.zeros(cout, device=dev)
    S.conv3d_wgrad(tx, tdy, (Z, Y, X), cin, cout, dw, db)
    rdw, rdb = conv3d_wgrad(x, dy)
    torch.cuda.synchronize()
    assert rel_l2(dw.cpu().numpy(), rdw) < 1e-5
    assert rel_l2(db.cpu().numpy(), rdb) < 1e-5
    S.check()


@pytest.mark.gpu
def test_conv3d_engines_agree_large(gpu_ctx):
    """tcgen05 and mma.sync on a 64 x 48 x 80 grid, 32 -> 32 channels: the same
    bf16 products, FP32 sums in another order."""
    import torch
    from tess2_gb300 import surrogate as S
    Z, Y, X, c = 64, 48, 80, 32
    g = torch.Generator(device="cuda:0").manual_seed(7)
    x = torch.randn(S.planar_shape(Z * Y * X, c), device="cuda:0", generator=g).to(torch.bfloat16)
    w = torch.randn((27, c, c), device="cuda:0", generator=g) * 0.1
    wb = torch.empty((27, c, c), dtype=torch.bfloat16, device="cuda:0")
    wt = torch.empty_like(wb)
    S.prepare_weights(w, c, c, wb, wt)
    b = torch.randn(c, device="cuda:0", generator=g)
    out = {}
    for e in (S.ENGINE_TCGEN05, S.ENGINE_MMA_SYNC):
        S.set_engine(e)
        y = torch.full(S.planar_shape(Z * Y * X, c), float("nan"), device="cuda:0")
        S.conv3d_fwd(x, (Z, Y, X), c, c, wb, b, relu=True, y_f32=y)
        out[e] = y
    S.set_engine(S.ENGINE_TCGEN05)
    S.check()
    a, m = out[S.ENGINE_TCGEN05], out[S.ENGINE_MMA_SYNC]
    assert torch.isfinite(a).all()
    assert float((a - m).abs().max()) < 1e-4 * float(m.abs().max())


@pytest.mark.gpu
def test_forward_graph_matches_forward(gpu_ctx):
    """The CUDA-graph replay gives the eager forward's output bit for bit, and
    sees weights updated in place after the capture."""
    import torch
    from tess2_gb300 import surrogate as S
    net = S.Surrogate((16, 12, 32), seed=4)
    g = torch.Generator(device="cuda:0").manual_seed(5)
    x1 = torch.rand(16 * 12 * 32, device="cuda:0", generator=g)
    x2 = torch.rand(16 * 12 * 32, device="cuda:0", generator=g)
    eager = net.forward(x1).clone()
    assert torch.equal(net.forward_graph(x1).clone(), eager)
    assert torch.equal(net.forward_graph(x2).clone(), net.forward(x2).clone())
    net.train_step(x1, x2, lr=1e-2)   # new weights, same buffers
    assert torch.equal(net.forward_graph(x1).clone(), net.forward(x1).clone())
    S.check()


@pytest.mark.gpu
def test_surrogate_learns(gpu_ctx):
    """A few Adam steps on a handful of small fields lower the loss, and the
    trained network beats its own input (the CIC grid) against DTFE on the
    training fields."""
    import torch
    from tess2_gb300 import surrogate as S
    fields = S.make_fields(gpu_ctx, range(5), 20000, 32, processes=1)
    net = S.Surrogate((32, 32, 32), seed=1)
    t = [(torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()) for x, y in fields]
    first = np.mean([net.train_step(x, y, lr=3e-3) for x, y in t])
    for _ in range(30):
        last = np.mean([net.train_step(x, y, lr=3e-3) for x, y in t])
    assert last < 0.7 * first
    err = np.mean([S.rel_l2(net.forward(x).cpu().numpy(), y.cpu().numpy()) for x, y in t])
    base = np.mean([S.rel_l2(x.cpu().numpy(), y.cpu().numpy()) for x, y in t])
    assert err < base
