"""The U-Net surrogate's kernels (tessgpu_unet_*) against the FP64 CPU oracle
(oracle/unet_oracle.py), the oracle's own backward pass against finite
differences, and the whole network's forward pass and parameter gradients."""
import numpy as np
import pytest

from conftest import rel_l2


def _bf16(a):
    """float32 values exactly representable in bf16 (round to nearest even)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def _planar(a):
    """(Z, Y, X, C) -> (C / 8, V, 8) chunk-planar"""
    Z, Y, X, C = a.shape
    return np.ascontiguousarray(np.asarray(a).reshape(-1, C // 8, 8).transpose(1, 0, 2))


def _unplanar(p, grid):
    X, Y, Z = grid
    p = np.asarray(p)
    return p.transpose(1, 0, 2).reshape(Z, Y, X, -1)


def _rand_params(seed, head_scale=0.1):
    from oracle.unet_oracle import CONVS, HEAD_C
    rng = np.random.default_rng(seed)
    parts = []
    for name, ci, co, _ in CONVS:
        fan = 27 * (1 if name == "e0a" else ci)
        w = rng.standard_normal((27, co, ci)) * np.sqrt(2.0 / fan)
        if name == "e0a":
            w[:, :, 1:] = 0.0
        parts += [w.ravel(), 0.05 * rng.standard_normal(co)]
    parts += [head_scale * rng.standard_normal(HEAD_C), [0.02]]
    return np.concatenate(parts).astype(np.float32)


def test_unet_oracle_gradients_finite_differences():
    """The oracle's hand-written backward pass against central differences (FP64, 8^3 grid)."""
    from oracle import unet_oracle as U
    rng = np.random.default_rng(3)
    flat = _rand_params(4, head_scale=0.3).astype(np.float64)
    field = rng.standard_normal((8, 8, 8))
    target = rng.standard_normal((8, 8, 8))
    P = U.split_params(flat)
    g = U.flat_grads(U.backward(P, U.forward(P, field), target))
    h = 1e-5
    # entries of every layer: its first weight that sees a nonzero input, a bias, the head
    picks = []
    off = 0
    for name, ci, co, _ in U.CONVS:
        picks += [off + 13 * co * ci + 5 * ci % (co * ci), off + 27 * co * ci + 1]
        off += 27 * co * ci + co
    picks += [off + 3, off + U.HEAD_C]
    for i in picks:
        e = np.zeros_like(flat)
        e[i] = h
        fd = (U.loss(U.split_params(flat + e), field, target) - U.loss(U.split_params(flat - e), field, target)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_unet_oracle_pool_upsample_adjoint():
    """<pool x, y> = <x, pool_grad y> and <up x, y> = <x, up_grad y>."""
    from oracle import unet_oracle as U
    rng = np.random.default_rng(1)
    x = rng.standard_normal((4, 6, 8, 3))
    y = rng.standard_normal((2, 3, 4, 3))
    assert abs((U.pool(x) * y).sum() - (x * U.pool_grad(y)).sum()) < 1e-10
    assert abs((U.upsample(y) * x).sum() - (y * U.upsample_grad(x)).sum()) < 1e-10


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _dev(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0").to(dtype)


CONV_CASES = [
    ((128, 4, 3), 16, 32), ((128, 4, 3), 32, 96), ((128, 2, 2), 96, 32), ((128, 2, 2), 32, 256),
    ((64, 4, 4), 32, 64), ((64, 4, 2), 192, 64), ((64, 2, 2), 64, 192),
    ((32, 8, 4), 64, 128), ((32, 4, 2), 384, 128), ((32, 4, 2), 128, 384),
    ((16, 8, 8), 128, 256), ((16, 8, 4), 256, 128),
]


@pytest.mark.gpu
@pytest.mark.parametrize("grid,cin,cout", CONV_CASES)
def test_unet_conv_matches_oracle(grid, cin, cout):
    """Forward convolution (bias, ReLU, output at a plane offset) and the masked
    form, against the FP64 oracle on bf16 inputs and weights."""
    import torch
    from oracle.surrogate_oracle import conv3d
    from tess2_gb300 import unet as U
    X, Y, Z = grid
    V = X * Y * Z
    rng = np.random.default_rng(cin * 1000 + cout + X)
    x = _bf16(rng.standard_normal((Z, Y, X, cin)))
    w = (rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin)).astype(np.float32)
    b = rng.standard_normal(cout).astype(np.float32)
    wd = _dev(w, torch.float32)
    wf = torch.empty(27 * cout * cin, dtype=torch.bfloat16, device="cuda:0")
    wb = torch.empty_like(wf)
    U.pack_weights(wd, cout, cin, wf, wb)
    xd = _dev(_planar(x), torch.bfloat16)
    y = torch.zeros((cout // 8 + 2, V, 8), dtype=torch.bfloat16, device="cuda:0")
    U.conv(xd, grid, cin, wf, cout, y, 2, bias=_dev(b, torch.float32), relu=True)
    mask = _bf16(rng.standard_normal((Z, Y, X, cout)))
    ym = torch.zeros((cout // 8, V, 8), dtype=torch.bfloat16, device="cuda:0")
    U.conv(xd, grid, cin, wf, cout, ym, 0, mask=_dev(_planar(mask), torch.bfloat16))
    U.check()
    yh = y.float().cpu().numpy()
    assert not yh[:2].any(), "planes before y_plane0 written"
    wq = _bf16(w)
    ref = conv3d(x, wq, b, relu=True)
    got = _unplanar(yh[2:], grid)
    assert rel_l2(got, ref) < 4e-3
    refm = conv3d(x, wq) * (mask > 0)
    assert rel_l2(_unplanar(ym.float().cpu().numpy(), grid), refm) < 4e-3


@pytest.mark.gpu
@pytest.mark.parametrize("grid,cin,cout", [((128, 4, 3), 16, 32), ((128, 2, 2), 96, 64), ((64, 4, 2), 192, 64),
                                           ((32, 8, 4), 64, 32)])
def test_unet_conv_tiles_per_item_same_bits(grid, cin, cout):
    """Several tiles per item (one MMA warp each, sharing the weights' stage)
    give the same bits as one tile per item (TESSGPU_UNET_TILES=1)."""
    import os
    import torch
    from tess2_gb300 import unet as U
    X, Y, Z = grid
    V = X * Y * Z
    rng = np.random.default_rng(cin + 3 * cout)
    x = _dev(_planar(_bf16(rng.standard_normal((Z, Y, X, cin)))), torch.bfloat16)
    w = _dev((rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin)).astype(np.float32), torch.float32)
    wf = torch.empty(27 * cout * cin, dtype=torch.bfloat16, device="cuda:0")
    wb = torch.empty_like(wf)
    U.pack_weights(w, cout, cin, wf, wb)
    out = []
    for tiles in (None, "1"):
        if tiles:
            os.environ["TESSGPU_UNET_TILES"] = tiles
        try:
            y = torch.zeros((cout // 8, V, 8), dtype=torch.bfloat16, device="cuda:0")
            U.conv(x, grid, cin, wf, cout, y, relu=True)
            U.check()
            out.append(y.view(torch.int16).cpu().numpy())
        finally:
            os.environ.pop("TESSGPU_UNET_TILES", None)
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
@pytest.mark.parametrize("grid,cin,cout", [((128, 4, 3), 32, 96), ((64, 4, 2), 64, 192), ((32, 4, 2), 128, 384),
                                           ((16, 8, 4), 256, 128)])
def test_unet_data_gradient_matches_oracle(grid, cin, cout):
    """The data gradient: the convolution with the packed data-gradient weights."""
    import torch
    from oracle.surrogate_oracle import conv3d_dgrad
    from tess2_gb300 import unet as U
    X, Y, Z = grid
    rng = np.random.default_rng(cin + cout)
    w = (rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cout)).astype(np.float32)
    dy = _bf16(rng.standard_normal((Z, Y, X, cout)))
    wf = torch.empty(27 * cout * cin, dtype=torch.bfloat16, device="cuda:0")
    wb = torch.empty_like(wf)
    U.pack_weights(_dev(w, torch.float32), cout, cin, wf, wb)
    dx = torch.zeros((cin // 8, X * Y * Z, 8), dtype=torch.bfloat16, device="cuda:0")
    U.conv(_dev(_planar(dy), torch.bfloat16), grid, cout, wb, cin, dx)
    U.check()
    ref = conv3d_dgrad(dy, _bf16(w))
    assert rel_l2(_unplanar(dx.float().cpu().numpy(), grid), ref) < 4e-3


@pytest.mark.gpu
@pytest.mark.parametrize("grid,cin,cout", [((128, 4, 3), 16, 32), ((128, 4, 3), 96, 32), ((128, 2, 2), 32, 96),
                                           ((64, 4, 4), 192, 64), ((32, 4, 2), 384, 128), ((16, 8, 8), 128, 256),
                                           ((32, 8, 4), 64, 16), ((16, 8, 8), 32, 64), ((128, 2, 2), 128, 128),
                                           ((64, 4, 2), 32, 32), ((64, 2, 2), 64, 128), ((64, 2, 2), 16, 16)])
def test_unet_wgrad_matches_oracle(grid, cin, cout):
    """Weight and bias gradients (FP32 sums of bf16 products): slab grids (X a
    multiple of 128, or X = 64 with two rows a tile) with 1, 2, 4 or 8 (dz, dy)
    pairs stacked in M, and the per-tap form for X of 16 or 32."""
    import torch
    from oracle.surrogate_oracle import conv3d_wgrad
    from tess2_gb300 import unet as U
    X, Y, Z = grid
    rng = np.random.default_rng(7 * cin + cout)
    x = _bf16(rng.standard_normal((Z, Y, X, cin)))
    dy = _bf16(rng.standard_normal((Z, Y, X, cout)))
    dw = torch.zeros((27, cout, cin), device="cuda:0")
    db = torch.zeros(cout, device="cuda:0")
    U.wgrad(_dev(_planar(x), torch.bfloat16), _dev(_planar(dy), torch.bfloat16), grid, cin, cout, dw, db)
    U.check()
    rdw, rdb = conv3d_wgrad(x, dy)
    assert rel_l2(dw.cpu().numpy(), rdw) < 1e-5
    assert rel_l2(db.cpu().numpy(), rdb) < 1e-5


@pytest.mark.gpu
def test_unet_pool_upsample_head_match_oracle():
    """Pooling, upsampling into a concatenation, their gradients, the head and its gradient."""
    import ctypes
    import torch
    from oracle import unet_oracle as O
    from tess2_gb300 import unet as U
    L = U._lib()
    s = U._stream()
    X, Y, Z, C = 16, 8, 4, 16
    V = X * Y * Z
    rng = np.random.default_rng(5)
    x = _bf16(rng.standard_normal((Z, Y, X, C)))
    xd = _dev(_planar(x), torch.bfloat16)
    p = torch.zeros((C // 8, V // 8, 8), dtype=torch.bfloat16, device="cuda:0")
    assert L.tessgpu_unet_pool(U._ptr(xd), X, Y, Z, C, U._ptr(p), s) == 0
    assert rel_l2(_unplanar(p.float().cpu().numpy(), (X // 2, Y // 2, Z // 2)), O.pool(x)) < 4e-3
    # upsample into planes 1.. of a buffer
    c = _bf16(rng.standard_normal((Z // 2, Y // 2, X // 2, C)))
    up = torch.zeros((C // 8 + 1, V, 8), dtype=torch.bfloat16, device="cuda:0")
    assert L.tessgpu_unet_upsample(U._ptr(_dev(_planar(c), torch.bfloat16)), X, Y, Z, C, U._ptr(up), 1, s) == 0
    uh = up.float().cpu().numpy()
    assert not uh[0].any()
    assert np.array_equal(_unplanar(uh[1:], (X, Y, Z)), O.upsample(c))
    # upsample gradient from planes 1.. of a gradient buffer
    g = _bf16(rng.standard_normal((Z, Y, X, C)))
    gbuf = np.zeros((C // 8 + 1, V, 8), np.float32)
    gbuf[1:] = _planar(g)
    ug = torch.zeros((C // 8, V // 8, 8), dtype=torch.bfloat16, device="cuda:0")
    assert L.tessgpu_unet_upsample_grad(U._ptr(_dev(gbuf, torch.bfloat16)), 1, X, Y, Z, C, U._ptr(ug), s) == 0
    assert rel_l2(_unplanar(ug.float().cpu().numpy(), (X // 2, Y // 2, Z // 2)), O.upsample_grad(g)) < 4e-3
    # pool gradient with a skip gradient (planes 1..) and the ReLU mask of the pooled activation
    act = _bf16(rng.standard_normal((Z, Y, X, C)))
    dp = _bf16(rng.standard_normal((Z // 2, Y // 2, X // 2, C)))
    pg = torch.zeros((C // 8, V, 8), dtype=torch.bfloat16, device="cuda:0")
    assert L.tessgpu_unet_pool_grad(U._ptr(_dev(_planar(dp), torch.bfloat16)), U._ptr(_dev(gbuf, torch.bfloat16)), 1,
                                    U._ptr(_dev(_planar(act), torch.bfloat16)), X, Y, Z, C, U._ptr(pg), s) == 0
    ref = (g + O.pool_grad(dp)) * (act > 0)
    assert rel_l2(_unplanar(pg.float().cpu().numpy(), (X, Y, Z)), ref) < 4e-3
    # head and its gradient (32 channels)
    Ch = 32
    a = np.maximum(_bf16(rng.standard_normal((Z, Y, X, Ch))), 0)
    wh = rng.standard_normal(Ch + 1).astype(np.float32)
    field = rng.standard_normal((Z, Y, X)).astype(np.float32)
    tgt = rng.standard_normal((Z, Y, X)).astype(np.float32)
    ad = _dev(_planar(a), torch.bfloat16)
    whd = _dev(wh, torch.float32)
    pred = torch.zeros(V, device="cuda:0")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    fd, td = _dev(field.ravel(), torch.float32), _dev(tgt.ravel(), torch.float32)
    assert L.tessgpu_unet_head(U._ptr(ad), Ch, U._ptr(whd), U._ptr(fd), V, U._ptr(pred), U._ptr(td), U._ptr(loss),
                               s) == 0
    rp = field.astype(np.float64) + a @ wh[:Ch].astype(np.float64) + wh[Ch]
    assert rel_l2(pred.cpu().numpy(), rp.ravel()) < 1e-6
    assert abs(loss.item() - ((rp - tgt) ** 2).sum()) < 1e-4 * ((rp - tgt) ** 2).sum()
    da = torch.zeros((Ch // 8, V, 8), dtype=torch.bfloat16, device="cuda:0")
    dwh = torch.zeros(Ch + 1, device="cuda:0")
    assert L.tessgpu_unet_head_grad(U._ptr(ad), Ch, U._ptr(whd), U._ptr(pred), U._ptr(td), V, ctypes.c_float(0.5),
                                    U._ptr(da), U._ptr(dwh), s) == 0
    gg = 2 * 0.5 * (pred.cpu().numpy().astype(np.float64).reshape(Z, Y, X) - tgt)
    rda = gg[..., None] * wh[:Ch] * (a > 0)
    assert rel_l2(_unplanar(da.float().cpu().numpy(), (X, Y, Z)), rda) < 4e-3
    rdw = np.concatenate([(a * gg[..., None]).reshape(-1, Ch).sum(0), [gg.sum()]])
    assert rel_l2(dwh.cpu().numpy(), rdw) < 1e-5


@pytest.mark.gpu
def test_unet_forward_and_gradients_match_oracle():
    """The whole U-Net on a 128 x 64 x 8 grid (levels down to 16 x 8 x 1): the
    network's part of the prediction and every parameter tensor's gradient
    against the FP64 oracle (bf16 activations and weights on the GPU)."""
    import torch
    from oracle import unet_oracle as O
    from tess2_gb300 import unet as U
    grid = (128, 64, 8)
    X, Y, Z = grid
    net = U.UNet(grid, seed=0)
    flat = _rand_params(11)
    net.params.copy_(torch.from_numpy(flat).cuda())
    net._pack()
    rng = np.random.default_rng(12)
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    field = (np.sin(xx / 7.0) * np.cos(yy / 5.0) + 0.3 * rng.standard_normal((Z, Y, X))).astype(np.float32)
    target = (np.tanh(field) + 0.1 * rng.standard_normal((Z, Y, X))).astype(np.float32)
    pred = net.forward(torch.from_numpy(field.ravel()).cuda(), torch.from_numpy(target.ravel()).cuda())
    net.backward()
    U.check()
    P = O.split_params(flat)
    A = O.forward(P, field)
    net_part = pred.cpu().numpy().reshape(Z, Y, X) - field
    assert rel_l2(net_part, A["pred"] - field) < 2e-2
    ref = O.flat_grads(O.backward(P, A, target))
    got = net.grads.cpu().numpy()
    for name, ci, co, _ in O.CONVS:
        a, b, c = net.slices[name]
        assert rel_l2(got[a:b], ref[a:b]) < 5e-2, name
        assert rel_l2(got[b:c], ref[b:c]) < 5e-2, name + " bias"
    a, _, c = net.slices["head"]
    assert rel_l2(got[a:c], ref[a:c]) < 2e-2


@pytest.mark.gpu
def test_unet_training_lowers_loss():
    """Twenty Adam steps on one field pair lower the loss."""
    import torch
    from tess2_gb300 import unet as U
    grid = (128, 64, 8)
    X, Y, Z = grid
    net = U.UNet(grid, seed=1)
    rng = np.random.default_rng(2)
    zz, yy, xx = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    field = (np.sin(xx / 9.0) + np.cos(yy / 6.0) + 0.2 * rng.standard_normal((Z, Y, X))).astype(np.float32)
    target = np.maximum(field, 0).astype(np.float32) * 1.5
    f, t = torch.from_numpy(field.ravel()).cuda(), torch.from_numpy(target.ravel()).cuda()
    losses = []
    for _ in range(20):
        net.loss.zero_()
        net.train_step(f, t, lr=3e-4)
        losses.append(net.loss.item())
    U.check()
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.5 * losses[0], losses


def _sym_particles(p, perm, flips):
    """particles under the symmetry that permute(perm) then flip(flips) applies to
    a (z, y, x) grid array of the unit cube: new axis a <- old axis 2 - perm[2 - a],
    mirrored when array dimension 2 - a is flipped"""
    q = np.empty_like(p)
    for a in range(3):
        c = p[:, 2 - perm[2 - a]]
        q[:, a] = 1.0 - c if (2 - a) in flips else c
    return q


@pytest.mark.parametrize("perm,flips", [([0, 1, 2], [0]), ([2, 1, 0], []), ([1, 2, 0], [1, 2]),
                                        ([0, 2, 1], [0, 1, 2])])
def test_moments_follow_cube_symmetries(perm, flips):
    """transform_moments (the training augmentation) on the moments of a particle
    set equals the moments of the transformed particles (FP64 oracle both ways)."""
    import torch
    from oracle.unet_oracle import cell_moments
    from tess2_gb300.unet import transform_moments
    S = 8
    rng = np.random.default_rng(3)
    p = rng.random((3000, 3))
    step = [1.0 / (S - 1)] * 3
    m = cell_moments(p, [0.0] * 3, step, [S] * 3)
    want = cell_moments(_sym_particles(p, perm, flips), [0.0] * 3, step, [S] * 3)
    got = transform_moments(torch.from_numpy(m.ravel()), S, perm, flips).view(10, S, S, S).numpy()
    assert np.allclose(got, want, atol=1e-9)


@pytest.mark.gpu
def test_unet_cell_moments_and_input_match_oracle():
    """tessgpu_unet_cell_moments (FP32 atomics) and tessgpu_unet_input_moments
    (bf16 channels) against the FP64 oracle on a clustered particle set."""
    import torch
    from oracle.unet_oracle import cell_moments, input_features
    from tess2_gb300 import host
    from tess2_gb300 import unet as U
    X, Y, Z = 16, 8, 12
    pts = host.mixture_particles(20000, 5).astype(np.float32)
    gmin, step = [0.01, -0.02, 0.0], [0.9 / (X - 1), 1.1 / (Y - 1), 1.0 / (Z - 1)]
    ref = cell_moments(pts, gmin, step, (X, Y, Z), f32=True)
    m = U.cell_moments(torch.from_numpy(pts).cuda(), gmin, step, (X, Y, Z))
    got = m.view(10, Z, Y, X).cpu().numpy()
    assert np.array_equal(got[0], ref[0])                       # counts exact
    assert np.allclose(got[1:], ref[1:], atol=2e-4 * max(1.0, ref[0].max()))
    field = np.random.default_rng(1).standard_normal((Z, Y, X)).astype(np.float32)
    x = torch.zeros(2 * X * Y * Z * 8, dtype=torch.bfloat16, device="cuda")
    L = U._lib()
    assert L.tessgpu_unet_input_moments(torch.from_numpy(field.ravel()).cuda().data_ptr(), m.data_ptr(), X * Y * Z,
                                        x.data_ptr(), None) == 0
    feats = _unplanar(x.float().cpu().numpy().reshape(2, X * Y * Z, 8), (X, Y, Z))
    want = input_features(field, ref)
    assert np.allclose(feats, want, rtol=1e-2, atol=2e-2)
    assert np.all(feats[..., 11:] == 0)
