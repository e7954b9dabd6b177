"""FP64 CPU oracle for the surrogate's U-Net.  TEST INFRASTRUCTURE ONLY:
tests/ use it to check the GPU's U-Net steps (convolutions of any channel
count, pooling, upsampling, head) and the whole network's forward pass and
parameter gradients.

Layout: activations (Z, Y, X, C), channel fastest; weights (27, c_out, c_in)
as in surrogate_oracle; the network and its parameter names as
tess2_gb300/unet.py (CONVS).  The backward pass is written out by hand and is
itself checked against central finite differences (tests/test_unet_oracle.py).
"""
import numpy as np

from oracle.surrogate_oracle import conv3d, conv3d_dgrad, conv3d_wgrad

CONVS = [
    ("e0a", 16, 32, 0), ("e0b", 32, 32, 0),
    ("e1a", 32, 64, 1), ("e1b", 64, 64, 1),
    ("e2a", 64, 128, 2), ("e2b", 128, 128, 2),
    ("bt", 128, 256, 3),
    ("d2", 384, 128, 2), ("d1", 192, 64, 1), ("d0", 96, 32, 0),
]
HEAD_C = 32


def pool(a):
    """2x2x2 means (Z, Y, X, C) -> (Z/2, Y/2, X/2, C)"""
    Z, Y, X, C = a.shape
    return np.asarray(a, np.float64).reshape(Z // 2, 2, Y // 2, 2, X // 2, 2, C).mean(axis=(1, 3, 5))


def pool_grad(g):
    """adjoint of pool: every fine voxel gets its coarse gradient / 8"""
    return upsample(g) / 8.0


def upsample(a):
    """nearest: (Z, Y, X, C) -> (2Z, 2Y, 2X, C)"""
    a = np.asarray(a, np.float64)
    return a.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)


def upsample_grad(g):
    """adjoint of upsample: sum over the 8 fine voxels"""
    Z, Y, X, C = g.shape
    return np.asarray(g, np.float64).reshape(Z // 2, 2, Y // 2, 2, X // 2, 2, C).sum(axis=(1, 3, 5))


def split_params(flat):
    """the flat parameter vector of tess2_gb300.unet.UNet -> {name: (W, b)}, head (w, b)"""
    flat = np.asarray(flat, np.float64)
    out, off = {}, 0
    for name, ci, co, _ in CONVS:
        w = flat[off:off + 27 * co * ci].reshape(27, co, ci)
        off += 27 * co * ci
        out[name] = (w, flat[off:off + co])
        off += co
    out["head"] = (flat[off:off + HEAD_C], flat[off + HEAD_C])
    return out


def forward(P, field):
    """Activations of every layer and the prediction for field (Z, Y, X)."""
    f = np.asarray(field, np.float64)
    A = {}
    x0 = np.zeros(f.shape + (16,))
    x0[..., 0] = f
    A["x0"] = x0

    def c(name, x):
        w, b = P[name]
        return conv3d(x, w, b, relu=True)

    A["e0a"] = c("e0a", x0)
    A["e0b"] = c("e0b", A["e0a"])
    A["p0"] = pool(A["e0b"])
    A["e1a"] = c("e1a", A["p0"])
    A["e1b"] = c("e1b", A["e1a"])
    A["p1"] = pool(A["e1b"])
    A["e2a"] = c("e2a", A["p1"])
    A["e2b"] = c("e2b", A["e2a"])
    A["p2"] = pool(A["e2b"])
    A["bt"] = c("bt", A["p2"])
    A["cat2"] = np.concatenate([upsample(A["bt"]), A["e2b"]], axis=3)
    A["d2"] = c("d2", A["cat2"])
    A["cat1"] = np.concatenate([upsample(A["d2"]), A["e1b"]], axis=3)
    A["d1"] = c("d1", A["cat1"])
    A["cat0"] = np.concatenate([upsample(A["d1"]), A["e0b"]], axis=3)
    A["d0"] = c("d0", A["cat0"])
    wh, bh = P["head"]
    A["pred"] = f + A["d0"] @ wh + bh
    return A


def loss(P, field, target):
    A = forward(P, field)
    return float(np.mean((A["pred"] - np.asarray(target, np.float64)) ** 2))


def backward(P, A, target):
    """Gradients of mean((pred - target)^2): {name: (dW, db)} and head (dw, db)."""
    G = {}
    g = 2.0 * (A["pred"] - np.asarray(target, np.float64)) / A["pred"].size
    wh, _ = P["head"]
    G["head"] = ((A["d0"] * g[..., None]).reshape(-1, HEAD_C).sum(0), g.sum())
    gd = g[..., None] * wh * (A["d0"] > 0)

    def back(name, x, gy, mask=None, want_x=True):
        dw, db = conv3d_wgrad(x, gy)
        G[name] = (dw, db)
        if not want_x:
            return None
        gx = conv3d_dgrad(gy, P[name][0])
        return gx * (mask > 0) if mask is not None else gx

    gcat0 = back("d0", A["cat0"], gd, A["cat0"])
    gd1 = upsample_grad(gcat0[..., :64])
    gcat1 = back("d1", A["cat1"], gd1, A["cat1"])
    gd2 = upsample_grad(gcat1[..., :128])
    gcat2 = back("d2", A["cat2"], gd2, A["cat2"])
    gbt = upsample_grad(gcat2[..., :256])
    gp2 = back("bt", A["p2"], gbt)
    ge2b = (gcat2[..., 256:] + pool_grad(gp2)) * (A["e2b"] > 0)
    ge2a = back("e2b", A["e2a"], ge2b, A["e2a"])
    gp1 = back("e2a", A["p1"], ge2a)
    ge1b = (gcat1[..., 128:] + pool_grad(gp1)) * (A["e1b"] > 0)
    ge1a = back("e1b", A["e1a"], ge1b, A["e1a"])
    gp0 = back("e1a", A["p0"], ge1a)
    ge0b = (gcat0[..., 64:] + pool_grad(gp0)) * (A["e0b"] > 0)
    ge0a = back("e0b", A["e0a"], ge0b, A["e0a"])
    back("e0a", A["x0"], ge0a, want_x=False)
    return G


def flat_grads(G):
    """{name: (dW, db)} -> the flat layout of UNet.grads"""
    parts = []
    for name, _, _, _ in CONVS:
        parts += [G[name][0].ravel(), np.ravel(G[name][1])]
    parts += [np.ravel(G["head"][0]), np.ravel(G["head"][1])]
    return np.concatenate(parts)


def cell_moments(xyz, grid_min, grid_step, dims, f32=False):
    """The particles' voxel moments (tessgpu_unet_cell_moments): each particle
    at its nearest grid point g (round half to even, as the kernel's
    float-to-int rounding), u = (p - g) / step; planes (10, Z, Y, X): count,
    sums of u_x, u_y, u_z, of u_x^2, u_y^2, u_z^2, u_x u_y, u_x u_z, u_y u_z,
    summed in FP64.  Particles whose nearest point is outside the grid are
    left out.  f32: the grid coordinate (p - min) * (1 / step) in FP32, as the
    kernel computes it, so that particles at a voxel boundary fall the same
    way; otherwise FP64."""
    X, Y, Z = (int(d) for d in dims)
    if f32:
        inv = (np.float32(1.0) / np.asarray(grid_step, np.float32)).astype(np.float32)
        f = ((np.asarray(xyz, np.float32) - np.asarray(grid_min, np.float32)) * inv).astype(np.float64)
    else:
        f = (np.asarray(xyz, np.float64) - np.asarray(grid_min, np.float64)) / np.asarray(grid_step, np.float64)
    i = np.rint(f).astype(np.int64)
    ok = np.all((i >= 0) & (i < np.array([X, Y, Z])), axis=1)
    f, i = f[ok], i[ok]
    u = f - i
    v = (i[:, 2] * Y + i[:, 1]) * X + i[:, 0]
    terms = [np.ones(len(u)), u[:, 0], u[:, 1], u[:, 2], u[:, 0] ** 2, u[:, 1] ** 2, u[:, 2] ** 2,
             u[:, 0] * u[:, 1], u[:, 0] * u[:, 2], u[:, 1] * u[:, 2]]
    m = np.zeros((10, X * Y * Z))
    for k, t in enumerate(terms):
        np.add.at(m[k], v, t)
    return m.reshape(10, Z, Y, X)


def input_features(field, m):
    """The 16 input channels tessgpu_unet_input_moments makes, FP64, (Z, Y, X, 16)."""
    n = m[0]
    safe = np.maximum(n, 1.0)
    f = np.zeros(n.shape + (16,))
    f[..., 0] = field
    f[..., 1] = np.log1p(n)
    mean = [np.where(n > 0, m[1 + a] / safe, 0.0) for a in range(3)]
    for a in range(3):
        f[..., 2 + a] = 2.0 * mean[a]
    pairs = [(4, 0, 0), (5, 1, 1), (6, 2, 2), (7, 0, 1), (8, 0, 2), (9, 1, 2)]
    for k, (plane, a, b) in enumerate(pairs):
        f[..., 5 + k] = np.where(n > 1, 12.0 * (m[plane] / safe - mean[a] * mean[b]), 0.0)
    return f
