"""FP64 CPU oracle for the surrogate's 3x3x3 convolutions.  TEST
INFRASTRUCTURE ONLY: tests/ use it to check the GPU kernels' forward pass,
data gradient and weight gradient.

Layout as the kernels: activations (Z, Y, X, C), channel fastest; weights
(27, c_out, c_in) with tap = (dz * 3 + dy) * 3 + dx for offsets -1..1; zero
outside the grid.
"""
import numpy as np


def _taps():
    for t in range(27):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def _shift(a, dz, dy, dx):
    """a[z + dz, y + dy, x + dx] with zeros outside (a: Z, Y, X, C)."""
    Z, Y, X, _ = a.shape
    p = np.pad(a, ((1, 1), (1, 1), (1, 1), (0, 0)))
    return p[1 + dz:1 + dz + Z, 1 + dy:1 + dy + Y, 1 + dx:1 + dx + X]


def conv3d(x, w, b=None, relu=False):
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    y = np.zeros(x.shape[:3] + (w.shape[1],))
    for t, dz, dy, dx in _taps():
        y += _shift(x, dz, dy, dx) @ w[t].T
    if b is not None:
        y += np.asarray(b, np.float64)
    return np.maximum(y, 0.0) if relu else y


def conv3d_dgrad(dy, w):
    """d/dx of sum(dy * conv3d(x, w))."""
    dy = np.asarray(dy, np.float64)
    w = np.asarray(w, np.float64)
    dx = np.zeros(dy.shape[:3] + (w.shape[2],))
    for t, dz, dyo, dxo in _taps():
        dx += _shift(dy, -dz, -dyo, -dxo) @ w[t]
    return dx


def conv3d_wgrad(x, dy):
    """d/dw and d/db of sum(dy * conv3d(x, w, b))."""
    x = np.asarray(x, np.float64)
    dy = np.asarray(dy, np.float64)
    cin, cout = x.shape[3], dy.shape[3]
    dw = np.zeros((27, cout, cin))
    for t, dz, dyo, dxo in _taps():
        xs = _shift(x, dz, dyo, dxo).reshape(-1, cin)
        dw[t] = dy.reshape(-1, cout).T @ xs
    return dw, dy.reshape(-1, cout).sum(0)
