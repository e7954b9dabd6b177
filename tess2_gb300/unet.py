"""The DTFE surrogate as a 3-D U-Net: cloud-in-cell grid in, DTFE grid out,
both as log(1 + rho / mean rho).  The plain DTFE path makes the training
fields, measures the network's error and is its fallback.

Four levels, 32 channels doubling per level (grid S -> S/2 -> S/4 -> S/8),
3x3x3 convolutions with ReLU, 2x2x2 average pooling down, nearest
upsampling up, the skips concatenated:

  e0a 16->32, e0b 32->32            level 0  (input: log CIC in channel 0 of 16,
                                              optionally the particles' voxel
                                              moments in channels 1-10)
  e1a 32->64, e1b 64->64            level 1  (pooled e0b)
  e2a 64->128, e2b 128->128         level 2  (pooled e1b)
  bt 128->256                       level 3  (pooled e2b)
  d2 [up(bt) | e2b] 384->128        level 2
  d1 [up(d2) | e1b] 192->64         level 1
  d0 [up(d1) | e0b] 96->32          level 0
  prediction = input + w . d0 + b   (1x1 head)

3.5 M parameters.  Every step runs in libtess2_gb300.so (tessgpu_unet_*):
convolutions forward and their data gradients as tcgen05 implicit GEMMs
(bf16 operands, FP32 accumulation in tensor memory), weight gradients on
tcgen05 too, pooling / upsampling / head / loss / Adam on the CUDA cores.
torch only holds the buffers.  The concatenations are free: each
concatenation buffer's first planes receive the upsampled tensor and the
next ones the encoder's output (chunk-planar layout, 8 channels per plane).
"""
import ctypes
import math
import time

import numpy as np

from . import api

CONVS = [  # name, c_in, c_out, level
    ("e0a", 16, 32, 0), ("e0b", 32, 32, 0),
    ("e1a", 32, 64, 1), ("e1b", 64, 64, 1),
    ("e2a", 64, 128, 2), ("e2b", 128, 128, 2),
    ("bt", 128, 256, 3),
    ("d2", 384, 128, 2), ("d1", 192, 64, 1), ("d0", 96, 32, 0),
]
HEAD_C = 32
MOMENT_PLANES = 10   # tessgpu_unet_cell_moments: count, 3 first and 6 second moments


def _lib():
    L = api.lib()
    vp, i, ll, f = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
    sig = {
        "tessgpu_unet_conv": [vp, i, i, i, i, vp, i, vp, i, vp, vp, i, vp],
        "tessgpu_unet_wgrad": [vp, vp, i, i, i, i, i, vp, vp, vp],
        "tessgpu_unet_pack_weights": [vp, i, i, vp, vp, vp],
        "tessgpu_unet_pool": [vp, i, i, i, i, vp, vp],
        "tessgpu_unet_pool_grad": [vp, vp, i, vp, i, i, i, i, vp, vp],
        "tessgpu_unet_upsample": [vp, i, i, i, i, vp, i, vp],
        "tessgpu_unet_upsample_grad": [vp, i, i, i, i, i, vp, vp],
        "tessgpu_unet_input": [vp, ll, vp, vp],
        "tessgpu_unet_cell_moments": [vp, ll, vp, vp, i, i, i, vp, vp],
        "tessgpu_unet_input_moments": [vp, vp, ll, vp, vp],
        "tessgpu_unet_head": [vp, i, vp, vp, ll, vp, vp, vp, vp],
        "tessgpu_unet_head_grad": [vp, i, vp, vp, vp, ll, f, vp, vp, vp],
        "tessgpu_unet_check": [vp],
        "tessgpu_adam": [vp, vp, vp, vp, i, f, f, f, f, i, vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    return L


def _ok(s, what):
    if s != 0:
        raise api.TessGpuError(s, what)


def _stream(stream=None):
    if stream is not None:
        return stream
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t, planes=0, V=0):
    """device address of t (bf16 chunk-planar) advanced by `planes` planes of V voxels"""
    return None if t is None else ctypes.c_void_p(t.data_ptr() + planes * V * 8 * t.element_size())


def conv(x, grid, cin, w_packed, cout, y, y_plane0=0, bias=None, relu=False, mask=None, stream=None):
    """y[planes y_plane0 ..] = relu?(conv3x3x3(x) + bias), or times (mask > 0) (data gradients)."""
    X, Y, Z = grid
    _ok(_lib().tessgpu_unet_conv(_ptr(x), X, Y, Z, cin, _ptr(w_packed), cout, _ptr(bias), int(relu), _ptr(mask),
                                 _ptr(y), y_plane0, _stream(stream)), "tessgpu_unet_conv")


def wgrad(x, dy, grid, cin, cout, dw, db=None, stream=None):
    """dw[27][cout][cin] += sum_v dy[v] x[v + tap]; db += sum_v dy[v]."""
    X, Y, Z = grid
    _ok(_lib().tessgpu_unet_wgrad(_ptr(x), _ptr(dy), X, Y, Z, cin, cout, _ptr(dw), _ptr(db), _stream(stream)),
        "tessgpu_unet_wgrad")


def pack_weights(w, cout, cin, w_fwd, w_bwd, stream=None):
    _ok(_lib().tessgpu_unet_pack_weights(_ptr(w), cout, cin, _ptr(w_fwd), _ptr(w_bwd), _stream(stream)),
        "tessgpu_unet_pack_weights")


def check(stream=None):
    """Raises when a tensor-core kernel's bounded wait ran out since the last check."""
    _ok(_lib().tessgpu_unet_check(_stream(stream)), "tessgpu_unet_check")


def conv_flops(grid, cin, cout):
    return 2.0 * 27 * cin * cout * grid[0] * grid[1] * grid[2]


class UNet:
    """The U-Net on a grid of S0 = (X, Y, Z) voxels at level 0 (each divisible
    by 8; X at level 0 a multiple of 128, and X / 2^l in {16, 32, 64} or a
    multiple of 128 at the other levels)."""

    def __init__(self, grid, seed=0, device="cuda:0", in_channels=1):
        import torch
        self.dev = torch.device(device)
        X, Y, Z = grid
        if X % 8 or Y % 8 or Z % 8:
            raise ValueError("grid sides must be divisible by 8")
        self.grids = [(X >> l, Y >> l, Z >> l) for l in range(4)]
        self.V = [g[0] * g[1] * g[2] for g in self.grids]
        rng = np.random.default_rng(seed)
        # parameters in one flat FP32 buffer: per conv W[27][cout][cin] then b[cout]; head w[32], b
        self.slices = {}
        off = 0
        for name, ci, co, _ in CONVS:
            self.slices[name] = (off, off + 27 * co * ci, off + 27 * co * ci + co)
            off += 27 * co * ci + co
        self.slices["head"] = (off, off + HEAD_C, off + HEAD_C + 1)
        off += HEAD_C + 1
        self.nparams = off
        p = np.zeros(off, np.float32)
        for name, ci, co, _ in CONVS:
            a, b, _ = self.slices[name]
            # e0a sees in_channels nonzero input channels (1: the CIC grid; 11 with the moments)
            fan = 27 * (in_channels if name == "e0a" else ci)
            w = rng.standard_normal((27, co, ci)).astype(np.float32) * math.sqrt(2.0 / fan)
            if name == "e0a":
                w[:, :, in_channels:] = 0.0
            p[a:b] = w.ravel()
        f32, bf = torch.float32, torch.bfloat16
        self.params = torch.from_numpy(p).to(self.dev)
        self.grads = torch.zeros(off, dtype=f32, device=self.dev)
        self.m = torch.zeros(off, dtype=f32, device=self.dev)
        self.v = torch.zeros(off, dtype=f32, device=self.dev)
        self.step = 0
        self.wf, self.wb = {}, {}
        for name, ci, co, _ in CONVS:
            self.wf[name] = torch.empty(27 * ci * co, dtype=bf, device=self.dev)
            self.wb[name] = torch.empty(27 * ci * co, dtype=bf, device=self.dev)

        def act(level, c):
            return torch.zeros((c // 8, self.V[level], 8), dtype=bf, device=self.dev)

        A = self.a = {}
        A["x0"] = act(0, 16)
        A["e0a"] = act(0, 32)
        A["cat0"] = act(0, 96)     # [up(d1) 64 | e0b 32]
        A["p0"] = act(1, 32)
        A["e1a"] = act(1, 64)
        A["cat1"] = act(1, 192)    # [up(d2) 128 | e1b 64]
        A["p1"] = act(2, 64)
        A["e2a"] = act(2, 128)
        A["cat2"] = act(2, 384)    # [up(bt) 256 | e2b 128]
        A["p2"] = act(3, 128)
        A["bt"] = act(3, 256)
        A["d2"] = act(2, 128)
        A["d1"] = act(1, 64)
        A["d0"] = act(0, 32)
        G = self.g = {}
        for k in ("d0", "e0b", "e0a"):
            G[k] = act(0, 32)
        G["cat0"] = act(0, 96)
        G["d1"] = act(1, 64)
        G["cat1"] = act(1, 192)
        G["e1b"] = act(1, 64)
        G["e1a"] = act(1, 64)
        G["p0"] = act(1, 32)
        G["d2"] = act(2, 128)
        G["cat2"] = act(2, 384)
        G["e2b"] = act(2, 128)
        G["e2a"] = act(2, 128)
        G["p1"] = act(2, 64)
        G["bt"] = act(3, 256)
        G["p2"] = act(3, 128)
        self.field = torch.zeros(self.V[0], dtype=f32, device=self.dev)
        self.target = torch.zeros(self.V[0], dtype=f32, device=self.dev)
        self.pred = torch.zeros(self.V[0], dtype=f32, device=self.dev)
        self.loss = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self._pack()

    # ---- parameters ----
    def w(self, name):
        a, b, _ = self.slices[name]
        return self.params[a:b]

    def b(self, name):
        _, b, c = self.slices[name]
        return self.params[b:c]

    def head(self):
        a, _, c = self.slices["head"]
        return self.params[a:c]

    def _pack(self, stream=None):
        for name, ci, co, _ in CONVS:
            pack_weights(self.w(name), co, ci, self.wf[name], self.wb[name], stream)

    def flops_forward(self):
        return sum(conv_flops(self.grids[l], ci, co) for _, ci, co, l in CONVS)

    # ---- forward ----
    def _conv(self, name, x, y, y_plane0=0, stream=None):
        ci, co, l = next((c[1], c[2], c[3]) for c in CONVS if c[0] == name)
        conv(x, self.grids[l], ci, self.wf[name], co, y, y_plane0, bias=self.b(name), relu=True, stream=stream)

    def forward(self, field=None, target=None, stream=None, moments=None):
        """Prediction (FP32, V0) for the field (FP32 log CIC, V0) -- by default the
        resident self.field; with a target the squared error is summed into self.loss.
        moments: the particles' voxel moments (cell_moments) as further input channels."""
        L = _lib()
        s = _stream(stream)
        A, V, G3 = self.a, self.V, self.grids
        if field is not None:
            self.field.copy_(field)
        if moments is not None:
            _ok(L.tessgpu_unet_input_moments(_ptr(self.field), _ptr(moments), V[0], _ptr(A["x0"]), s),
                "tessgpu_unet_input_moments")
        else:
            _ok(L.tessgpu_unet_input(_ptr(self.field), V[0], _ptr(A["x0"]), s), "tessgpu_unet_input")
        self._conv("e0a", A["x0"], A["e0a"], stream=s)
        self._conv("e0b", A["e0a"], A["cat0"], 8, stream=s)
        _ok(L.tessgpu_unet_pool(_ptr(A["cat0"], 8, V[0]), *G3[0], 32, _ptr(A["p0"]), s), "pool")
        self._conv("e1a", A["p0"], A["e1a"], stream=s)
        self._conv("e1b", A["e1a"], A["cat1"], 16, stream=s)
        _ok(L.tessgpu_unet_pool(_ptr(A["cat1"], 16, V[1]), *G3[1], 64, _ptr(A["p1"]), s), "pool")
        self._conv("e2a", A["p1"], A["e2a"], stream=s)
        self._conv("e2b", A["e2a"], A["cat2"], 32, stream=s)
        _ok(L.tessgpu_unet_pool(_ptr(A["cat2"], 32, V[2]), *G3[2], 128, _ptr(A["p2"]), s), "pool")
        self._conv("bt", A["p2"], A["bt"], stream=s)
        _ok(L.tessgpu_unet_upsample(_ptr(A["bt"]), *G3[2], 256, _ptr(A["cat2"]), 0, s), "upsample")
        self._conv("d2", A["cat2"], A["d2"], stream=s)
        _ok(L.tessgpu_unet_upsample(_ptr(A["d2"]), *G3[1], 128, _ptr(A["cat1"]), 0, s), "upsample")
        self._conv("d1", A["cat1"], A["d1"], stream=s)
        _ok(L.tessgpu_unet_upsample(_ptr(A["d1"]), *G3[0], 64, _ptr(A["cat0"]), 0, s), "upsample")
        self._conv("d0", A["cat0"], A["d0"], stream=s)
        if target is not None:
            self.target.copy_(target)
        _ok(L.tessgpu_unet_head(_ptr(A["d0"]), HEAD_C, _ptr(self.head()), _ptr(self.field), V[0], _ptr(self.pred),
                                _ptr(self.target) if target is not None else None,
                                _ptr(self.loss) if target is not None else None, s), "tessgpu_unet_head")
        return self.pred

    # ---- backward ----
    def _back(self, name, x, gy, gx=None, mask=None, stream=None):
        """weight/bias gradient of conv `name` (input x, output gradient gy) and, unless
        gx is None, its input gradient (times (mask > 0) when given)"""
        ci, co, l = next((c[1], c[2], c[3]) for c in CONVS if c[0] == name)
        a, b, c = self.slices[name]
        wgrad(x, gy, self.grids[l], ci, co, self.grads[a:b], self.grads[b:c], stream)
        if gx is not None:
            conv(gy, self.grids[l], co, self.wb[name], ci, gx, 0, mask=mask, stream=stream)

    def backward(self, stream=None):
        """Gradients of mean((pred - target)^2) into self.grads (zeroed here)."""
        L = _lib()
        s = _stream(stream)
        A, G, V, G3 = self.a, self.g, self.V, self.grids
        self.grads.zero_()
        a, _, c = self.slices["head"]
        _ok(L.tessgpu_unet_head_grad(_ptr(A["d0"]), HEAD_C, _ptr(self.head()), _ptr(self.pred), _ptr(self.target),
                                     V[0], ctypes.c_float(1.0 / V[0]), _ptr(G["d0"]), _ptr(self.grads[a:c]), s),
            "tessgpu_unet_head_grad")
        self._back("d0", A["cat0"], G["d0"], G["cat0"], mask=A["cat0"], stream=s)
        _ok(L.tessgpu_unet_upsample_grad(_ptr(G["cat0"]), 0, *G3[0], 64, _ptr(G["d1"]), s), "upsample_grad")
        self._back("d1", A["cat1"], G["d1"], G["cat1"], mask=A["cat1"], stream=s)
        _ok(L.tessgpu_unet_upsample_grad(_ptr(G["cat1"]), 0, *G3[1], 128, _ptr(G["d2"]), s), "upsample_grad")
        self._back("d2", A["cat2"], G["d2"], G["cat2"], mask=A["cat2"], stream=s)
        _ok(L.tessgpu_unet_upsample_grad(_ptr(G["cat2"]), 0, *G3[2], 256, _ptr(G["bt"]), s), "upsample_grad")
        self._back("bt", A["p2"], G["bt"], G["p2"], stream=s)
        _ok(L.tessgpu_unet_pool_grad(_ptr(G["p2"]), _ptr(G["cat2"]), 32, _ptr(A["cat2"], 32, V[2]), *G3[2], 128,
                                     _ptr(G["e2b"]), s), "pool_grad")
        self._back("e2b", A["e2a"], G["e2b"], G["e2a"], mask=A["e2a"], stream=s)
        self._back("e2a", A["p1"], G["e2a"], G["p1"], stream=s)
        _ok(L.tessgpu_unet_pool_grad(_ptr(G["p1"]), _ptr(G["cat1"]), 16, _ptr(A["cat1"], 16, V[1]), *G3[1], 64,
                                     _ptr(G["e1b"]), s), "pool_grad")
        self._back("e1b", A["e1a"], G["e1b"], G["e1a"], mask=A["e1a"], stream=s)
        self._back("e1a", A["p0"], G["e1a"], G["p0"], stream=s)
        _ok(L.tessgpu_unet_pool_grad(_ptr(G["p0"]), _ptr(G["cat0"]), 8, _ptr(A["cat0"], 8, V[0]), *G3[0], 32,
                                     _ptr(G["e0b"]), s), "pool_grad")
        self._back("e0b", A["e0a"], G["e0b"], G["e0a"], mask=A["e0a"], stream=s)
        self._back("e0a", A["x0"], G["e0a"], None, stream=s)

    def adam(self, lr, b1=0.9, b2=0.999, eps=1e-8, stream=None):
        s = _stream(stream)
        self.step += 1
        _ok(_lib().tessgpu_adam(_ptr(self.params), _ptr(self.grads), _ptr(self.m), _ptr(self.v), self.nparams,
                                lr, b1, b2, eps, self.step, s), "tessgpu_adam")
        self._pack(s)

    def train_step(self, field, target, lr=1e-3, stream=None, moments=None):
        """One Adam step on one field; returns nothing (the summed squared error
        accumulates in self.loss, read it when convenient)."""
        self.forward(field, target, stream, moments)
        self.backward(stream)
        self.adam(lr, stream=stream)


# ---------------------------------------------------------------------------
# fields, training, evaluation
# ---------------------------------------------------------------------------
def cell_moments(xyz, grid_min, grid_step, dims, out=None, stream=None):
    """The particles' voxel moments (MOMENT_PLANES x V FP32, device): xyz a
    device tensor of (n, 3) float32, the grid's points grid_min + i * grid_step,
    dims (X, Y, Z)."""
    import torch
    X, Y, Z = (int(d) for d in dims)
    if out is None:
        out = torch.empty(MOMENT_PLANES * X * Y * Z, dtype=torch.float32, device=xyz.device)
    gmin = (ctypes.c_float * 3)(*[float(v) for v in grid_min])
    gstep = (ctypes.c_float * 3)(*[float(v) for v in grid_step])
    _ok(_lib().tessgpu_unet_cell_moments(_ptr(xyz), int(xyz.shape[0]), gmin, gstep, X, Y, Z, _ptr(out),
                                         _stream(stream)), "tessgpu_unet_cell_moments")
    return out


_PAIR = {(0, 1): 7, (1, 0): 7, (0, 2): 8, (2, 0): 8, (1, 2): 9, (2, 1): 9}


def transform_moments(m, S, perm, flips):
    """The voxel moments of the particle set mapped by a symmetry of the cube,
    given as the (z, y, x) array's dimension permutation and the flipped
    dimensions of the permuted array (as applied to the grids): the planes are
    permuted and flipped like the grids, the offsets' components permuted and
    negated along flipped axes, the second moments transformed as R M R^T."""
    import torch
    t = m.view(MOMENT_PLANES, S, S, S).permute(0, *[p + 1 for p in perm])
    if flips:
        t = torch.flip(t, [f + 1 for f in flips])
    # array dimension d is physical axis 2 - d
    src = [2 - perm[2 - a] for a in range(3)]           # new axis a <- old axis src[a]
    sign = [-1.0 if (2 - a) in flips else 1.0 for a in range(3)]
    out = torch.empty((MOMENT_PLANES, S, S, S), dtype=m.dtype, device=m.device)
    out[0] = t[0]
    for a in range(3):
        out[1 + a] = sign[a] * t[1 + src[a]]
        out[4 + a] = t[4 + src[a]]
    for a, b in ((0, 1), (0, 2), (1, 2)):
        out[_PAIR[(a, b)]] = sign[a] * sign[b] * t[_PAIR[(src[a], src[b])]]
    return out.view(-1)


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def pdf_error(pred, target, bins=64):
    """L1 distance between the histograms (densities) of two log-density fields
    over the target's range: 0 = identical one-point PDFs, 2 = disjoint."""
    t = np.asarray(target, np.float64).ravel()
    p = np.asarray(pred, np.float64).ravel()
    lo, hi = float(t.min()), float(t.max()) + 1e-12
    ht, _ = np.histogram(np.clip(t, lo, hi), bins=bins, range=(lo, hi))
    hp, _ = np.histogram(np.clip(p, lo, hi), bins=bins, range=(lo, hi))
    return float(np.abs(ht / max(ht.sum(), 1) - hp / max(hp.sum(), 1)).sum())


def _field_worker(args):
    """(seed, n_particles): the seed's particle set and its Qhull tets (host, in a
    spawned worker process)."""
    from . import host
    seed, n = args
    pts = host.mixture_particles(n, int(seed))
    blk = host.decompose(pts)[0]
    blk["tets"] = host.delaunay_tets(blk["particles"])
    blk["vert_to_tet"] = host.vert_to_tet_host(blk["particles"].shape[0], blk["tets"])
    return blk


def log_density(grid):
    """log(1 + rho / mean rho), FP32"""
    g = np.asarray(grid, np.float64)
    return np.log1p(g / max(g.mean(), 1e-30)).astype(np.float32)


def make_fields(seeds, n_particles, side, processes=None, device=0, log=None, moments=False):
    """(x, y[, m]) per seed: log densities of the CIC and the DTFE grid (side^3,
    one block in the unit box) of the seed's particle set (50 % uniform + 50 %
    in 256 Gaussian clumps, sigma 0.01), and with moments the particles' voxel
    moments on the DTFE grid's points (a device tensor).  Host Qhull in spawned
    worker processes, the GPU passes as each set arrives.  Returns the fields,
    the wall time of the whole run and the seconds of the GPU passes."""
    import multiprocessing as mp
    import os
    import torch
    from .api import DENSE_CIC, DENSE_DTFE, Context
    procs = processes or min(len(seeds), os.cpu_count() or 1)
    out = []
    t0 = time.time()
    gpu_s = 0.0
    ctx = None
    with mp.get_context("spawn").Pool(procs) as pool:
        for i, blk in enumerate(pool.imap(_field_worker, [(s, n_particles) for s in seeds])):
            if ctx is None:
                ctx = Context(device)
            g0 = time.time()
            gni = [side] * 3
            cic = ctx.dense(DENSE_CIC, [blk], gni)["grid"]
            r = ctx.dense(DENSE_DTFE, [blk], gni)
            item = (log_density(cic).ravel(), log_density(r["grid"]).ravel())
            if moments:
                xyz = torch.from_numpy(np.ascontiguousarray(blk["particles"], np.float32)).to(f"cuda:{device}")
                m = cell_moments(xyz, r["info"]["grid_phys_mins"], r["info"]["grid_step_size"], gni)
                torch.cuda.synchronize()
                item = item + (m,)
            gpu_s += time.time() - g0
            out.append(item)
            if log and (i + 1) % 8 == 0:
                log(f"fields: {i + 1}/{len(seeds)} after {time.time() - t0:.0f} s")
    return out, time.time() - t0, gpu_s


def _events_ms(fn, reps):
    import torch
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def timings(side=128, reps=10, seed=0):
    """Forward and training-step times of a randomly initialised network on a
    side^3 grid of random input (CUDA events), with the FLOP counts."""
    import torch
    net = UNet((side, side, side), seed=seed)
    g = torch.Generator(device=net.dev).manual_seed(seed)
    x = torch.rand(side ** 3, device=net.dev, generator=g)
    y = torch.rand(side ** 3, device=net.dev, generator=g)
    fwd = _events_ms(lambda: net.forward(x), reps)
    step = _events_ms(lambda: net.train_step(x, y, lr=1e-4), reps)
    check()
    ff = net.flops_forward()
    # a training step: forward + data gradient (all convs but e0a) + weight gradient
    fb = ff + sum(conv_flops(net.grids[l], ci, co) * (1 if n == "e0a" else 2) for n, ci, co, l in CONVS)
    return dict(grid=side, params=net.nparams, forward_ms=fwd, forward_gflop=ff / 1e9,
                forward_tflops=ff / (fwd * 1e-3) / 1e12, train_step_ms=step, train_step_gflop=fb / 1e9,
                train_step_tflops=fb / (step * 1e-3) / 1e12)


def layer_times(side=128, reps=5, seed=0):
    """Per convolution of a randomly initialised network on a side^3 grid:
    forward, data-gradient and weight-gradient times (CUDA events) and TFLOP/s."""
    import torch
    net = UNet((side, side, side), seed=seed)
    g = torch.Generator(device=net.dev).manual_seed(seed)
    x = torch.rand(side ** 3, device=net.dev, generator=g)
    net.forward(x, x)
    net.backward()
    A, G = net.a, net.g
    io = {  # name: (input, output, output plane, output gradient, input gradient)
        "e0a": (A["x0"], A["e0a"], 0, G["e0a"], None), "e0b": (A["e0a"], A["cat0"], 8, G["e0b"], G["e0a"]),
        "e1a": (A["p0"], A["e1a"], 0, G["e1a"], G["p0"]), "e1b": (A["e1a"], A["cat1"], 16, G["e1b"], G["e1a"]),
        "e2a": (A["p1"], A["e2a"], 0, G["e2a"], G["p1"]), "e2b": (A["e2a"], A["cat2"], 32, G["e2b"], G["e2a"]),
        "bt": (A["p2"], A["bt"], 0, G["bt"], G["p2"]), "d2": (A["cat2"], A["d2"], 0, G["d2"], G["cat2"]),
        "d1": (A["cat1"], A["d1"], 0, G["d1"], G["cat1"]), "d0": (A["cat0"], A["d0"], 0, G["d0"], G["cat0"]),
    }
    out = []
    for name, ci, co, l in CONVS:
        xi, yo, yp, gy, gx = io[name]
        gr = net.grids[l]
        fl = conv_flops(gr, ci, co)
        a, b, c = net.slices[name]
        f = _events_ms(lambda: conv(xi, gr, ci, net.wf[name], co, yo, yp, bias=net.b(name), relu=True), reps)
        d = _events_ms(lambda: conv(gy, gr, co, net.wb[name], ci, gx), reps) if gx is not None else 0.0
        w = _events_ms(lambda: wgrad(xi, gy, gr, ci, co, net.grads[a:b], net.grads[b:c]), reps)
        out.append(dict(name=name, grid=gr[0], c_in=ci, c_out=co, gflop=fl / 1e9, fwd_ms=f, fwd_tflops=fl / f / 1e9,
                        dgrad_ms=d, dgrad_tflops=fl / d / 1e9 if d else None, wgrad_ms=w, wgrad_tflops=fl / w / 1e9))
    check()
    return out


def _train(net, fields, side, epochs, lr, seed, use_moments, log=None):
    """Adam over the fields, one field a step under a random one of the cube's
    48 symmetries (DTFE commutes with them: axis flips and a permutation; the
    voxel moments transform with them), cosine learning-rate decay.  Returns
    the per-epoch mean squared errors, the seconds and the steps."""
    import torch
    S = side
    aug = np.random.default_rng(seed)
    losses = []
    torch.cuda.synchronize()
    t0 = time.time()
    steps, total = 0, epochs * len(fields)
    for ep in range(epochs):
        order = np.random.default_rng(seed + ep).permutation(len(fields))
        net.loss.zero_()
        for k in order:
            flips = [d for d in range(3) if aug.integers(2)]
            perm = [int(a) for a in aug.permutation(3)]
            x, y = (t.view(S, S, S).permute(*perm) for t in fields[k][:2])
            if flips:
                x, y = torch.flip(x, flips), torch.flip(y, flips)
            x, y = x.contiguous().view(-1), y.contiguous().view(-1)
            m = transform_moments(fields[k][2], S, perm, flips) if use_moments else None
            net.train_step(x, y, lr=lr * 0.5 * (1 + math.cos(math.pi * steps / total)), moments=m)
            steps += 1
        losses.append(net.loss.item() / (len(fields) * net.V[0]))
        if log:
            log(f"epoch {ep}: train mse {losses[-1]:.5f}" + (" (moments)" if use_moments else " (CIC only)"))
    torch.cuda.synchronize()
    return losses, time.time() - t0, steps


def _evaluate(net, fields, use_moments):
    out = []
    for f in fields:
        x, y = f[0], f[1]
        p = net.forward(x, moments=f[2] if use_moments else None).cpu().numpy()
        yh = y.cpu().numpy()
        a = x.cpu().numpy().astype(np.float64)
        out.append(dict(err=rel_l2(p, yh), pdf=pdf_error(p, yh), cic=rel_l2(x.cpu().numpy(), yh),
                        s=[1.0, float(a.std()), float((a == 0).mean()), float(a.max())]))
    return out


def train_and_evaluate(n_train=48, n_val=16, n_particles=2097152, side=128, epochs=12, lr=3e-4, seed=7,
                       processes=None, bound=0.05, log=None, moments=True, compare=True):
    """Trains the U-Net on fields the plain path makes, then per validation
    field: relative L2 of the log density against DTFE, the density-PDF error,
    the CIC input's own error (the method without the network).  moments: the
    network also sees the particles' voxel moments (input channels 1-10);
    compare: a second network on the same fields with the CIC grid alone, for
    the difference the moments make.  Fallback: a predicted error per field
    (a least-squares fit, on the training fields, of the network's error
    against statistics of its input), and the fields whose prediction exceeds
    `bound` recomputed exactly by the plain path."""
    import torch
    tr, t_tr, g_tr = make_fields(range(10_000 + seed * 1000, 10_000 + seed * 1000 + n_train), n_particles, side,
                                 processes, log=log, moments=moments)
    va, t_va, g_va = make_fields(range(900_000 + seed * 1000, 900_000 + seed * 1000 + n_val), n_particles, side,
                                 processes, log=log, moments=moments)
    dev = torch.device("cuda:0")
    tx = [tuple(torch.from_numpy(a).to(dev) if isinstance(a, np.ndarray) else a for a in f) for f in tr]
    vx = [tuple(torch.from_numpy(a).to(dev) if isinstance(a, np.ndarray) else a for a in f) for f in va]
    extra = {}
    if moments and compare:
        base = UNet((side, side, side), seed=seed, in_channels=1)
        _train(base, tx, side, epochs, lr, seed, False, log)
        eb = _evaluate(base, vx, False)
        extra = dict(val_rel_l2_cic_only=float(np.mean([e["err"] for e in eb])),
                     val_pdf_error_cic_only=float(np.mean([e["pdf"] for e in eb])))
        del base
    net = UNet((side, side, side), seed=seed, in_channels=11 if moments else 1)
    losses, t_train, steps = _train(net, tx, side, epochs, lr, seed, moments, log)
    check()
    etr, eva = _evaluate(net, tx, moments), _evaluate(net, vx, moments)
    # the error predictor: least squares on the training fields' input statistics
    A = np.array([e["s"] for e in etr])
    coef, *_ = np.linalg.lstsq(A, np.array([e["err"] for e in etr]), rcond=None)
    pred_err = [float(np.dot(coef, e["s"])) for e in eva]
    fallback = [i for i, pe in enumerate(pred_err) if pe > bound]
    served = [0.0 if i in fallback else e["err"] for i, e in enumerate(eva)]
    m0 = vx[0][2] if moments else None
    fwd_ms = _events_ms(lambda: net.forward(vx[0][0], moments=m0), 10)
    mom_ms = None
    if moments:
        # the moments' own cost at serving time: the deposit of the field's particles
        pts = torch.rand(n_particles, 3, device=dev)
        mbuf = torch.empty_like(m0)
        mom_ms = _events_ms(lambda: cell_moments(pts, [0.0] * 3, [1.0 / (side - 1)] * 3, [side] * 3, out=mbuf), 10)
    check()
    return dict(n_train=n_train, n_val=n_val, particles=n_particles, grid=side, epochs=epochs, steps=steps,
                params=net.nparams, inputs="log CIC + voxel moments" if moments else "log CIC",
                train_mse=losses, train_s=t_train, train_step_ms=1e3 * t_train / max(steps, 1),
                fields_wall_s=t_tr + t_va, fields_gpu_s=g_tr + g_va,
                val_rel_l2=float(np.mean([e["err"] for e in eva])),
                val_rel_l2_max=float(np.max([e["err"] for e in eva])),
                val_pdf_error=float(np.mean([e["pdf"] for e in eva])),
                cic_rel_l2=float(np.mean([e["cic"] for e in eva])),
                train_rel_l2=float(np.mean([e["err"] for e in etr])),
                predicted_error=pred_err, actual_error=[e["err"] for e in eva], bound=bound,
                fallback_fields=len(fallback), served_rel_l2=float(np.mean(served)),
                forward_ms=fwd_ms, moments_ms=mom_ms,
                forward_tflops=net.flops_forward() / (fwd_ms * 1e-3) / 1e12, net=net, **extra)
