"""The DTFE surrogate: a small 3-D convolutional network that maps the cheap
cloud-in-cell density grid (DENSE_CIC, no Delaunay needed) of a particle set
to its DTFE density grid, both as log(1 + rho / mean rho).  The plain DTFE
path makes the training fields, measures the network's error, and is the
fallback.

Five 3x3x3 convolutions, channels 16 -> 16 -> 32 -> 32 -> 16 -> 16 (the input
grid in channel 0 of 16, the prediction in channel 0 of the last layer, ReLU
between), and a skip: prediction = input + network.  Forward, data gradient
and weight gradient run in libtess2_gb300.so's kernels (tessgpu_conv3d_*:
tensor-core implicit GEMM, bf16 activations and weights, FP32 accumulation
and master weights, Adam); torch holds the buffers and does the elementwise
loss.
"""
import ctypes
import math
import os
import time

import numpy as np

from . import api

LAYERS = [(16, 16), (16, 32), (32, 32), (32, 16), (16, 16)]   # (c_in, c_out)


def _lib():
    L = api.lib()
    vp, i = ctypes.c_void_p, ctypes.c_int
    sig = {
        "tessgpu_conv3d_fwd": (i, [vp, i, i, i, i, i, vp, vp, i, vp, vp, vp]),
        "tessgpu_conv3d_wgrad": (i, [vp, vp, i, i, i, i, i, vp, vp, vp]),
        "tessgpu_conv3d_prepare_weights": (i, [vp, i, i, vp, vp, vp]),
        "tessgpu_relu_grad": (i, [vp, vp, ctypes.c_longlong, vp, vp]),
        "tessgpu_adam": (i, [vp, vp, vp, vp, i, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, i,
                             vp]),
        "tessgpu_conv3d_set_engine": (i, [i]),
        "tessgpu_conv3d_check": (i, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def _ok(s, what):
    if s != 0:
        raise api.TessGpuError(s, what)


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _s(stream):
    """The CUDA stream for a call: torch's current stream unless one is given
    (so that the kernels follow torch's ordering and can be captured in a CUDA
    graph)."""
    if stream is not None:
        return stream
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def planar_shape(V, c):
    """Shape of a chunk-planar activation tensor: channel c of voxel v at [c // 8, v, c % 8]."""
    return (c // 8, V, 8)


def to_planar(a):
    """(V, c) channels-last numpy array -> (c // 8, V, 8) chunk-planar copy."""
    a = np.asarray(a)
    V, c = a.shape
    return np.ascontiguousarray(a.reshape(V, c // 8, 8).transpose(1, 0, 2))


def from_planar(a):
    """(c // 8, V, 8) chunk-planar numpy array -> (V, c) channels-last copy."""
    a = np.asarray(a)
    n, V, _ = a.shape
    return np.ascontiguousarray(a.transpose(1, 0, 2).reshape(V, n * 8))


def conv3d_fwd(x, shape, cin, cout, w_bf16, bias=None, relu=False, y_bf16=None, y_f32=None, stream=None):
    Z, Y, X = shape
    _ok(_lib().tessgpu_conv3d_fwd(_p(x), X, Y, Z, cin, cout, _p(w_bf16), _p(bias), 1 if relu else 0, _p(y_bf16),
                                  _p(y_f32), _s(stream)), "tessgpu_conv3d_fwd")


ENGINE_TCGEN05, ENGINE_MMA_SYNC = 0, 1


def set_engine(engine):
    """ENGINE_TCGEN05 (the default: tcgen05 with tensor-memory accumulators
    where c_in and c_out are 16 or 32) or ENGINE_MMA_SYNC (mma.sync for every
    shape); process-wide."""
    _ok(_lib().tessgpu_conv3d_set_engine(engine), "tessgpu_conv3d_set_engine")


def check(stream=None):
    """Synchronises; raises if a tcgen05 convolution gave up on a bounded wait."""
    _ok(_lib().tessgpu_conv3d_check(_s(stream)), "tessgpu_conv3d_check")


def conv3d_wgrad(x, dy, shape, cin, cout, dw, db=None, stream=None):
    Z, Y, X = shape
    _ok(_lib().tessgpu_conv3d_wgrad(_p(x), _p(dy), X, Y, Z, cin, cout, _p(dw), _p(db), _s(stream)),
        "tessgpu_conv3d_wgrad")


def prepare_weights(w, cout, cin, w_bf16, wt_bf16, stream=None):
    _ok(_lib().tessgpu_conv3d_prepare_weights(_p(w), cout, cin, _p(w_bf16), _p(wt_bf16), _s(stream)),
        "tessgpu_conv3d_prepare_weights")


def relu_grad(g, y, out, stream=None):
    _ok(_lib().tessgpu_relu_grad(_p(g), _p(y), g.numel(), _p(out), _s(stream)), "tessgpu_relu_grad")


def adam(w, g, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8, stream=None):
    _ok(_lib().tessgpu_adam(_p(w), _p(g), _p(m), _p(v), w.numel(), lr, b1, b2, eps, step, _s(stream)),
        "tessgpu_adam")


def forward_flops(shape):
    V = shape[0] * shape[1] * shape[2]
    return sum(2 * 27 * ci * co * V for ci, co in LAYERS)


class Surrogate:
    """The network on one CUDA device, for fields of one grid shape (Z, Y, X)."""

    def __init__(self, shape, seed=0, device="cuda:0"):
        import torch
        self.torch = torch
        self.shape = tuple(int(s) for s in shape)
        self.V = self.shape[0] * self.shape[1] * self.shape[2]
        self.dev = device
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.mw, self.vw, self.mb, self.vb, self.wb, self.wt = [], [], [], [], [], [], [], []
        for li, (ci, co) in enumerate(LAYERS):
            fan_in = 27 * ci
            std = math.sqrt(2.0 / fan_in) * (0.1 if li == len(LAYERS) - 1 else 1.0)
            w = (torch.randn((27, co, ci), generator=g) * std).to(device)
            self.w.append(w)
            self.b.append(torch.zeros(co, device=device))
            for lst, n in ((self.mw, w), (self.vw, w)):
                lst.append(torch.zeros_like(n))
            self.mb.append(torch.zeros(co, device=device))
            self.vb.append(torch.zeros(co, device=device))
            self.wb.append(torch.empty((27, co, ci), dtype=torch.bfloat16, device=device))
            self.wt.append(torch.empty((27, ci, co), dtype=torch.bfloat16, device=device))
        self.step = 0
        self._sync_weights()
        V = self.V
        # activations chunk-planar: (c / 8, V, 8)
        self.x16 = torch.zeros(planar_shape(V, 16), dtype=torch.bfloat16, device=device)
        self.act = [torch.empty(planar_shape(V, co), dtype=torch.bfloat16, device=device) for _, co in LAYERS]
        self.out = torch.empty(planar_shape(V, LAYERS[-1][1]), dtype=torch.float32, device=device)
        cmax = max(max(ci, co) for ci, co in LAYERS)
        self.g32 = torch.empty(V * cmax, dtype=torch.float32, device=device)   # data gradient, (c/8, V, 8) in front
        self.dz = [torch.empty(planar_shape(V, co), dtype=torch.bfloat16, device=device) for _, co in LAYERS]
        self.dw = [torch.zeros_like(w) for w in self.w]
        self.db = [torch.zeros_like(b) for b in self.b]

    def _sync_weights(self):
        for li, (ci, co) in enumerate(LAYERS):
            prepare_weights(self.w[li], co, ci, self.wb[li], self.wt[li])

    def forward(self, x_log):
        """Prediction (V,) FP32 for the input log-density (V,) FP32 on the device."""
        self.x16.zero_()
        self.x16[0, :, 0] = x_log.to(self.torch.bfloat16)
        src = self.x16
        for li, (ci, co) in enumerate(LAYERS):
            last = li == len(LAYERS) - 1
            conv3d_fwd(src, self.shape, ci, co, self.wb[li], self.b[li], relu=not last,
                       y_bf16=None if last else self.act[li], y_f32=self.out if last else None)
            src = self.act[li]
        return x_log + self.out[0, :, 0]

    def forward_graph(self, x_log):
        """forward() replayed from a CUDA graph captured on the first call (the
        five convolution launches and the elementwise work, no host work per
        call).  Returns a view of the graph's own output buffer, overwritten by
        the next call; weights updated in place since are seen."""
        torch = self.torch
        if getattr(self, "_graph", None) is None:
            self._gx = x_log.detach().clone()
            side = torch.cuda.Stream(device=self.dev)
            side.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(side):
                self.forward(self._gx)   # launch set-up (attributes, first use) outside the capture
            torch.cuda.current_stream().wait_stream(side)
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                self._gy = self.forward(self._gx)
            self._graph = graph
        self._gx.copy_(x_log)
        self._graph.replay()
        return self._gy

    def train_step(self, x_log, y_log, lr=1e-3):
        """One Adam step on the mean squared error of the log-density; returns the loss."""
        torch = self.torch
        pred = self.forward(x_log)
        diff = pred - y_log
        loss = float((diff * diff).mean())
        L = len(LAYERS)
        self.dz[L - 1].zero_()
        self.dz[L - 1][0, :, 0] = (diff * (2.0 / self.V)).to(torch.bfloat16)
        for li in range(L - 1, -1, -1):
            ci, co = LAYERS[li]
            inp = self.x16 if li == 0 else self.act[li - 1]
            self.dw[li].zero_()
            self.db[li].zero_()
            conv3d_wgrad(inp, self.dz[li], self.shape, ci, co, self.dw[li], self.db[li])
            if li > 0:
                # the data gradient: the same convolution with the flipped, transposed weights
                g = self.g32[:self.V * ci].view(planar_shape(self.V, ci))
                conv3d_fwd(self.dz[li], self.shape, co, ci, self.wt[li], None, relu=False, y_f32=g)
                relu_grad(g, self.act[li - 1], self.dz[li - 1])
        self.step += 1
        for li in range(L):
            adam(self.w[li], self.dw[li], self.mw[li], self.vw[li], lr, self.step)
            adam(self.b[li], self.db[li], self.mb[li], self.vb[li], lr, self.step)
        self._sync_weights()
        return loss

    def state(self):
        return {f"w{i}": w.cpu().numpy() for i, w in enumerate(self.w)} | \
            {f"b{i}": b.cpu().numpy() for i, b in enumerate(self.b)}

    def load(self, state):
        for i in range(len(LAYERS)):
            self.w[i].copy_(self.torch.from_numpy(state[f"w{i}"]))
            self.b[i].copy_(self.torch.from_numpy(state[f"b{i}"]))
        self._sync_weights()


# ---------------------------------------------------------------------------
# training fields from the plain path
# ---------------------------------------------------------------------------
def log_density(grid):
    g = np.asarray(grid, np.float64)
    return np.log1p(g / max(g.mean(), 1e-30)).astype(np.float32)


def make_fields(ctx, seeds, n_particles, side, processes=None):
    """(x_log, y_log) pairs for each seed: the CIC and DTFE grids (side^3) of a
    mixture particle set in the unit box (one block; host Qhull in parallel
    processes, one per set)."""
    from . import host
    blocks = []
    for s in seeds:
        pts = host.mixture_particles(n_particles, int(s), frac_uniform=0.5, n_clumps=64, sigma=0.02)
        blocks.append(host.decompose(pts)[0])
    blocks = host.tessellate(blocks, processes=processes)
    out = []
    gni = [side] * 3
    for b in blocks:
        cic = ctx.dense(api.DENSE_CIC, [b], gni)["grid"]
        dtfe = ctx.dense(api.DENSE_DTFE, [b], gni)["grid"]
        out.append((log_density(cic).ravel(), log_density(dtfe).ravel()))
    return out


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def forward_ms(net, x, engine=ENGINE_TCGEN05, reps=10, graph=False):
    """Mean forward time (ms, CUDA events) of net on the resident input x with
    the given convolution engine (graph: replayed from a CUDA graph); the
    engine is reset to tcgen05 after."""
    import torch
    set_engine(engine)
    fwd = net.forward_graph if graph else net.forward
    try:
        for _ in range(3):
            fwd(x)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fwd(x)
        e1.record()
        torch.cuda.synchronize()
        check()
    finally:
        set_engine(ENGINE_TCGEN05)
    return e0.elapsed_time(e1) / reps


def forward_throughput(side, engine=ENGINE_TCGEN05, reps=5, seed=3):
    """(ms, TFLOP/s) of one forward pass of a randomly initialised network on
    a side^3 grid of random log densities."""
    import torch
    net = Surrogate((side, side, side), seed=seed)
    g = torch.Generator(device=net.dev).manual_seed(seed)
    x = torch.rand(side ** 3, device=net.dev, generator=g)
    ms = forward_ms(net, x, engine=engine, reps=reps)
    return ms, forward_flops(net.shape) / (ms * 1e-3) / 1e12


def layer_times(side, engine=ENGINE_TCGEN05, reps=5, seed=3):
    """Per-layer forward times on a side^3 grid of random input (random
    weights): [(c_in, c_out, ms, TFLOP/s)], CUDA events around each launch."""
    import torch
    net = Surrogate((side, side, side), seed=seed)
    g = torch.Generator(device=net.dev).manual_seed(seed)
    x = torch.rand(side ** 3, device=net.dev, generator=g)
    V = side ** 3
    set_engine(engine)
    try:
        net.forward(x)   # fills every layer's input
        torch.cuda.synchronize()
        out = []
        for li, (ci, co) in enumerate(LAYERS):
            last = li == len(LAYERS) - 1
            src = net.x16 if li == 0 else net.act[li - 1]
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            for _ in range(reps):
                conv3d_fwd(src, net.shape, ci, co, net.wb[li], net.b[li], relu=not last,
                           y_bf16=None if last else net.act[li], y_f32=net.out if last else None)
            ev[1].record()
            torch.cuda.synchronize()
            ms = ev[0].elapsed_time(ev[1]) / reps
            out.append((ci, co, ms, 2.0 * 27 * ci * co * V / (ms * 1e-3) / 1e12))
        check()
    finally:
        set_engine(ENGINE_TCGEN05)
    return out


def wgrad_times(side, engine=ENGINE_TCGEN05, reps=3, seed=5):
    """Per-layer weight-gradient times on a side^3 grid of random activations
    and output gradients: [(c_in, c_out, ms, TFLOP/s)] (2 * 27 * c_in * c_out
    FLOP per voxel), CUDA events around each launch."""
    import torch
    V = side ** 3
    g = torch.Generator(device="cuda:0").manual_seed(seed)
    set_engine(engine)
    out = []
    try:
        for ci, co in LAYERS:
            x = torch.randn(planar_shape(V, ci), device="cuda:0", generator=g).to(torch.bfloat16)
            dy = torch.randn(planar_shape(V, co), device="cuda:0", generator=g).to(torch.bfloat16)
            dw = torch.zeros((27, co, ci), device="cuda:0")
            db = torch.zeros(co, device="cuda:0")
            conv3d_wgrad(x, dy, (side, side, side), ci, co, dw, db)
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            for _ in range(reps):
                conv3d_wgrad(x, dy, (side, side, side), ci, co, dw, db)
            ev[1].record()
            torch.cuda.synchronize()
            ms = ev[0].elapsed_time(ev[1]) / reps
            out.append((ci, co, ms, 2.0 * 27 * ci * co * V / (ms * 1e-3) / 1e12))
        check()
    finally:
        set_engine(ENGINE_TCGEN05)
    return out


def train_and_evaluate(n_train=32, n_val=8, n_particles=262144, side=64, epochs=8, lr=2e-3, seed=7, log=None):
    """Trains on fields the plain path makes and reports validation error, the
    CIC input's own error (the method without the network), and throughputs."""
    import torch
    from .api import Context
    ctx = Context(0)
    t0 = time.time()
    train = make_fields(ctx, range(1000 + seed * 10000, 1000 + seed * 10000 + n_train), n_particles, side)
    val = make_fields(ctx, range(900000 + seed * 1000, 900000 + seed * 1000 + n_val), n_particles, side)
    t_fields = time.time() - t0
    net = Surrogate((side, side, side), seed=seed)
    dev = net.dev
    tx = [(torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)) for x, y in train]
    vx = [(torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)) for x, y in val]
    losses = []
    torch.cuda.synchronize()
    t0 = time.time()
    steps = 0
    for ep in range(epochs):
        order = np.random.default_rng(seed + ep).permutation(len(tx))
        el = []
        for k in order:
            el.append(net.train_step(tx[k][0], tx[k][1], lr=lr * (0.5 ** (ep // 3))))
            steps += 1
        losses.append(float(np.mean(el)))
        if log:
            log(f"epoch {ep}: train mse {losses[-1]:.5f}")
    torch.cuda.synchronize()
    t_train = time.time() - t0
    errs, base = [], []
    for x, y in vx:
        p = net.forward(x)
        errs.append(rel_l2(p.cpu().numpy(), y.cpu().numpy()))
        base.append(rel_l2(x.cpu().numpy(), y.cpu().numpy()))
    # inference throughput (forward only, input resident)
    x = vx[0][0]
    for _ in range(3):
        net.forward(x)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        net.forward(x)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / reps
    flops = forward_flops(net.shape)
    fwd_mma_ms = forward_ms(net, x, engine=ENGINE_MMA_SYNC)
    fwd_graph_ms = forward_ms(net, x, graph=True)
    return dict(n_train=n_train, n_val=n_val, particles=n_particles, grid=side, epochs=epochs, steps=steps,
                train_mse=losses, val_rel_l2=float(np.mean(errs)), val_rel_l2_max=float(np.max(errs)),
                cic_rel_l2=float(np.mean(base)), fields_s=t_fields, train_s=t_train,
                train_step_ms=1e3 * t_train / max(steps, 1), forward_ms=fwd_ms, forward_gflop=flops / 1e9,
                forward_tflops=flops / (fwd_ms * 1e-3) / 1e12, forward_mma_sync_ms=fwd_mma_ms,
                forward_graph_ms=fwd_graph_ms, net=net)
