"""Benchmark: DTFE density of 2,097,152 particles onto a 512^3 grid.

Workload (default): 50% uniform + 50% from 256 Gaussian clumps (sigma 0.01,
Dirichlet(1) weights) in [0,1)^3, float32, unit mass, split into 2x2x2 DIY
blocks with a 0.05 ghost zone; host Qhull tets per block (scipy "Qt", one
process per block); DTFE, mixed precision (FP32 + FP64 fix-up), onto a 512^3
float32 grid.  A step is one full DTFE pass over all blocks: star volumes,
vertex densities, grid zeroing, tet rasterisation (+ FP64 fix-up pass).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value: grid points/s with particles and tets resident in HBM (tessgpu_batch_dense;
       the blocks' stages alternate between two streams);
e2e:   the same metric through the host-buffer call tessgpu_dense, host->device
       copies of particles and tet_t records from pinned memory and the grid
       device->host copy inside the timed region (pipelined per block).
stage_ms: kernel times from a separate pass with the stages run one after the
       other (CUDA events on the launching stream); the roofline uses them.
--impl reference times the reference's own estimator (DENSE_TESS, restated
bit-exactly in oracle/) on the host cores, one process per block, on a sample
of cells per block.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DTFE grid pts/s, 2M pts->512^3, mixed vs FP64 at rel-L2<=1e-6"
UNIT = "grid_pts/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--particles", type=int, default=2097152)
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--blocks", type=int, default=2, help="blocks per axis")
    ap.add_argument("--ghost", type=float, default=0.05)
    ap.add_argument("--frac-uniform", type=float, default=0.5, help="fraction of uniform background particles")
    ap.add_argument("--clumps", type=int, default=256, help="Gaussian clumps")
    ap.add_argument("--sigma", type=float, default=0.01, help="clump sigma")
    ap.add_argument("--sigma-range", type=float, nargs=2, default=None,
                    help="clump sigmas log-uniform in [lo, hi] instead of --sigma")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-spans", action="store_true",
                    help="print the host-buffer call's per-stream spans (upload, compute, download), pinned and "
                         "pageable arrays, on a '# e2e spans' line")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the FP64-mode and DENSE_TESS comparison runs")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="skip training and timing the DTFE surrogate network")
    ap.add_argument("--surrogate-train", action="store_true",
                    help="instead of the DTFE benchmark: make fields of 2,097,152 particles -> 128^3 with the plain "
                         "path, train the U-Net surrogate on them and validate it (one JSON line)")
    ap.add_argument("--surrogate-fields", type=int, default=48, help="training fields for --surrogate-train")
    ap.add_argument("--surrogate-val", type=int, default=16, help="validation fields for --surrogate-train")
    ap.add_argument("--surrogate-epochs", type=int, default=12)
    ap.add_argument("--surrogate-lr", type=float, default=3e-4)
    ap.add_argument("--surrogate-particles", type=int, default=2097152,
                    help="particles per field for --surrogate-train (configuration 4: 2,097,152)")
    ap.add_argument("--sets", type=int, default=0,
                    help="batched independent sets instead: this many particle sets, counts log-uniform in "
                         "[10,000, 500,000], each on its own grid of side 64/128/192/256, all in one call")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the sampled checks against the CPU oracle at the benchmark's size")
    ap.add_argument("--no-rows", action="store_true",
                    help="skip the timings of the stages around the path (reorder_neighbors, incomplete_cells, "
                         "projection, WriteGrid)")
    return ap.parse_args()


def prepare(args, timings=False):
    from tess2_gb300 import host
    t0 = time.time()
    pts = host.mixture_particles(args.particles, args.seed, frac_uniform=args.frac_uniform, n_clumps=args.clumps,
                                 sigma=args.sigma, sigma_range=tuple(args.sigma_range) if args.sigma_range else None)
    blocks = host.decompose(pts, (args.blocks,) * 3, args.ghost)
    t1 = time.time()
    blocks = host.tessellate(blocks, processes=min(len(blocks), os.cpu_count() or 1))
    if timings:
        return blocks, time.time() - t0, time.time() - t1
    return blocks, time.time() - t0


def workload_config(args, blocks):
    T = sum(int(b["tets"].shape[0]) for b in blocks)
    N = sum(int(b["particles"].shape[0]) for b in blocks)
    G = args.grid ** 3
    sig = (f"sigma log-uniform {args.sigma_range[0]}..{args.sigma_range[1]}" if args.sigma_range
           else f"sigma {args.sigma}")
    mix = f"{100 * args.frac_uniform:.0f}% uniform + {100 * (1 - args.frac_uniform):.0f}% {args.clumps} clumps {sig}"
    return dict(workload=f"DTFE {args.particles} particles ({mix}) -> "
                         f"{args.grid}^3 float32, {args.blocks}x{args.blocks}x{args.blocks} blocks, ghost {args.ghost}",
                particles=args.particles, particles_with_ghosts=N, tets=T, grid=[args.grid] * 3,
                blocks=args.blocks ** 3, ghost=args.ghost, seed=args.seed, mode="mixed FP32 + FP64 fix-up",
                l2="inputs and grid larger than L2 (tets+grid > 1 GB vs 126 MB L2); no flush")


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.p = None
        # raw samples (the JSON line carries their summary); BENCH_CLOCKS_DIR keeps them elsewhere
        self.path = os.path.join(os.environ.get("BENCH_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"clocks_{os.getpid()}.csv")
        self.device = device

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return dict(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))


# ---------------------------------------------------------------------------
# CPU legs (the oracle: restated reference estimator and FP64 DTFE)
# ---------------------------------------------------------------------------
_W = {}


def _ref_init(block, share, data6, gni):
    """A reference-arm worker: one block's share of cells, the block's
    circumcenters computed once."""
    from oracle.oracle import TessCells
    _W["tc"] = TessCells(block, data6, gni)
    _W["share"] = np.asarray(share, np.int32)


def _ref_cells(frac, seed):
    """DENSE_TESS on a seeded random fraction of this worker's cells: (seconds, cells)."""
    share = _W["share"]
    rng = np.random.default_rng(seed)
    n = int(round(frac * share.size))
    cells = np.sort(rng.choice(share, size=n, replace=False)) if n < share.size else share
    t0 = time.perf_counter()
    _W["tc"].run(cells)
    return time.perf_counter() - t0, int(cells.size)


def data_bounds6(blocks):
    mn = np.min([b["bounds_min"] for b in blocks], axis=0)
    mx = np.max([b["bounds_max"] for b in blocks], axis=0)
    return np.concatenate([mn, mx]).astype(np.float32)


def dtfe_cpu_baseline(blocks, gni, stride=16):
    """FP64 DTFE oracle, one core, block 0, every stride-th tet rasterised;
    extrapolated to the full workload."""
    from oracle.oracle import Restated
    O = Restated()
    b0 = blocks[0]
    d6 = data_bounds6(blocks)
    t0 = time.perf_counter()
    O.dtfe([b0], gni, want_owner=False, want_rho=False, data6=d6, raster_stride=10 ** 9)
    t_w = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.dtfe([b0], gni, want_owner=False, want_rho=False, data6=d6, raster_stride=stride)
    t_s = time.perf_counter() - t0
    per_block = t_w + max(t_s - t_w, 0.0) * stride
    total_tets = sum(b["tets"].shape[0] for b in blocks)
    full = per_block * total_tets / b0["tets"].shape[0]
    G = float(np.prod(gni))
    return dict(value=G / full, unit=UNIT, cores=1, kind="port",
                sample=f"FP64 DTFE oracle on block 0 ({b0['tets'].shape[0]} tets), star volumes over all tets, "
                       f"every {stride}th tet rasterised; {t_w + t_s:.1f} s measured, {full:.0f} s extrapolated "
                       f"for all {len(blocks)} blocks")


def dense_tess_cpu(blocks, gni, steps, warmup, target_s=2.0):
    """The reference estimator (restated DENSE_TESS) on every host core: a step
    processes all cells when that takes at most 4 s, else a seeded random
    sample sized from two pilots to take about target_s.  Returns (dict, step
    seconds list)."""
    d6 = data_bounds6(blocks)
    cores = os.cpu_count() or 1
    total_cells = sum(b["num_orig"] for b in blocks)
    shares = ref_workers(blocks, max(cores, len(blocks)))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    pools = [ctx.Pool(1, initializer=_ref_init, initargs=(blocks[bi], share, d6, gni)) for bi, share in shares]
    try:
        def step(frac, seed):
            t0 = time.perf_counter()
            rs = [p.apply_async(_ref_cells, (frac, seed * 1000 + w)) for w, p in enumerate(pools)]
            out = [r.get() for r in rs]
            return time.perf_counter() - t0, sum(n for _, n in out)

        step(0.0, 0)   # workers up, circumcenters done
        init_s = time.perf_counter() - t0
        # pilots at two fractions: step time ~ a + b * fraction
        w1, _ = step(0.005, 1)
        w2, _ = step(0.02, 2)
        b = max((w2 - w1) / 0.015, 1e-6)
        a = max(w1 - 0.005 * b, 0.0)
        frac = 1.0 if a + b <= 4.0 else float(min(1.0, max(0.005, (target_s - a) / b)))
        for k in range(warmup):
            step(frac, 10 + k)
        walls, dones = [], []
        for k in range(steps):
            w, done = step(frac, 100 + k)
            walls.append(w)
            dones.append(done)
    finally:
        for p in pools:
            p.close()
            p.join()
    wall = statistics.mean(walls)
    f_eff = statistics.mean(dones) / total_cells
    G = float(np.prod(gni))
    value = G * f_eff / wall
    sample = ("reference DENSE_TESS estimator (restated bit-exactly), "
              + (f"all {total_cells} cells of the {len(blocks)} blocks per step" if frac >= 1.0 else
                 f"a seeded random {100 * f_eff:.2f}% of the {total_cells} cells per step (every block, a fresh "
                 f"sample each step); full pass = step time / fraction")
              + f", on {len(pools)} processes of {cores} host cores")
    return dict(value=value, unit=UNIT, cores=len(pools), kind="port", sample=sample, full_pass_s=wall / f_eff,
                step_s=wall, fraction=f_eff, worker_setup_s=init_s), walls


def ref_workers(blocks, procs):
    """procs workers spread over the blocks in proportion to their cells
    (at least one each); a block's cells are dealt out to its workers in turn."""
    cells = np.array([b["num_orig"] for b in blocks], np.float64)
    nw = np.maximum(1, np.floor(procs * cells / cells.sum())).astype(int)
    while nw.sum() < procs:
        nw[np.argmax(cells / nw)] += 1
    out = []
    for bi, b in enumerate(blocks):
        idx = np.arange(b["num_orig"], dtype=np.int32)
        for w in range(nw[bi]):
            out.append((bi, idx[w::nw[bi]]))
    return out


def run_reference(args):
    """--impl reference: the reference's estimator for this path, dense()
    DENSE_TESS (restated bit-exactly in oracle/, the reference's own sources
    not being on the GPU host), on every host core.  A step processes every
    cell of the 8 blocks when that takes at most 4 s, else a seeded random
    sample of each block's cells (a fresh sample per step, the same fraction
    everywhere) sized from two pilots to take about 2 s; value = the grid
    points per second at which the whole workload finishes (G x fraction /
    step time)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    blocks, prep_s, qhull_s = prepare(args, timings=True)
    gni = [args.grid] * 3
    r, walls = dense_tess_cpu(blocks, gni, args.steps, args.warmup)
    value = r["value"]
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=args.gpus, steps=args.steps, warmup=args.warmup,
                ms_per_step=1e3 * r["step_s"], higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
                data="synthetic", impl="reference", config=workload_config(args, blocks),
                cpu_baseline=dict(value=value, unit=UNIT, cores=r["cores"], kind="port", sample=r["sample"]),
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                full_pass_s=r["full_pass_s"], cells_per_s=sum(b["num_orig"] for b in blocks) / r["full_pass_s"],
                particles_per_s=args.particles / r["full_pass_s"], delaunay_s=qhull_s,
                delaunay_note=f"host Qhull of the {len(blocks)} blocks, one process per block (wall), not in value",
                worker_setup_s=r["worker_setup_s"],
                note="the reference has no DTFE; its own estimator for this path (dense() DENSE_TESS) is timed")
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the stages either side of the density path, on the same blocks
# ---------------------------------------------------------------------------
def _event_ms(fn, reps):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def time_rows(ctx, batch, blocks, gni, hbm, local):
    """Device times of reorder_neighbors, incomplete_cells, the projected DTFE
    step and ProjectGrid, and WriteGrid's file bandwidth, each with its
    algorithmic bytes against the HBM peak."""
    import tempfile
    import torch
    from tess2_gb300.api import DENSE_DTFE, grid_floats
    dev = f"cuda:{local}"
    rows = {}
    T = sum(int(b["tets"].shape[0]) for b in blocks)
    # reorder_neighbors over every block's tets (block-local numbering), neighbours shuffled per tet
    rng = np.random.default_rng(1)
    shuffled = []
    for b in blocks:
        t = b["tets"].copy()
        perm = np.argsort(rng.random((t.shape[0], 4)), axis=1)
        t[:, 4:] = np.take_along_axis(t[:, 4:], perm, axis=1)
        shuffled.append(t)
    src = [torch.from_numpy(t).to(dev) for t in shuffled]
    work = [x.clone() for x in src]

    t_ro = []
    ctx.set_timing(True)
    for _ in range(5):
        for w, x in zip(work, src):
            w.copy_(x)
        torch.cuda.synchronize()
        tot = 0.0
        for w in work:
            ctx.reorder_neighbors_device(w.data_ptr(), w.shape[0])
            tot += sum(m for _, m in ctx.stage_times())
        t_ro.append(tot)
    ctx.set_timing(False)
    ms = statistics.median(t_ro)
    ok = all(np.array_equal(w.cpu().numpy(), b["tets"]) for w, b in zip(work, blocks))
    # bytes: the tet record read and its neighbours written (48 B) + 4 neighbour vertex rows (64 B)
    rb = 112.0 * T
    rows["reorder_neighbors"] = dict(ms=ms, tets=T, tets_per_s=T / (ms * 1e-3), restores_qhull_order=ok,
                                     algorithmic_bytes=rb, achieved_gbs=rb / (ms * 1e-3) / 1e9,
                                     frac=rb / (ms * 1e-3) / 1e9 / hbm)
    # incomplete_cells for every block against the other blocks' boxes
    links = [np.array([np.concatenate([o["bounds_min"], o["bounds_max"]]) for k, o in enumerate(blocks) if k != i],
                      np.float32) for i in range(len(blocks))]
    C = sum(int(b["num_orig"]) for b in blocks)
    dm = torch.zeros(C, dtype=torch.int64, device=dev)
    ctx.set_timing(True)
    t_ic = []
    for _ in range(5):
        enq = batch.incomplete_cells(links, dm.data_ptr())
        t_ic.append(sum(ms for name, ms in ctx.stage_times()))
    ctx.set_timing(False)
    ms = statistics.median(t_ic)
    # bytes: 32 B of tet record + 48 B of vertex positions per tet, 8 B per mask
    ib = 80.0 * T + 8.0 * C
    rows["incomplete_cells"] = dict(ms=ms, tets=T, tets_per_s=T / (ms * 1e-3), enqueued=int(enq.sum()),
                                    algorithmic_bytes=ib, achieved_gbs=ib / (ms * 1e-3) / 1e9,
                                    frac=ib / (ms * 1e-3) / 1e9 / hbm)
    # projected DTFE (x-y plane) and ProjectGrid
    nfl, L = grid_floats(blocks, DENSE_DTFE, gni, project=True)
    gp = torch.empty(nfl, device=dev)
    for _ in range(2):
        batch.dense(DENSE_DTFE, gni, gp.data_ptr(), project=True, want_info=False)
    ctx.set_timing(True)
    batch.dense(DENSE_DTFE, gni, gp.data_ptr(), project=True, want_info=False)
    st = dict(ctx.stage_times())
    ctx.set_timing(False)
    step = _event_ms(lambda: batch.dense(DENSE_DTFE, gni, gp.data_ptr(), project=True, want_info=False), 3)
    G = float(np.prod(gni))
    pl = st.get("project_layers", float("nan"))
    out2 = torch.empty(gni[0] * gni[1], device=dev)
    ps = _event_ms(lambda: ctx.project_grid(gp.data_ptr(), L, gni[0] * gni[1], out2.data_ptr()), 10)
    rows["dtfe_projected"] = dict(ms_per_step=step, layers=L, grid_pts_per_s=G / (step * 1e-3),
                                  project_layers_ms=pl, project_layers_gbs=(4.0 * G + 4.0 * nfl) / (pl * 1e-3) / 1e9,
                                  project_grid_ms=ps)
    # WriteGrid of the 3-D grid: device -> pinned -> file (local disk of the host)
    g3 = torch.empty(int(G), device=dev).uniform_()
    torch.cuda.synchronize()
    d = tempfile.mkdtemp()
    path = os.path.join(d, "grid.raw")
    ctx.write_grid(g3.data_ptr(), int(G), path)
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        ctx.write_grid(g3.data_ptr(), int(G), path)
    tw = (time.perf_counter() - t0) / reps
    ok = os.path.getsize(path) == 4 * int(G)
    os.remove(path)
    os.rmdir(d)
    h = torch.empty(int(G), dtype=torch.float32, pin_memory=True)
    td = _event_ms(lambda: h.copy_(g3, non_blocking=True), 3)
    rows["write_grid"] = dict(bytes=4 * int(G), s=tw, gbs=4 * G / tw / 1e9, size_ok=ok,
                              d2h_pinned_gbs=4 * G / (td * 1e-3) / 1e9, dir=tempfile.gettempdir())
    return rows


# ---------------------------------------------------------------------------
# the surrogate network against the plain path
# ---------------------------------------------------------------------------
def time_surrogate(args, peaks, local, blocks, prep_s):
    """The U-Net surrogate against the plain path at 128^3 (configuration 4's
    grid): the network's forward pass and training step (random weights, CUDA
    events), and the plain DTFE path on this run's own particles onto 128^3 --
    the GPU pass with the tets resident, and with this run's host Delaunay time
    added.  Its error against DTFE comes from --surrogate-train (fields of
    2,097,152 particles; too long for this run)."""
    import torch
    from tess2_gb300 import unet as U
    from tess2_gb300.api import DENSE_DTFE, Context
    side = 128
    t = U.timings(side, reps=10)
    ctx = Context(local)
    batch = ctx.upload(blocks)
    g = torch.empty(side ** 3, device=f"cuda:{local}")
    gni = [side] * 3
    dtfe_ms = U._events_ms(lambda: batch.dense(DENSE_DTFE, gni, g.data_ptr(), want_info=False), 10)
    batch.free()
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    t.update(plain_gpu_ms=dtfe_ms, plain_host_delaunay_s=prep_s,
             fields_per_s=1e3 / t["forward_ms"], plain_gpu_fields_per_s=1e3 / dtfe_ms,
             plain_with_delaunay_fields_per_s=1.0 / (prep_s + dtfe_ms * 1e-3),
             speedup_vs_plain_gpu=dtfe_ms / t["forward_ms"],
             speedup_vs_plain_with_delaunay=(prep_s + dtfe_ms * 1e-3) / (t["forward_ms"] * 1e-3),
             tensor_frac_of_bf16_peak=t["forward_tflops"] / bf16,
             train_tensor_frac_of_bf16_peak=t["train_step_tflops"] / bf16,
             bf16_peak_source="measured MEASURED_PEAKS.json bf16_tflops" if "bf16_tflops" in peaks else "fallback",
             network="U-Net, 4 levels, 32-256 channels, 3x3x3 convolutions, concatenated skips",
             kernels="tcgen05 bf16 implicit GEMM with TMEM accumulators, TMA-fed (forward, data gradient, "
                     "weight gradient)")
    return t


def train_surrogate(args):
    """--surrogate-train: configuration 4 -- fields of 2,097,152 particles
    (--surrogate-particles) -> 128^3 made by the plain path (host Qhull, GPU CIC and DTFE), the U-Net
    trained on them, validated on held-out seeds; one JSON line."""
    from tess2_gb300 import unet as U
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    log = lambda m: print("# " + m, flush=True)
    r = U.train_and_evaluate(n_train=args.surrogate_fields, n_val=args.surrogate_val,
                             n_particles=args.surrogate_particles, side=128,
                             epochs=args.surrogate_epochs, lr=args.surrogate_lr, log=log)
    r.pop("net")
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    r.update(metric="surrogate validation relative L2 of log(1 + rho / mean) vs DTFE, 128^3",
             value=r["val_rel_l2"], unit="relative L2", higher_is_better=False,
             tensor_frac_of_bf16_peak=r["forward_tflops"] / bf16,
             fields_per_s=1e3 / r["forward_ms"],
             plain_with_delaunay_fields_per_s=(args.surrogate_fields + args.surrogate_val) / r["fields_wall_s"],
             data="synthetic: seeded particle sets, 50% uniform + 50% in 256 clumps sigma 0.01")
    print(json.dumps(r), flush=True)


# ---------------------------------------------------------------------------
# parity at the benchmark's size, on samples the CPU oracle can recompute
# ---------------------------------------------------------------------------
def full_size_parity(ctx, blocks, gni, grid, DENSE_DTFE, DENSE_TESS, MODE_MIXED, MODE_FP64, stride=16,
                     cells_per_block=1000):
    """DTFE owners and values of every 16th tet of each block against the FP64
    oracle (mixed and FP64 modes), and the DENSE_TESS per-cell grid-point
    counts of a seeded random sample of every block's cells against the
    restated reference (oracle/parity.py)."""
    import torch
    from oracle import parity
    t0 = time.perf_counter()
    G = grid.numel()
    b = ctx.upload(blocks)
    b.keep_debug(True)
    out = {}
    for mode in (MODE_MIXED, MODE_FP64):
        b.dense(DENSE_DTFE, gni, grid.data_ptr(), mode=mode, want_info=False)
        _, own, _ = b.debug_outputs(grid_points=G)
        out[mode] = (grid.cpu().numpy(), own)
    total = sum(int(x["num_orig"]) for x in blocks)
    b.dense(DENSE_TESS, gni, grid.data_ptr(), want_info=False)
    counts, _, _ = b.debug_outputs(cells=total)
    b.free()
    torch.cuda.synchronize()
    smp = parity.dtfe_oracle_sample(blocks, gni, stride)
    res = {}
    for mode, name, tol in ((MODE_MIXED, "dtfe_mixed", 1e-6), (MODE_FP64, "dtfe_fp64", 1e-12)):
        r = parity.dtfe_compare(out[mode][0], out[mode][1], smp, stride)
        r["bound"] = tol
        r["ok"] = bool(r["owners_equal"] and r["no_extra"] and r["rel_l2"] <= tol)
        res[name] = r
    del out, smp
    cells = parity.tess_cell_sample(blocks, cells_per_block, seed=11)
    ref = parity.tess_counts_oracle(blocks, gni, cells)
    off, same, n = 0, 0, 0
    for blk, c, r in zip(blocks, cells, ref):
        same += int(np.count_nonzero(counts[off + c] == r))
        n += int(c.size)
        off += int(blk["num_orig"])
    res["dense_tess_cell_counts"] = dict(cells=n, equal=same, ok=same == n, seed=11,
                                         sample=f"{cells_per_block} random cells of each block")
    res["seconds"] = time.perf_counter() - t0
    return res


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    # host Qhull in spawned processes before the first CUDA call
    blocks, prep_s = prepare(args)
    import torch
    from tess2_gb300 import build as tbuild
    tbuild.build()
    from tess2_gb300.api import DENSE_DTFE, DENSE_TESS, MODE_FP64, MODE_MIXED, Context
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    gni = [args.grid] * 3
    G = int(np.prod(gni))
    cfg = workload_config(args, blocks)
    T, N = cfg["tets"], cfg["particles_with_ghosts"]

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    ctx = Context(local)
    batch = ctx.upload(blocks)
    grid = torch.empty(G, dtype=torch.float32, device=f"cuda:{local}")
    gptr = grid.data_ptr()

    def step(mode=MODE_MIXED):
        batch.dense(DENSE_DTFE, gni, gptr, mode=mode, want_info=False)

    # untimed warm-up
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.5)   # nvidia-smi needs a moment before its first sample
    for _ in range(2):   # keep the GPU busy while the sampler starts
        step()
    torch.cuda.synchronize()
    launches0 = ctx.launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    ev0.record()
    for _ in range(args.steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    launches = ctx.launches() - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    if dist is not None:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * G / (ms * 1e-3)

    # kernel times: the same step with its stages run one after the other over
    # all blocks (TESSGPU_BATCH_OVERLAP=0), CUDA events between the stages on
    # the launching stream; the timed steps above interleave blocks on two
    # streams, where a kernel's own duration is not defined
    os.environ["TESSGPU_BATCH_OVERLAP"] = "0"
    ctx.set_timing(True)
    stage_sum = {}
    ks = max(3, args.steps // 2)
    try:
        for _ in range(ks):
            step()
            for name, sms in ctx.stage_times():
                stage_sum[name] = stage_sum.get(name, 0.0) + sms
    finally:
        ctx.set_timing(False)
        os.environ.pop("TESSGPU_BATCH_OVERLAP", None)
    stage_ms = {k: v / ks for k, v in stage_sum.items()}
    stage_ms["serial_step"] = sum(stage_ms.values())

    # the step's DTFE accounting (one more untimed call with info)
    info = batch.dense(DENSE_DTFE, gni, gptr, mode=MODE_MIXED, want_info=True)
    mixed = grid.clone()

    extra = {}
    if not args.no_extra:
        # plain FP64 GPU path: the comparison target, and the accuracy reference at full size
        for _ in range(2):
            step(MODE_FP64)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        k64 = max(2, args.steps // 3)
        e0.record()
        for _ in range(k64):
            step(MODE_FP64)
        e1.record()
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1) / k64
        info64 = batch.dense(DENSE_DTFE, gni, gptr, mode=MODE_FP64, want_info=True)
        d = (mixed.double() - grid.double()).norm() / grid.double().norm()
        extra["fp64_mode"] = dict(value=G / (ms64 * 1e-3), unit=UNIT, ms_per_step=ms64,
                                  grid_pts_assigned=info64["grid_pts_assigned"])
        extra["mixed_speedup_vs_fp64"] = ms64 / ms
        extra["mixed_vs_fp64_rel_l2"] = float(d)
        extra["owners_identical"] = info64["grid_pts_assigned"] == info["grid_pts_assigned"]
        # the reference's estimator on the GPU (DENSE_TESS), same blocks and grid
        batch.dense(DENSE_TESS, gni, gptr, want_info=False)
        torch.cuda.synchronize()
        e0.record()
        kt = 2
        for _ in range(kt):
            batch.dense(DENSE_TESS, gni, gptr, want_info=False)
        e1.record()
        torch.cuda.synchronize()
        mst = e0.elapsed_time(e1) / kt
        it = batch.dense(DENSE_TESS, gni, gptr, want_info=True)
        # its roofline: 12 B/particle + 32 B/tet + 4 B/grid point of HBM, and
        # 8 FP32 operations per face-plane test (probes x faces); no measured
        # FP32 peak exists, so the nominal 152 SMs x 128 lanes x 2 x 2.07 GHz
        tb = 12.0 * N + 32.0 * T + 4.0 * G
        tf = 8.0 * it["face_tests"]
        fp32_nominal = 152 * 128 * 2 * 2.07e9
        extra["dense_tess_gpu"] = dict(value=G / (mst * 1e-3), unit=UNIT, ms_per_step=mst,
                                       cells_deposited=it["check_mass"], cell_probes=it["cell_probes"],
                                       face_tests=it["face_tests"], algorithmic_bytes=tb,
                                       achieved_gbs=tb / (mst * 1e-3) / 1e9, hbm_frac=tb / (mst * 1e-3) / 1e9 / hbm,
                                       achieved_gflops=tf / (mst * 1e-3) / 1e9,
                                       fp32_frac_of_nominal=tf / (mst * 1e-3) / fp32_nominal)
        # Voronoi cell volumes as the reference computes them (float,
        # bit-identical to its volume()) against FP64 cell volumes, for
        # block 0's own particles
        b0 = blocks[0]
        n0 = int(b0["num_orig"])
        v32 = ctx.volume(b0["vert_to_tet"], b0["tets"], b0["particles"], n=n0)
        v64 = ctx.volume_f64(b0["vert_to_tet"], b0["tets"], b0["particles"], n=n0)
        fin = (v32 > 0) & (v64 > 0)
        dv = v32[fin].astype(np.float64) - v64[fin]
        extra["cell_volume_vs_fp64"] = dict(
            cells=n0, finite=int(fin.sum()), rel_l2=float(np.linalg.norm(dv) / max(np.linalg.norm(v64[fin]), 1e-300)),
            max_rel=float(np.max(np.abs(dv) / v64[fin])) if fin.any() else 0.0,
            infinite_cells_agree=bool(np.array_equal(v32 < 0, v64 < 0)),
            sample="block 0's own particles; float volumes bit-identical to the reference's volume()")

    # roofline of the dominant kernel: the mixed rasteriser.  Algorithmic bytes
    # per launch of the brick kernel: the pair list 4 B per (tet, brick) pair,
    # tet vertex indices 16 B per tet, particle position 16 B and density 4 B
    # per particle (each read once), 4 B per grid point written (every point of
    # the blocks' boxes, zeros included); the row kernel writes only the
    # assigned points (the grid is zeroed by a separate memset).
    assigned = info["grid_pts_assigned"]
    pairs = info.get("brick_pairs", 0)
    if pairs:
        raster_bytes = 4.0 * pairs + 16.0 * T + 20.0 * N + 4.0 * G
        rkernel = "k_raster_bricks<float,...> (mixed DTFE brick rasteriser), duration from the serial stage pass"
    else:
        raster_bytes = 16.0 * T + 20.0 * N + 4.0 * assigned
        rkernel = "k_raster<float,...> (mixed DTFE row rasteriser), duration from the serial stage pass"

    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    r_ms = stage_ms.get("raster", float("nan"))
    achieved = raster_bytes / (r_ms * 1e-3) / 1e9
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "dtfe_raster_traffic.json")))
        if prof.get("grid") == args.grid and prof.get("particles") == args.particles and \
                bool(prof.get("brick", False)) == bool(pairs):
            traffic = prof.get("dram_bytes_per_launch")
    except Exception:
        pass
    roofline = dict(bound="hbm", kernel=rkernel, achieved=achieved, peak=hbm,
                    unit="GB/s", frac=achieved / hbm, traffic=traffic, algorithmic_bytes=raster_bytes,
                    kernel_ms=r_ms, peak_source=peak_src + " MEASURED_PEAKS.json hbm_gbs" if peak_src == "measured"
                    else "fallback 6.8 TB/s")
    # the whole step against the same peak: 32 B/tet + 64 B/particle + 8 B/grid point
    step_bytes = 32.0 * T + 64.0 * N + 8.0 * G
    step_roof = dict(algorithmic_bytes=step_bytes, achieved=step_bytes / (ms * 1e-3) / 1e9, frac=
                     step_bytes / (ms * 1e-3) / 1e9 / hbm)

    # end to end through the host-buffer call
    e2e = None
    if not args.no_e2e:
        pinned = []
        hblocks = []
        for b in blocks:
            nb = dict(b)
            nb.pop("vert_to_tet", None)   # DTFE does not read it; the call gets tess2's particles and tets
            for k in ("particles", "tets"):
                a = np.ascontiguousarray(b[k])
                t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0]).dtype, pin_memory=True)
                t.numpy()[...] = a
                pinned.append(t)
                nb[k] = t.numpy()
            hblocks.append(nb)
        out = torch.empty((args.grid,) * 3, dtype=torch.float32, pin_memory=True).numpy()
        for _ in range(2):
            ctx.dense(DENSE_DTFE, hblocks, gni, out=out)
        ke = max(2, args.steps // 2)
        t0 = time.perf_counter()
        for _ in range(ke):
            ctx.dense(DENSE_DTFE, hblocks, gni, out=out)
        te = (time.perf_counter() - t0) / ke
        h2d = sum(b["particles"].nbytes + b["tets"].nbytes for b in blocks)
        # the same call on pageable host memory, as tess2's malloc'd block
        # arrays and new[]'d density array are
        pblocks = []
        for b in blocks:
            nb = dict(b)
            nb.pop("vert_to_tet", None)
            nb["particles"] = np.array(b["particles"], copy=True)
            nb["tets"] = np.array(b["tets"], copy=True)
            pblocks.append(nb)
        pout = np.empty((args.grid,) * 3, np.float32)
        for _ in range(2):
            ctx.dense(DENSE_DTFE, pblocks, gni, out=pout)
        t0 = time.perf_counter()
        for _ in range(ke):
            ctx.dense(DENSE_DTFE, pblocks, gni, out=pout)
        tp = (time.perf_counter() - t0) / ke
        if args.e2e_spans:
            spans = {}
            for name, bl, o in (("pinned", hblocks, out), ("pageable", pblocks, pout),
                                ("pageable in, pinned out", pblocks, out), ("pinned in, pageable out", hblocks, pout)):
                ctx.dense(DENSE_DTFE, bl, gni, out=o)
                runs = []
                ctx.set_timing(True)
                for _ in range(5):   # the call with the median time to the last block
                    ctx.dense(DENSE_DTFE, bl, gni, out=o)
                    runs.append({k: round(v, 3) for k, v in ctx.stage_times()})
                ctx.set_timing(False)
                runs.sort(key=lambda r: r.get("blocks_done", 0.0) + r.get("downloads_done", 0.0))
                spans[name] = runs[len(runs) // 2]
            print("# e2e spans " + json.dumps(spans), flush=True)
        e2e = dict(value=G / te, unit=UNIT, ms_per_step=te * 1e3, h2d_bytes_per_step=int(h2d),
                   d2h_bytes_per_step=int(4 * G), api="tessgpu_dense (host buffers, pinned)",
                   pageable=dict(value=G / tp, ms_per_step=tp * 1e3,
                                 api="tessgpu_dense (pageable numpy arrays, as tess2's malloc/new[] buffers)"))
        del pblocks, pout

    rows = None
    if not args.no_rows:
        rows = time_rows(ctx, batch, blocks, gni, hbm, local)
        extra["rows"] = rows
    if not args.no_surrogate:
        extra["surrogate"] = time_surrogate(args, peaks, local, blocks, prep_s)

    parity = None
    if rank == 0 and not args.no_parity:
        parity = full_size_parity(ctx, blocks, gni, grid, DENSE_DTFE, DENSE_TESS, MODE_MIXED, MODE_FP64)
    if rank == 0 and not args.no_extra and not args.no_cpu:
        # the reference's estimator on the host cores: the like-for-like pair of dense_tess_gpu
        dt, _ = dense_tess_cpu(blocks, gni, steps=3, warmup=1)
        extra["dense_tess_cpu"] = dt
        if "dense_tess_gpu" in extra:
            extra["dense_tess_gpu_over_cpu"] = extra["dense_tess_gpu"]["value"] / dt["value"]

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            cpu = dtfe_cpu_baseline(blocks, gni)
        except Exception as e:  # the baseline is reported, never the product path
            cpu = dict(value=None, unit=UNIT, cores=1, kind="port", sample=f"failed: {e}")

    if rank == 0:
        # the long detail objects on a comment line first; the JSON line itself stays short
        details = dict(rows=extra.pop("rows", None), surrogate=extra.get("surrogate"),
                       raster_variant_ms=info["raster_variant_ms"], config=cfg)
        print("# details " + json.dumps(details), flush=True)
        sur = extra.pop("surrogate", None)
        if sur:
            extra["surrogate"] = {k: sur.get(k) for k in ("forward_ms", "fields_per_s", "speedup_vs_plain_gpu",
                                                          "speedup_vs_plain_with_delaunay", "forward_tflops",
                                                          "tensor_frac_of_bf16_peak", "train_step_ms",
                                                          "train_step_tflops")}
        cfg_short = {k: cfg[k] for k in ("workload", "particles", "particles_with_ghosts", "tets", "blocks", "mode",
                                         "l2")}
        line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
                    ms_per_step=ms, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
                    data="synthetic", config=cfg_short, roofline=roofline, cpu_baseline=cpu, e2e=e2e,
                    gpu_launches=int(launches), clocks=clk, particles_per_s=world * args.particles / (ms * 1e-3),
                    stage_ms=stage_ms, step_roofline=step_roof, parity=parity, fp64_fixup_tets=info["fp64_tets"],
                    exact_tests=info["exact_tests"], grid_pts_assigned=assigned, brick_pairs=pairs,
                    rows_visited=info["rows_visited"], points_tested=info["points_tested"],
                    raster_variant=info["raster_variant"], host_prep_s=prep_s, **extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# batched independent sets (uneven blocks, each with its own grid)
# ---------------------------------------------------------------------------
def _set_particles(seed_n):
    from tess2_gb300 import host
    seed, n = seed_n
    pts = host.mixture_particles(n, seed, frac_uniform=0.5, n_clumps=256, sigma=0.01)
    return pts, host.delaunay_tets(pts)


def make_sets(nsets, seed):
    """nsets particle sets: counts log-uniform in [1e4, 5e5], the benchmark's
    mixture at seed + i, grid side uniform in {64, 128, 192, 256}."""
    from tess2_gb300 import host
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(1e4), np.log(5e5), nsets)).astype(int)
    sides = rng.choice([64, 128, 192, 256], nsets)
    with mp.get_context("spawn").Pool(min(nsets, os.cpu_count() or 1)) as pool:
        res = pool.map(_set_particles, [(seed + 1 + i, int(c)) for i, c in enumerate(counts)])
    blocks = []
    for i, (pts, tets) in enumerate(res):
        blocks.append(dict(gid=i, particles=pts, tets=tets, vert_to_tet=host.vert_to_tet_host(len(pts), tets),
                           num_orig=len(pts), bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
                           data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32)))
    gni = [[int(x)] * 3 for x in sides]
    return blocks, gni


def run_sets(args):
    import torch
    from tess2_gb300 import build as tbuild
    t0 = time.time()
    blocks, gni = make_sets(args.sets, args.seed)
    prep_s = time.time() - t0
    tbuild.build()
    from tess2_gb300.api import Context, MODE_FP64, MODE_MIXED, sets_offsets
    ctx = Context(0)
    total, off = sets_offsets(gni)
    b = ctx.upload(blocks)
    out = torch.empty(total, dtype=torch.float32, device="cuda:0")
    info = b.dense_sets(gni, out.data_ptr())                 # picks the brick shape
    for _ in range(args.warmup):
        b.dense_sets(gni, out.data_ptr(), graph=True, want_info=False)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(0.5)
    for _ in range(2):
        b.dense_sets(gni, out.data_ptr(), graph=True, want_info=False)
    torch.cuda.synchronize()
    l0 = ctx.launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        b.dense_sets(gni, out.data_ptr(), graph=True, want_info=False)
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    launches = (ctx.launches() - l0) / args.steps
    info = b.dense_sets(gni, out.data_ptr(), graph=True)
    # the same sets one call per set (one block each, no graph) for comparison
    one = []
    singles = [ctx.upload([blk]) for blk in blocks]
    from tess2_gb300.api import DENSE_DTFE
    for rep in range(3):
        torch.cuda.synchronize()
        e0.record()
        for i, sb in enumerate(singles):
            sb.dense(DENSE_DTFE, gni[i], out.data_ptr() + 4 * int(off[i]), want_info=False)
        e1.record()
        torch.cuda.synchronize()
        one.append(e0.elapsed_time(e1))
    for sb in singles:
        sb.free()
    # parity: every set's grid against the FP64 oracle (every 16th tet) on a sample of sets
    par = None
    if not args.no_parity:
        from oracle import parity
        got = out.cpu().numpy()
        rng = np.random.default_rng(3)
        pick = sorted(rng.choice(len(blocks), size=min(6, len(blocks)), replace=False).tolist())
        worst = 0.0
        ok = True
        for i in pick:
            n = int(np.prod(gni[i]))
            smp = parity.dtfe_oracle_sample([blocks[i]], gni[i], 16, processes=1)
            idx, own, val = smp
            g = got[off[i]:off[i] + n][idx].astype(np.float64)
            v = val.astype(np.float64)
            r = float(np.linalg.norm(g - v) / max(np.linalg.norm(v), 1e-300))
            worst = max(worst, r)
            ok = ok and r <= 1e-6
        par = dict(sets_checked=pick, worst_rel_l2_vs_fp64=worst, bound=1e-6, ok=ok,
                   sample="every 16th tet of each checked set, FP64 oracle")
    N = sum(len(x["particles"]) for x in blocks)
    T = sum(len(x["tets"]) for x in blocks)
    line = dict(metric="DTFE grid pts/s, batched uneven sets (one persistent launch, CUDA graph)",
                value=total / (ms * 1e-3), unit="grid_pts/s", n_gpus=1, steps=args.steps, warmup=args.warmup,
                ms_per_step=ms, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
                data="synthetic",
                config=dict(workload=f"{args.sets} independent sets, counts log-uniform in [1e4, 5e5] (50% uniform + "
                                     f"50% 256 clumps sigma 0.01 each), grids of side 64/128/192/256",
                            particles=N, tets=T, grid_points=total, sides=[g[0] for g in gni]),
                particles_per_s=N / (ms * 1e-3), kernels_per_step=launches, graph_launches_per_step=1,
                raster_launches_per_step=1, raster_variant=info["raster_variant"],
                raster_variant_ms=info["raster_variant_ms"], brick_pairs=info["brick_pairs"],
                one_call_per_set_ms=min(one), speedup_vs_one_call_per_set=min(one) / ms,
                clocks=clk, parity=par, host_prep_s=prep_s)
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.surrogate_train:
        train_surrogate(args)
    elif args.sets:
        run_sets(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
