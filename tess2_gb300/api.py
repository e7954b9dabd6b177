"""Python mirror of tess2's geometry/density interface over the C ABI
(include/tess2_gb300.h).  Names and argument meanings follow the reference:

  fill_vert_to_tet   src/tess.cpp:767-787
  fill_circumcenters src/volume.cpp:6-11      (circumcenter, src/tet.cpp:37-66)
  complete           src/tet.cpp:337-378      (all vertices at once)
  volume             src/volume.cpp:13-54     (all vertices at once)
  dense              src/dense.cpp:30-103     (DENSE_TESS, DENSE_CIC, plus DENSE_DTFE; project)
  ProjectGrid        src/dense.cpp:881-1023   (project_grid)
  WriteGrid          src/dense.cpp:751-870    (write_grid, write_last_grid)
  reorder_neighbors  src/tess-qhull.c:161-225
  incomplete_cells   src/tess.cpp:492-628

Everything runs in libtess2_gb300.so on the GPU; there is no CPU fallback.
If the library is missing the calls raise.
"""
import ctypes
import os

import numpy as np

from . import build as _build

DENSE_TESS, DENSE_CIC, DENSE_DTFE = 0, 1, 2
MODE_MIXED, MODE_FP64 = 0, 1

_STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "no CUDA device", 4: "star overflow",
           5: "face overflow", 6: "edge ring overflow", 7: "malformed mesh", 8: "unsupported", 9: "I/O error",
           10: "a bounded wait inside a kernel ran out", 11: "a device work list outgrew its buffer"}


class TessGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"tessgpu status {code} ({_STATUS.get(code, '?')}): {msg}")
        self.code = code


class Block(ctypes.Structure):
    """tessgpu_block"""
    _fields_ = [("gid", ctypes.c_int),
                ("bounds_min", ctypes.c_float * 3), ("bounds_max", ctypes.c_float * 3),
                ("data_min", ctypes.c_float * 3), ("data_max", ctypes.c_float * 3),
                ("num_orig_particles", ctypes.c_int), ("num_particles", ctypes.c_int),
                ("particles", ctypes.c_void_p), ("num_tets", ctypes.c_int),
                ("tets", ctypes.c_void_p), ("vert_to_tet", ctypes.c_void_p)]


class Link(ctypes.Structure):
    """tessgpu_link: a neighbour's core bounds and wrap direction"""
    _fields_ = [("bounds_min", ctypes.c_float * 3), ("bounds_max", ctypes.c_float * 3), ("wrap", ctypes.c_int * 3)]


def make_links(links6, wrap3=None):
    """ctypes array of Link from (L, 6) boxes (min xyz, max xyz) and optional (L, 3) wraps."""
    l6 = np.asarray(links6, np.float32).reshape(-1, 6)
    arr = (Link * max(len(l6), 1))()
    for i, row in enumerate(l6):
        for d in range(3):
            arr[i].bounds_min[d] = row[d]
            arr[i].bounds_max[d] = row[3 + d]
            arr[i].wrap[d] = 0 if wrap3 is None else int(np.asarray(wrap3).reshape(-1, 3)[i][d])
    return arr


class DenseParams(ctypes.Structure):
    """tessgpu_dense_params"""
    _fields_ = [("alg", ctypes.c_int), ("mode", ctypes.c_int), ("num_given_bounds", ctypes.c_int),
                ("given_mins", ctypes.c_float * 3), ("given_maxs", ctypes.c_float * 3),
                ("mass", ctypes.c_float), ("eps", ctypes.c_float), ("glo_num_idx", ctypes.c_int * 3),
                ("use_data_bounds", ctypes.c_int), ("data_mins", ctypes.c_float * 3),
                ("data_maxs", ctypes.c_float * 3), ("project", ctypes.c_int)]


class DenseInfo(ctypes.Structure):
    """tessgpu_dense_info"""
    _fields_ = [("data_mins", ctypes.c_float * 3), ("data_maxs", ctypes.c_float * 3),
                ("grid_phys_mins", ctypes.c_float * 3), ("grid_phys_maxs", ctypes.c_float * 3),
                ("grid_step_size", ctypes.c_float * 3),
                ("max_dense", ctypes.c_double), ("tot_mass", ctypes.c_double), ("check_mass", ctypes.c_double),
                ("grid_pts_assigned", ctypes.c_longlong), ("fp64_tets", ctypes.c_longlong),
                ("exact_tests", ctypes.c_longlong), ("rows_visited", ctypes.c_longlong),
                ("points_tested", ctypes.c_longlong), ("raster_variant", ctypes.c_int),
                ("raster_variant_ms", ctypes.c_float * 8), ("grid_layers", ctypes.c_int),
                ("grid_floats", ctypes.c_longlong), ("cell_probes", ctypes.c_longlong),
                ("face_tests", ctypes.c_longlong), ("brick_pairs", ctypes.c_longlong)]

    def as_dict(self):
        return dict(data_mins=np.array(self.data_mins[:], np.float32), data_maxs=np.array(self.data_maxs[:], np.float32),
                    grid_phys_mins=np.array(self.grid_phys_mins[:], np.float32),
                    grid_phys_maxs=np.array(self.grid_phys_maxs[:], np.float32),
                    grid_step_size=np.array(self.grid_step_size[:], np.float32),
                    max_dense=self.max_dense, tot_mass=self.tot_mass, check_mass=self.check_mass,
                    grid_pts_assigned=self.grid_pts_assigned, fp64_tets=self.fp64_tets,
                    exact_tests=self.exact_tests, rows_visited=self.rows_visited,
                    points_tested=self.points_tested, raster_variant=self.raster_variant,
                    raster_variant_ms=list(self.raster_variant_ms), grid_layers=self.grid_layers,
                    grid_floats=self.grid_floats, cell_probes=self.cell_probes, face_tests=self.face_tests,
                    brick_pairs=self.brick_pairs)


_LIB = None
_VP = ctypes.c_void_p
_I = ctypes.c_int


def library_path():
    return _build.LIB


def lib():
    """The loaded libtess2_gb300.so (raises when it has not been built)."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing: build it with tess2_gb300.build.build()")
        L = ctypes.CDLL(path)
        sig = {
            "tessgpu_create": (_I, [_I, _VP, ctypes.POINTER(_VP)]),
            "tessgpu_destroy": (None, [_VP]),
            "tessgpu_last_error": (ctypes.c_char_p, [_VP]),
            "tessgpu_sync": (_I, [_VP]),
            "tessgpu_launch_count": (ctypes.c_longlong, [_VP]),
            "tessgpu_fill_vert_to_tet": (_I, [_VP, _I, _VP, _I, _VP]),
            "tessgpu_fill_circumcenters": (_I, [_VP, _VP, _I, _VP, _I, _VP]),
            "tessgpu_complete_all": (_I, [_VP, _VP, _I, _VP, _I, _VP, _I, _VP]),
            "tessgpu_volumes": (_I, [_VP, _VP, _I, _VP, _I, _VP, _I, _VP, _VP]),
            "tessgpu_volumes_f64": (_I, [_VP, _VP, _I, _VP, _I, _VP, _I, _VP]),
            "tessgpu_dense": (_I, [_VP, _I, _VP, _VP, _VP, _VP, _VP]),
            "tessgpu_block_grid_points": (ctypes.c_longlong, [_I, _VP, _I, _VP, _VP]),
            "tessgpu_batch_upload": (_I, [_VP, _I, _VP, ctypes.POINTER(_VP)]),
            "tessgpu_batch_wrap_device": (_I, [_VP, _I, _VP, ctypes.POINTER(_VP)]),
            "tessgpu_batch_free": (None, [_VP]),
            "tessgpu_batch_dense": (_I, [_VP, _VP, _VP, _VP, _VP]),
            "tessgpu_batch_keep_debug": (_I, [_VP, _I]),
            "tessgpu_batch_debug_outputs": (_I, [_VP, _VP, _VP, _VP, _VP]),
            "tessgpu_set_timing": (_I, [_VP, _I]),
            "tessgpu_reorder_neighbors": (_I, [_VP, _VP, _I]),
            "tessgpu_reorder_neighbors_device": (_I, [_VP, _VP, _I]),
            "tessgpu_stage_times": (_I, [_VP, _VP, _VP, _I]),
            "tessgpu_dtfe_densities_noalloc": (_I, [_VP, _I, _VP, _I, _VP, ctypes.c_float, _I, _VP, _VP]),
            "tessgpu_dense_grid_floats": (ctypes.c_longlong, [_I, _VP, _VP, _VP]),
            "tessgpu_project_grid": (_I, [_VP, _VP, _I, ctypes.c_longlong, _VP]),
            "tessgpu_write_grid": (_I, [_VP, _VP, ctypes.c_longlong, ctypes.c_char_p]),
            "tessgpu_write_last_grid": (_I, [_VP, ctypes.c_char_p]),
            "tessgpu_incomplete_cells": (_I, [_VP, _VP, _I, _VP, _I, _VP, _VP]),
            "tessgpu_batch_incomplete_cells": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, _VP]),
            "tessgpu_sets_grid_floats": (ctypes.c_longlong, [_I, _VP, _VP]),
            "tessgpu_batch_dense_sets": (_I, [_VP, _VP, _VP, ctypes.c_float, ctypes.c_float, _I, _VP, _I, _VP]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data


def make_blocks(blocks):
    """blocks: dicts with particles (N,3) f32, tets (T,8) i32, optional
    vert_to_tet (N,) i32, num_orig, bounds_min/max, data_min/max, gid."""
    arr = (Block * len(blocks))()
    keep = []
    for i, b in enumerate(blocks):
        p = np.ascontiguousarray(b["particles"], dtype=np.float32)
        t = np.ascontiguousarray(b["tets"], dtype=np.int32).reshape(-1, 8)
        v = b.get("vert_to_tet")
        v = None if v is None else np.ascontiguousarray(v, dtype=np.int32)
        keep += [p, t, v]
        blk = arr[i]
        blk.gid = int(b.get("gid", i))
        for d in range(3):
            blk.bounds_min[d] = b["bounds_min"][d]
            blk.bounds_max[d] = b["bounds_max"][d]
            blk.data_min[d] = b.get("data_min", b["bounds_min"])[d]
            blk.data_max[d] = b.get("data_max", b["bounds_max"])[d]
        blk.num_orig_particles = int(b.get("num_orig", p.shape[0]))
        blk.num_particles = int(p.shape[0])
        blk.particles = p.ctypes.data
        blk.num_tets = int(t.shape[0])
        blk.tets = t.ctypes.data
        blk.vert_to_tet = None if v is None else v.ctypes.data
    return arr, keep


def make_params(alg, glo_num_idx, mass=1.0, eps=1e-4, mode=MODE_MIXED, given=None, data_bounds=None,
                project=False):
    """data_bounds=(mins, maxs) fixes dense()'s data bounds (every rank's all-reduced
    bounds when this process holds a share of the blocks); project projects onto
    the x-y plane (dense()'s project flag)."""
    p = DenseParams()
    p.project = 1 if project else 0
    if data_bounds is not None:
        p.use_data_bounds = 1
        for d in range(3):
            p.data_mins[d] = data_bounds[0][d]
            p.data_maxs[d] = data_bounds[1][d]
    p.alg = int(alg)
    p.mode = int(mode)
    if given is not None:
        p.num_given_bounds = 3
        for d in range(3):
            p.given_mins[d] = given[0][d]
            p.given_maxs[d] = given[1][d]
    p.mass = mass
    p.eps = eps
    for d in range(3):
        p.glo_num_idx[d] = int(glo_num_idx[d])
    return p


class Context:
    """tessgpu_ctx on one CUDA device; stream is a cudaStream_t handle or None."""

    def __init__(self, device=0, stream=None):
        self._h = _VP()
        s = lib().tessgpu_create(device, stream, ctypes.byref(self._h))
        if s != 0:
            raise TessGpuError(s, "tessgpu_create failed")

    def close(self):
        if self._h:
            lib().tessgpu_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s):
        if s != 0:
            raise TessGpuError(s, lib().tessgpu_last_error(self._h).decode())

    @property
    def handle(self):
        return self._h

    def launches(self):
        return lib().tessgpu_launch_count(self._h)

    def set_timing(self, on=True):
        self._check(lib().tessgpu_set_timing(self._h, 1 if on else 0))

    def stage_times(self):
        """[(stage, ms)] of the last dense call (CUDA events on the context's stream)."""
        names = (ctypes.c_char_p * 32)()
        ms = (ctypes.c_float * 32)()
        n = lib().tessgpu_stage_times(self._h, names, ms, 32)
        return [(names[i].decode(), float(ms[i])) for i in range(n)]

    # --- reference-named calls -------------------------------------------
    def fill_vert_to_tet(self, num_particles, tets):
        tets = np.ascontiguousarray(tets, np.int32)
        out = np.empty(num_particles, np.int32)
        self._check(lib().tessgpu_fill_vert_to_tet(self._h, num_particles, _p(tets), tets.shape[0], _p(out)))
        return out

    def reorder_neighbors(self, tets):
        """reorder_neighbors (src/tess-qhull.c:161-225) on a copy of (T, 8) tet_t records."""
        out = np.array(tets, dtype=np.int32, copy=True, order="C")
        self._check(lib().tessgpu_reorder_neighbors(self._h, _p(out), out.shape[0]))
        return out

    def reorder_neighbors_device(self, d_tets, num_tets):
        """in place on tet_t records in device memory (address d_tets)"""
        self._check(lib().tessgpu_reorder_neighbors_device(self._h, ctypes.c_void_p(d_tets), num_tets))

    def incomplete_cells(self, block, links6, wrap3=None, last_neighbor=0):
        """incomplete_cells (src/tess.cpp:492-628) for one host block: (masks, enqueued),
        masks a uint64 per original particle with bit i set to send it to link i."""
        arr, keep = make_blocks([block])
        links = make_links(links6, wrap3)
        nl = int(np.asarray(links6).size // 6)
        masks = np.zeros(max(arr[0].num_orig_particles, 1), np.uint64)
        enq = ctypes.c_longlong()
        self._check(lib().tessgpu_incomplete_cells(self._h, arr, nl, links, int(last_neighbor), _p(masks),
                                                   ctypes.byref(enq)))
        del keep
        return masks[:arr[0].num_orig_particles], int(enq.value)

    def fill_circumcenters(self, tets, particles):
        tets = np.ascontiguousarray(tets, np.int32)
        particles = np.ascontiguousarray(particles, np.float32)
        out = np.empty((tets.shape[0], 3), np.float32)
        self._check(lib().tessgpu_fill_circumcenters(self._h, _p(particles), particles.shape[0], _p(tets),
                                                     tets.shape[0], _p(out)))
        return out

    def complete(self, tets, vert_to_tet, particles, n=None):
        tets = np.ascontiguousarray(tets, np.int32)
        v = np.ascontiguousarray(vert_to_tet, np.int32)
        particles = np.ascontiguousarray(particles, np.float32)
        n = v.shape[0] if n is None else n
        out = np.empty(n, np.int32)
        self._check(lib().tessgpu_complete_all(self._h, _p(particles), particles.shape[0], _p(tets), tets.shape[0],
                                               _p(v), n, _p(out)))
        return out

    def volume(self, vert_to_tet, tets, particles, n=None, areas=False):
        tets = np.ascontiguousarray(tets, np.int32)
        v = np.ascontiguousarray(vert_to_tet, np.int32)
        particles = np.ascontiguousarray(particles, np.float32)
        n = v.shape[0] if n is None else n
        out = np.empty(n, np.float32)
        ar = np.empty(n, np.float32) if areas else None
        self._check(lib().tessgpu_volumes(self._h, _p(particles), particles.shape[0], _p(tets), tets.shape[0], _p(v),
                                          n, _p(out), _p(ar)))
        return (out, ar) if areas else out

    def volume_f64(self, vert_to_tet, tets, particles, n=None):
        tets = np.ascontiguousarray(tets, np.int32)
        v = np.ascontiguousarray(vert_to_tet, np.int32)
        particles = np.ascontiguousarray(particles, np.float32)
        n = v.shape[0] if n is None else n
        out = np.empty(n, np.float64)
        self._check(lib().tessgpu_volumes_f64(self._h, _p(particles), particles.shape[0], _p(tets), tets.shape[0],
                                              _p(v), n, _p(out)))
        return out

    def dense(self, alg, blocks, glo_num_idx, mass=1.0, eps=1e-4, mode=MODE_MIXED, given=None, block_arrays=False,
              global_grid=True, out=None, data_bounds=None, project=False):
        """dense() over host blocks.  Returns dict(grid=(nz,ny,nx) float32 -- (ny,nx)
        when projecting, after ProjectGrid -- info=..., blocks=[...])."""
        arr, keep = make_blocks(blocks)
        p = make_params(alg, glo_num_idx, mass, eps, mode, given, data_bounds, project)
        grid = None
        if global_grid:
            shape = (glo_num_idx[1], glo_num_idx[0]) if project else (glo_num_idx[2], glo_num_idx[1], glo_num_idx[0])
            grid = out if out is not None else np.empty(shape, np.float32)
        bd = None
        barrays = None
        if block_arrays:
            barrays = []
            ptrs = (ctypes.c_void_p * len(blocks))()
            for i in range(len(blocks)):
                n = lib().tessgpu_block_grid_points(len(blocks), arr, i, ctypes.byref(p), None)
                a = np.empty(max(n, 0), np.float32)
                barrays.append(a)
                ptrs[i] = a.ctypes.data
            bd = ptrs
        info = DenseInfo()
        self._check(lib().tessgpu_dense(self._h, len(blocks), arr, ctypes.byref(p), _p(grid), bd, ctypes.byref(info)))
        del keep
        return dict(grid=grid, info=info.as_dict(), blocks=barrays)

    def upload(self, blocks):
        return Batch(self, blocks, device=False)

    # --- ProjectGrid / WriteGrid -----------------------------------------
    def project_grid(self, d_layers, num_layers, layer_floats, d_out):
        """ProjectGrid (src/dense.cpp:881-1023): d_out = sum of the layers, in order (device addresses)."""
        self._check(lib().tessgpu_project_grid(self._h, ctypes.c_void_p(d_layers), int(num_layers), int(layer_floats),
                                               ctypes.c_void_p(d_out)))

    def write_grid(self, d_grid, num_floats, path):
        """WriteGrid's raw float32 file (src/dense.cpp:751-870) from device memory at d_grid."""
        self._check(lib().tessgpu_write_grid(self._h, ctypes.c_void_p(d_grid), int(num_floats), os.fsencode(path)))

    def write_last_grid(self, path):
        """WriteGrid after dense(): the last Context.dense call's global grid."""
        self._check(lib().tessgpu_write_last_grid(self._h, os.fsencode(path)))


def sets_offsets(glo_num_idx):
    """(total floats, per-set first float) of the output of Batch.dense_sets."""
    gni = np.ascontiguousarray(np.asarray(glo_num_idx, np.int32).reshape(-1, 3))
    off = np.zeros(len(gni), np.int64)
    n = lib().tessgpu_sets_grid_floats(len(gni), _p(gni), _p(off))
    if n < 0:
        raise ValueError("a set's grid has fewer than 2 points on an axis")
    return int(n), off


def grid_floats(blocks, alg, glo_num_idx, project=False, **kw):
    """(floats, layers) of the device grid Batch.dense writes for these blocks."""
    arr, keep = make_blocks(blocks)
    p = make_params(alg, glo_num_idx, project=project, **kw)
    layers = ctypes.c_int()
    n = lib().tessgpu_dense_grid_floats(len(blocks), arr, ctypes.byref(p), ctypes.byref(layers))
    del keep
    return int(n), int(layers.value)


class Batch:
    """tessgpu_batch: blocks resident on the GPU."""

    def __init__(self, ctx, blocks, device=False):
        self.ctx = ctx
        self._arr, self._keep = make_blocks(blocks) if not device else blocks
        self._h = _VP()
        f = lib().tessgpu_batch_wrap_device if device else lib().tessgpu_batch_upload
        ctx._check(f(ctx.handle, len(self._arr), self._arr, ctypes.byref(self._h)))
        if not device:
            self._keep = None   # host arrays were copied

    def free(self):
        if self._h:
            lib().tessgpu_batch_free(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def keep_debug(self, on=True):
        self.ctx._check(lib().tessgpu_batch_keep_debug(self._h, 1 if on else 0))

    def dense(self, alg, glo_num_idx, d_grid, mass=1.0, eps=1e-4, mode=MODE_MIXED, given=None, want_info=True,
              data_bounds=None, project=False):
        """dense() into the device grid at address d_grid (an int, e.g. torch tensor.data_ptr());
        projected: the grid holds info['grid_layers'] x-y layers (grid_floats() floats)."""
        p = make_params(alg, glo_num_idx, mass, eps, mode, given, data_bounds, project)
        info = DenseInfo() if want_info else None
        self.ctx._check(lib().tessgpu_batch_dense(self.ctx.handle, self._h, ctypes.byref(p), ctypes.c_void_p(d_grid),
                                                  ctypes.byref(info) if info is not None else None))
        return info.as_dict() if info is not None else None

    def dense_sets(self, glo_num_idx, d_out, mass=1.0, eps=1e-4, mode=MODE_MIXED, graph=False, want_info=True):
        """DTFE of every block as an independent set onto its own grid (glo_num_idx:
        one (nx, ny, nz) per block) into device memory at d_out, set b at
        sets_offsets(glo_num_idx)[b]; graph=True records the step into a CUDA graph
        once and replays it."""
        gni = np.ascontiguousarray(np.asarray(glo_num_idx, np.int32).reshape(-1, 3))
        info = DenseInfo() if want_info else None
        self.ctx._check(lib().tessgpu_batch_dense_sets(self.ctx.handle, self._h, _p(gni), ctypes.c_float(mass),
                                                       ctypes.c_float(eps), int(mode), ctypes.c_void_p(d_out),
                                                       1 if graph else 0,
                                                       ctypes.byref(info) if info is not None else None))
        return info.as_dict() if info is not None else None

    def incomplete_cells(self, links6_per_block, d_masks, wrap3_per_block=None, last_neighbor=None):
        """incomplete_cells for every block; masks (one uint64 per original particle of
        the batch, blocks in order) go to device memory at d_masks.  Returns enqueued per block."""
        nb = len(links6_per_block)
        off = np.zeros(nb + 1, np.int32)
        rows, wraps = [], []
        for b, l6 in enumerate(links6_per_block):
            l6 = np.asarray(l6, np.float32).reshape(-1, 6)
            off[b + 1] = off[b] + len(l6)
            rows.append(l6)
            w = None if wrap3_per_block is None else wrap3_per_block[b]
            wraps.append(np.zeros((len(l6), 3), np.int32) if w is None else np.asarray(w, np.int32).reshape(-1, 3))
        links = make_links(np.concatenate(rows) if rows else np.zeros((0, 6), np.float32),
                           np.concatenate(wraps) if wraps else None)
        last = None if last_neighbor is None else np.ascontiguousarray(last_neighbor, np.int32)
        enq = np.zeros(nb, np.int64)
        self.ctx._check(lib().tessgpu_batch_incomplete_cells(self.ctx.handle, self._h, _p(off), links, _p(last),
                                                             ctypes.c_void_p(d_masks), _p(enq)))
        return enq

    def debug_outputs(self, cells=None, grid_points=None, particles=None):
        cc = np.empty(cells, np.int32) if cells else None
        ow = np.empty(grid_points, np.int32) if grid_points else None
        rh = np.empty(particles, np.float32) if particles else None
        self.ctx._check(lib().tessgpu_batch_debug_outputs(self.ctx.handle, self._h, _p(cc), _p(ow), _p(rh)))
        return cc, ow, rh
