"""ctypes bindings for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two libraries share one block layout (orc_block / ref_block):
  * oracle/_build/libtess_oracle.so -- the plain-C restatement (tess_oracle.c),
    built here and on any machine by ``make -C oracle``;
  * oracle/_ref/libtess_ref.so      -- the reference's own src/tet.cpp,
    src/volume.cpp and src/dense.cpp compiled unmodified (``make -C oracle ref``),
    available only where the reference sources are.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker or the timed CPU baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libtess_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtess_ref.so")

_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)


class Block(ctypes.Structure):
    """orc_block / ref_block: one DIY block as plain arrays."""
    _fields_ = [("gid", ctypes.c_int),
                ("bounds_min", ctypes.c_float * 3), ("bounds_max", ctypes.c_float * 3),
                ("data_min", ctypes.c_float * 3), ("data_max", ctypes.c_float * 3),
                ("num_orig_particles", ctypes.c_int), ("num_particles", ctypes.c_int),
                ("particles", ctypes.c_void_p), ("num_tets", ctypes.c_int),
                ("tets", ctypes.c_void_p), ("vert_to_tet", ctypes.c_void_p)]


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def build(ref=False):
    """Compile the restated oracle (and the reference build when asked)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


class _Lib:
    def __init__(self, path, prefix):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        self.p = prefix

    def f(self, name):
        return getattr(self.lib, self.p + name)


def make_blocks(blocks):
    """blocks: list of dicts with particles (N,3) f32, tets (T,8) i32,
    vert_to_tet (N,) i32, num_orig, bounds_min/max, data_min/max, gid.
    Returns (ctypes array of Block, keepalive list)."""
    arr = (Block * len(blocks))()
    keep = []
    for i, b in enumerate(blocks):
        p = np.ascontiguousarray(b["particles"], dtype=np.float32)
        t = np.ascontiguousarray(b["tets"], dtype=np.int32)
        v = np.ascontiguousarray(b["vert_to_tet"], dtype=np.int32)
        keep += [p, t, v]
        blk = arr[i]
        blk.gid = int(b.get("gid", i))
        for d in range(3):
            blk.bounds_min[d] = b["bounds_min"][d]
            blk.bounds_max[d] = b["bounds_max"][d]
            blk.data_min[d] = b["data_min"][d]
            blk.data_max[d] = b["data_max"][d]
        blk.num_orig_particles = int(b["num_orig"])
        blk.num_particles = int(p.shape[0])
        blk.particles = p.ctypes.data
        blk.num_tets = int(t.shape[0])
        blk.tets = t.ctypes.data
        blk.vert_to_tet = v.ctypes.data
    return arr, keep


class Oracle:
    """Common calls of the restated oracle ("orc_") and the reference build ("ref_")."""

    def __init__(self, which="oracle"):
        if which == "oracle":
            self._l = _Lib(ORACLE_SO, "orc_")
        else:
            self._l = _Lib(REF_SO, "ref_")
        self.which = which

    def fill_circumcenters(self, particles, tets):
        out = np.empty((tets.shape[0], 3), np.float32)
        self._l.f("fill_circumcenters")(_ptr(particles), _ptr(tets), ctypes.c_int(tets.shape[0]), _ptr(out))
        return out

    def complete_all(self, tets, vert_to_tet):
        out = np.empty(vert_to_tet.shape[0], np.int32)
        self._l.f("complete_all")(_ptr(tets), ctypes.c_int(tets.shape[0]), _ptr(vert_to_tet),
                                  ctypes.c_int(vert_to_tet.shape[0]), _ptr(out))
        return out

    def volumes(self, particles, tets, vert_to_tet, n=None):
        n = vert_to_tet.shape[0] if n is None else n
        out = np.empty(n, np.float32)
        self._l.f("volumes")(ctypes.c_int(n), _ptr(vert_to_tet), _ptr(tets), ctypes.c_int(tets.shape[0]),
                             _ptr(particles), _ptr(out))
        return out

    def neighbor_edges(self, v, tets, t, cap=4096):
        pairs = np.empty(2 * cap, np.int32)
        fin = ctypes.c_int(0)
        n = self._l.f("neighbor_edges")(ctypes.c_int(v), _ptr(tets), ctypes.c_int(t), _ptr(pairs),
                                       ctypes.c_int(cap), ctypes.byref(fin))
        if n < 0:
            raise ValueError("neighbor_edges overflow")
        return pairs[:2 * n].reshape(n, 2).copy(), bool(fin.value)

    def dense(self, alg, blocks, glo_num_idx, mass=1.0, eps=1e-4, given=None, cell_counts=False, data6=None,
              project=False, block_arrays=False):
        """dense() into a global grid (z, y, x order, x fastest).  data6 (restated
        oracle only) fixes the data bounds, as DataBounds' all-reduce would.
        project (restated oracle only): x-y projection; grid is then (y, x) after
        ProjectGrid and block_arrays returns each block's array before it."""
        arr, keep = make_blocks(blocks)
        gni = np.ascontiguousarray(glo_num_idx, dtype=np.int32)
        grid = np.zeros((gni[1], gni[0]) if project else (gni[2], gni[1], gni[0]), np.float32)
        g6 = np.zeros(6, np.float32)
        d6 = np.zeros(6, np.float32)
        st = np.zeros(3, np.float64)
        ngiven = 0
        gmin = gmax = None
        if given is not None:
            ngiven = 3
            gmin = np.ascontiguousarray(given[0], dtype=np.float32)
            gmax = np.ascontiguousarray(given[1], dtype=np.float32)
        res = {}
        if self.which == "oracle":
            total = sum(int(b["num_orig"]) for b in blocks)
            cc = np.zeros(max(total, 1), np.int32) if cell_counts else None
            fn = self._l.f("dense_ex")
            fn.restype = ctypes.c_long
            db = None if data6 is None else np.ascontiguousarray(data6, np.float32)
            # per-block array sizes bound: a block array never exceeds the global grid
            bo = np.zeros(len(blocks) * int(np.prod(gni)) // (int(gni[2]) if project else 1), np.float32) \
                if block_arrays else None
            lost = fn(ctypes.c_int(alg), ctypes.c_int(len(blocks)), arr, _ptr(db), ctypes.c_int(1 if project else 0),
                      ctypes.c_int(ngiven), _ptr(gmin), _ptr(gmax), ctypes.c_float(mass), ctypes.c_float(eps),
                      _ptr(gni), _ptr(grid), _ptr(bo), _ptr(g6), _ptr(d6), _ptr(st), _ptr(cc))
            res["lost"] = int(lost)
            if block_arrays:
                res["block_concat"] = bo
            if cell_counts:
                res["cell_counts"] = cc[:total]
        else:
            self._l.f("dense")(ctypes.c_int(alg), ctypes.c_int(len(blocks)), arr, ctypes.c_int(ngiven),
                               _ptr(gmin), _ptr(gmax), ctypes.c_float(mass), ctypes.c_float(eps), _ptr(gni),
                               _ptr(grid), _ptr(g6), _ptr(d6), _ptr(st))
        res.update(grid=grid, grid_min=g6[:3].copy(), grid_step=g6[3:].copy(), data_min=d6[:3].copy(),
                   data_max=d6[3:].copy(), max_dense=st[0], tot_mass=st[1], check_mass=st[2])
        del keep
        return res

    def dense_write(self, alg, blocks, glo_num_idx, path, project=False, mass=1.0, eps=1e-4, given=None):
        """The reference build only: dense() then WriteGrid(outfile=path), as
        examples/dense/main.cpp calls them.  Returns the blocks' arrays as dense()
        leaves them and the dense_stats values; the file is at path."""
        assert self.which == "ref"
        arr, keep = make_blocks(blocks)
        gni = np.ascontiguousarray(glo_num_idx, dtype=np.int32)
        nb = len(blocks)
        bo = np.zeros(nb * int(np.prod(gni)), np.float32)
        sizes = np.zeros(nb, np.int32)
        st = np.zeros(3, np.float64)
        ngiven = 0
        gmin = gmax = None
        if given is not None:
            ngiven = 3
            gmin = np.ascontiguousarray(given[0], dtype=np.float32)
            gmax = np.ascontiguousarray(given[1], dtype=np.float32)
        self._l.f("dense_write")(ctypes.c_int(alg), ctypes.c_int(nb), arr, ctypes.c_int(ngiven), _ptr(gmin),
                                 _ptr(gmax), ctypes.c_float(mass), ctypes.c_float(eps), _ptr(gni),
                                 ctypes.c_int(1 if project else 0), os.fsencode(path), _ptr(bo), _ptr(sizes),
                                 _ptr(st))
        del keep
        out, off = [], 0
        for n in sizes:
            out.append(bo[off:off + n].copy())
            off += n
        return dict(blocks=out, max_dense=st[0], tot_mass=st[1], check_mass=st[2])

    def side_of_plane(self, box6, tet, particles, j):
        """side_of_plane (src/tet.cpp:70-119)."""
        box6 = np.ascontiguousarray(box6, np.float32)
        tet = np.ascontiguousarray(tet, np.int32)
        particles = np.ascontiguousarray(particles, np.float32)
        return int(self._l.f("side_of_plane")(_ptr(box6), _ptr(tet), _ptr(particles), ctypes.c_int(j)))

    def distance(self, u, v):
        """distance (src/tet.cpp:146-153)."""
        fn = self._l.f("distance")
        fn.restype = ctypes.c_float
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        return np.float32(fn(_ptr(u), _ptr(v)))

    def cell_grid_pts(self, block, cell, data_min, data_max, grid_min, grid_step, mass=1.0, eps=1e-4,
                      cap=1 << 16):
        arr, keep = make_blocks([block])
        idx = np.empty(3 * cap, np.int32)
        m = np.empty(cap, np.float64)
        cb = np.zeros(6, np.float32)
        dm = np.ascontiguousarray(data_min, np.float32)
        dx = np.ascontiguousarray(data_max, np.float32)
        gm = np.ascontiguousarray(grid_min, np.float32)
        gs = np.ascontiguousarray(grid_step, np.float32)
        n = self._l.f("cell_grid_pts")(arr, ctypes.c_int(cell), _ptr(dm), _ptr(dx), _ptr(gm), _ptr(gs),
                                      ctypes.c_float(mass), ctypes.c_float(eps), _ptr(idx), _ptr(m),
                                      ctypes.c_int(cap), _ptr(cb))
        del keep
        k = max(n, 0)
        return n, idx[:3 * min(k, cap)].reshape(-1, 3).copy(), m[:min(k, cap)].copy(), cb


class Restated(Oracle):
    """Extra calls that only the restated oracle has (FP64 references, DTFE, predicates)."""

    def __init__(self):
        super().__init__("oracle")

    def fill_vert_to_tet(self, num_particles, tets):
        out = np.empty(num_particles, np.int32)
        self._l.f("fill_vert_to_tet")(ctypes.c_int(num_particles), _ptr(tets), ctypes.c_int(tets.shape[0]),
                                      _ptr(out))
        return out

    def reorder_neighbors(self, tets):
        out = np.array(tets, dtype=np.int32, copy=True, order="C")
        self._l.f("reorder_neighbors")(_ptr(out), ctypes.c_int(out.shape[0]))
        return out

    def fill_circumcenters_f64(self, particles, tets):
        out = np.empty((tets.shape[0], 3), np.float64)
        self._l.f("fill_circumcenters_f64")(_ptr(particles), _ptr(tets), ctypes.c_int(tets.shape[0]), _ptr(out))
        return out

    def volume_areas(self, particles, tets, vert_to_tet, n=None):
        """volume() (src/volume.cpp:13-54) and each cell's summed face area, in float."""
        n = vert_to_tet.shape[0] if n is None else n
        vol = np.empty(n, np.float32)
        area = np.empty(n, np.float32)
        self._l.f("volume_areas")(ctypes.c_int(n), _ptr(vert_to_tet), _ptr(tets), ctypes.c_int(tets.shape[0]),
                                  _ptr(particles), _ptr(vol), _ptr(area))
        return vol, area

    def volumes_f64(self, particles, tets, vert_to_tet, n=None):
        n = vert_to_tet.shape[0] if n is None else n
        out = np.empty(n, np.float64)
        self._l.f("volumes_f64")(ctypes.c_int(n), _ptr(vert_to_tet), _ptr(tets), ctypes.c_int(tets.shape[0]),
                                 _ptr(particles), _ptr(out))
        return out

    def orient3d_exact(self, a, b, c, d):
        a, b, c, d = (np.ascontiguousarray(x, np.float32) for x in (a, b, c, d))
        return int(self._l.f("orient3d_exact")(_ptr(a), _ptr(b), _ptr(c), _ptr(d)))

    def tet_contains(self, particles, tet, p):
        particles = np.ascontiguousarray(particles, np.float32)
        tet = np.ascontiguousarray(tet, np.int32)
        p = np.ascontiguousarray(p, np.float32)
        return bool(self._l.f("tet_contains")(_ptr(particles), _ptr(tet), _ptr(p)))

    def incomplete_cells(self, block, links6, wrap3=None, last_neighbor=0):
        """incomplete_cells (src/tess.cpp:492-628) for one block: (masks, enqueued),
        masks a uint64 per original particle, bit i = send to link i."""
        arr, keep = make_blocks([block])
        l6 = np.ascontiguousarray(links6, np.float32).reshape(-1, 6)
        w3 = None if wrap3 is None else np.ascontiguousarray(wrap3, np.int32).reshape(-1, 3)
        masks = np.zeros(max(int(block["num_orig"]), 1), np.uint64)
        fn = self._l.f("incomplete_cells")
        fn.restype = ctypes.c_long
        n = fn(arr, ctypes.c_int(l6.shape[0]), _ptr(l6), _ptr(w3), ctypes.c_int(last_neighbor), _ptr(masks))
        del keep
        return masks[:int(block["num_orig"])], int(n)

    def box_distance(self, box6, c):
        fn = self._l.f("box_distance")
        fn.restype = ctypes.c_float
        box6 = np.ascontiguousarray(box6, np.float32)
        c = np.ascontiguousarray(c, np.float32)
        return np.float32(fn(_ptr(box6), _ptr(c)))

    @staticmethod
    def z_layers(block_zmin, nz):
        """Layer of each z index of a projected grid: one layer per distinct
        first z index of the blocks' BlockGridParams boxes, ascending."""
        starts = sorted(set(int(min(max(z, 0), nz - 1)) for z in block_zmin))
        zl = np.zeros(nz, np.int32)
        for l, z0 in enumerate(starts):
            zl[z0:] = l
        return zl, max(len(starts), 1)

    @staticmethod
    def project_layers(grid3, zl, dz):
        """z-projection of a (z, y, x) float32 grid into layers: layer l
        accumulates grid * dz over its z indices in ascending z, in float32."""
        nl = int(zl.max()) + 1
        out = np.zeros((nl,) + grid3.shape[1:], np.float32)
        dz = np.float32(dz)
        for z in range(grid3.shape[0]):
            out[zl[z]] = out[zl[z]] + grid3[z] * dz
        return out

    @staticmethod
    def sum_layers(layers):
        """ProjectGrid's column sum: layer 0 plus layers 1.. in order, in float32."""
        acc = layers[0].copy()
        for l in range(1, layers.shape[0]):
            acc = acc + layers[l]
        return acc

    def dtfe(self, blocks, glo_num_idx, mass=1.0, eps=1e-4, given=None, want_owner=True, want_rho=True,
             data6=None, raster_stride=1):
        arr, keep = make_blocks(blocks)
        gni = np.ascontiguousarray(glo_num_idx, dtype=np.int32)
        grid = np.zeros((gni[2], gni[1], gni[0]), np.float32)
        owner = np.empty(grid.shape, np.int32) if want_owner else None
        nv = sum(int(np.asarray(b["particles"]).shape[0]) for b in blocks)
        rho = np.empty(max(nv, 1), np.float64) if want_rho else None
        g6 = np.zeros(6, np.float32)
        ngiven = 0
        gmin = gmax = None
        if given is not None:
            ngiven = 3
            gmin = np.ascontiguousarray(given[0], dtype=np.float32)
            gmax = np.ascontiguousarray(given[1], dtype=np.float32)
        fn = self._l.f("dtfe_f64_sample")
        fn.restype = ctypes.c_long
        db = None if data6 is None else np.ascontiguousarray(data6, np.float32)
        n = fn(ctypes.c_int(len(blocks)), arr, _ptr(db), ctypes.c_int(ngiven), _ptr(gmin), _ptr(gmax),
               ctypes.c_float(mass), ctypes.c_float(eps), _ptr(gni), ctypes.c_int(raster_stride), _ptr(grid),
               _ptr(rho), _ptr(owner), _ptr(g6))
        del keep
        return dict(grid=grid, owner=owner, rho=rho[:nv] if rho is not None else None, assigned=int(n),
                    grid_min=g6[:3].copy(), grid_step=g6[3:].copy())


class TessCells:
    """The reference estimator's per-cell work (DENSE_TESS, IterateCells,
    src/dense.cpp:220-313) for one block on chosen cells, through the restated
    oracle; the block's circumcenters are computed once, here.  Used to time
    the reference on samples of cells."""

    def __init__(self, block, data6, glo_num_idx, mass=1.0, eps=1e-4):
        self.o = Restated()
        self.arr, self.keep = make_blocks([block])
        t = np.ascontiguousarray(block["tets"], np.int32)
        p = np.ascontiguousarray(block["particles"], np.float32)
        self.cc = np.empty((max(t.shape[0], 1), 3), np.float32)
        self.o._l.f("fill_circumcenters")(_ptr(p), _ptr(t), ctypes.c_int(t.shape[0]), _ptr(self.cc))
        self.keep += [t, p]
        self.d6 = np.ascontiguousarray(data6, np.float32)
        self.gni = np.ascontiguousarray(glo_num_idx, np.int32)
        self.grid = np.zeros(int(np.prod(self.gni)), np.float32)
        self.mass, self.eps = mass, eps
        self.fn = self.o._l.f("dense_tess_cells")
        self.fn.restype = ctypes.c_long

    def run(self, cells, counts=False):
        """Cells (particle indices of the block) through CellBounds, CellGridPts and
        the deposits; returns how many deposited (and, with counts, each cell's
        CellGridPts result: -1 skipped, else its grid points)."""
        c = np.ascontiguousarray(cells, np.int32)
        cnt = np.empty(c.shape[0], np.int32) if counts else None
        n = int(self.fn(self.arr, _ptr(self.cc), _ptr(c), ctypes.c_int(c.shape[0]), _ptr(self.d6),
                        _ptr(self.gni), ctypes.c_float(self.mass), ctypes.c_float(self.eps), _ptr(self.grid),
                        _ptr(cnt)))
        return (n, cnt) if counts else n

