"""The C ABI without a GPU: the library builds and loads, exports every symbol
include/tess2_gb300.h declares, and its host-only logic (dense()'s grid
parameters) matches the reference's restatement."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_blocks

HEADER = os.path.join(ROOT, "include", "tess2_gb300.h")


@pytest.fixture(scope="module")
def built():
    from tess2_gb300 import build
    return build.build()


def declared_symbols():
    src = open(HEADER).read()
    decl = r"^(?:tessgpu_status|void|const char\*|long long|int)\s+\**(tessgpu_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, src, flags=re.M)))


def test_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    names = declared_symbols()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_no_device_is_reported(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from tess2_gb300.api import Context, TessGpuError
    with pytest.raises(TessGpuError) as e:
        Context(0)
    assert e.value.code == 3


def test_block_grid_points_match_reference(built, oracle):
    """tessgpu_block_grid_points is BlockGridParams (src/dense.cpp:575-648) on
    the host; compare with the restated oracle's for every golden block."""
    from tess2_gb300.api import lib, make_blocks, make_params
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    for gni in ([40, 40, 40], [33, 65, 17], [512, 512, 512]):
        arr, keep = make_blocks(blocks)
        p = make_params(0, gni)
        r = oracle.dense(0, blocks[:1], [9, 9, 9])  # loads the library
        del r
        from oracle.oracle import _ptr
        O = oracle._l
        dmin = np.min([b["bounds_min"] for b in blocks], 0).astype(np.float32)
        dmax = np.max([b["bounds_max"] for b in blocks], 0).astype(np.float32)
        gmin, gmax, step = (np.zeros(3, np.float32) for _ in range(3))
        gn = np.array(gni, np.int32)
        O.f("grid_step_params")(ctypes.c_int(0), None, None, _ptr(dmin), _ptr(dmax), _ptr(gmin), _ptr(gmax),
                                _ptr(step), _ptr(gn))
        from oracle.oracle import make_blocks as omb
        oarr, okeep = omb(blocks)
        for i in range(len(blocks)):
            o9 = (ctypes.c_int * 9)()
            n = lib().tessgpu_block_grid_points(len(blocks), arr, i, ctypes.byref(p), o9)
            mn, mx, num = (np.zeros(3, np.int32) for _ in range(3))
            O.f("block_grid_params")(ctypes.byref(oarr[i]), _ptr(gmin), _ptr(step), ctypes.c_float(1e-4), _ptr(dmin),
                                     _ptr(dmax), _ptr(gn), _ptr(mn), _ptr(mx), _ptr(num))
            assert list(o9) == list(mn) + list(mx) + list(num)
            assert n == int(np.prod(num))
        # the blocks' index boxes tile the grid
        cover = np.zeros(gni[::-1], np.int32) if np.prod(gni) < 5e6 else None
        if cover is not None:
            for i in range(len(blocks)):
                o9 = (ctypes.c_int * 9)()
                lib().tessgpu_block_grid_points(len(blocks), arr, i, ctypes.byref(p), o9)
                cover[o9[2]:o9[5] + 1, o9[1]:o9[4] + 1, o9[0]:o9[3] + 1] += 1
            assert np.all(cover == 1)


def test_invalid_arguments_rejected(built):
    from tess2_gb300.api import lib, make_params
    p = make_params(0, [1, 8, 8])   # a grid axis with one point has no step
    assert lib().tessgpu_block_grid_points(1, None, 0, ctypes.byref(p), None) == -1
