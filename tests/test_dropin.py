"""The compiled drop-in (tess2_gb300/dropin/dense_gpu.cpp, volume_gpu.cpp,
topology_gpu.cpp): tess2's own signatures -- dense(), WriteGrid(),
dense_stats(), volume(), fill_circumcenters(), and complete() and
fill_vert_to_tet() with C linkage -- over the GPU library.

CPU: the sources compile against tess2's own headers where a tess2 checkout
is present (TESS2_REF, or a "reference" directory beside this repository),
which checks every signature against the reference.

GPU: the sources are built with the test driver against stand-in headers
(tests/dropin_shim) and called as tess2's examples/dense/main.cpp calls them:
the blocks' density arrays and the WriteGrid file must equal what the
reference's own dense() and WriteGrid wrote (tests/golden/writegrid.npz,
projected) and what tessgpu_dense computes; volume() and
fill_circumcenters() must equal the reference's bits."""
import ctypes
import importlib.util
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, WRITEGRID_CASES, load_case_blocks, load_single, load_writegrid


def _build_mod():
    spec = importlib.util.spec_from_file_location("dropin_build", os.path.join(ROOT, "tests", "dropin_shim", "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _tess_include():
    cand = os.environ.get("TESS2_REF") or os.path.join(os.path.dirname(ROOT), "reference")
    inc = os.path.join(cand, "include")
    return inc if os.path.isfile(os.path.join(inc, "tess", "dense.hpp")) else None


def test_dropin_compiles_against_reference_headers():
    inc = _tess_include()
    if inc is None:
        pytest.skip("no tess2 checkout here")
    m = _build_mod()
    m.compile_against(inc)
    syms = []
    for f in ("dense_gpu.cpp.ref.o", "volume_gpu.cpp.ref.o", "topology_gpu.cpp.ref.o"):
        out = subprocess.run(["nm", "-C", "--defined-only", os.path.join(m.OUT, f)], capture_output=True, text=True)
        syms += out.stdout.splitlines()
    text = "\n".join(syms)
    for sig in ("dense(alg, int, float*, float*, bool, float*, float, float*, float*, float*, float*, float*, float, "
                "int*, diy::Master&)",
                "WriteGrid(int, int, char*, bool, int*, float, float*, float*, int, float*, float*, diy::Master&, "
                "diy::Assigner&)",
                "dense_stats(double*, diy::Master&, float*, float*, int*)",
                "fill_circumcenters(std::vector<float, std::allocator<float> >&, tet_t*, int, float*)",
                "volume(int, int*, tet_t*, int, float*, std::vector<float, std::allocator<float> > const&)"):
        assert sig in text, sig
    # C linkage, as tess2 declares them (tet-neighbors.h, tess.h): unmangled symbols
    raw = subprocess.run(["nm", "--defined-only", os.path.join(m.OUT, "topology_gpu.cpp.ref.o")], capture_output=True,
                         text=True).stdout.split()
    assert "complete" in raw and "fill_vert_to_tet" in raw


@pytest.fixture(scope="module")
def dropin():
    lib = ctypes.CDLL(_build_mod().build())
    lib.dropin_dense.restype = ctypes.c_int
    return lib


def _run(lib, alg, blocks, gni, project, outfile):
    from oracle.oracle import make_blocks
    arr, keep = make_blocks(blocks)
    g = np.ascontiguousarray(gni, np.int32)
    cap = len(blocks) * int(np.prod(gni))
    out = np.zeros(cap, np.float32)
    sizes = np.zeros(len(blocks), np.int32)
    g6 = np.zeros(6, np.float32)
    rc = lib.dropin_dense(ctypes.c_int(alg), ctypes.c_int(len(blocks)), arr, g.ctypes.data, ctypes.c_float(1.0),
                          ctypes.c_float(1e-4), ctypes.c_int(1 if project else 0),
                          os.fsencode(str(outfile)) if outfile else None, out.ctypes.data,
                          ctypes.c_longlong(cap), sizes.ctypes.data, g6.ctypes.data)
    assert rc == 0
    del keep
    return out[:int(sizes.sum())], sizes


@pytest.mark.gpu
@pytest.mark.parametrize("alg,tag", [(0, "tess"), (1, "cic")])
@pytest.mark.parametrize("name", WRITEGRID_CASES)
def test_dropin_dense_writegrid_vs_reference(dropin, gpu_ctx, tmp_path, name, alg, tag):
    d, blocks, gni = load_case_blocks(name)
    w = load_writegrid()
    out = tmp_path / "proj.raw"
    arrays, sizes = _run(dropin, alg, blocks, gni, True, out)
    np.testing.assert_allclose(arrays, w[f"{name}_{tag}_proj_blocks"], rtol=2e-5, atol=0)
    assert np.array_equal(sizes, w[f"{name}_{tag}_proj_block_sizes"])
    f = np.fromfile(out, np.float32)
    np.testing.assert_allclose(f, w[f"{name}_{tag}_proj_file"].ravel(), rtol=2e-5, atol=0)
    # 3-D: the same block arrays tessgpu_dense gives, and the file is the global grid
    out3 = tmp_path / "grid.raw"
    a3, _ = _run(dropin, alg, blocks, gni, False, out3)
    r = gpu_ctx.dense(alg, blocks, gni, block_arrays=True)
    ref = np.concatenate(r["blocks"])
    np.testing.assert_allclose(a3, ref, rtol=2e-5, atol=0)
    np.testing.assert_allclose(np.fromfile(out3, np.float32), r["grid"].ravel(), rtol=2e-5, atol=0)


@pytest.mark.gpu
def test_dropin_dtfe_estimator(dropin, gpu_ctx):
    """TESS2_GB300_ESTIMATOR=dtfe: dense() runs DTFE; the block arrays equal
    tessgpu_dense's DTFE arrays bit for bit."""
    d, blocks, gni = load_case_blocks("blocks8_mix8192_seed3")
    os.environ["TESS2_GB300_ESTIMATOR"] = "dtfe"
    try:
        arrays, _ = _run(dropin, 0, blocks, gni, False, None)
    finally:
        os.environ.pop("TESS2_GB300_ESTIMATOR", None)
    r = gpu_ctx.dense(2, blocks, gni, block_arrays=True)
    assert np.array_equal(arrays, np.concatenate(r["blocks"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1_uniform4096_seed1", "mix2048_seed7"])
def test_dropin_volume_and_circumcenters(dropin, name):
    d = load_single(name)
    p = np.ascontiguousarray(d["particles"], np.float32)
    t = np.ascontiguousarray(d["tets"], np.int32)
    v2t = np.ascontiguousarray(d["vert_to_tet"], np.int32)
    cc = np.zeros((len(t), 3), np.float32)
    vol = np.zeros(len(p), np.float32)
    dropin.dropin_volumes(p.ctypes.data, ctypes.c_int(len(p)), t.ctypes.data, ctypes.c_int(len(t)), v2t.ctypes.data,
                          cc.ctypes.data, vol.ctypes.data)
    assert np.array_equal(cc.view(np.uint32), np.ascontiguousarray(d["circumcenters"], np.float32).view(np.uint32))
    assert np.array_equal(vol.view(np.uint32), np.ascontiguousarray(d["volumes"], np.float32).view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1_uniform4096_seed1", "mix2048_seed7"])
def test_dropin_complete_and_vert_to_tet(dropin, name):
    """complete() per vertex equals the reference's (goldens); fill_vert_to_tet()
    reallocs and fills vert_to_tet exactly as the reference (the last tet wins)."""
    from tess2_gb300 import host
    d = load_single(name)
    p = np.ascontiguousarray(d["particles"], np.float32)
    t = np.ascontiguousarray(d["tets"], np.int32)
    v2t = np.ascontiguousarray(d["vert_to_tet"], np.int32)
    comp = np.zeros(len(p), np.int32)
    v2t_out = np.full(len(p), -7, np.int32)
    dropin.dropin_topology(p.ctypes.data, ctypes.c_int(len(p)), t.ctypes.data, ctypes.c_int(len(t)), v2t.ctypes.data,
                           comp.ctypes.data, v2t_out.ctypes.data)
    assert np.array_equal(comp, np.ascontiguousarray(d["complete"], np.int32))
    assert np.array_equal(v2t_out, host.vert_to_tet_host(len(p), t))
    assert np.array_equal(v2t_out, v2t)
