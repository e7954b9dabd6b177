import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    """The restated CPU oracle (built here or on the GPU host from oracle/)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    from oracle.oracle import Restated
    return Restated()


def load_single(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def load_blocks(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    blocks = []
    for i in range(int(d["nblocks"])):
        blocks.append(dict(gid=int(d[f"b{i}_gid"]), particles=d[f"b{i}_particles"], tets=d[f"b{i}_tets"],
                           vert_to_tet=d[f"b{i}_vert_to_tet"], num_orig=int(d[f"b{i}_num_orig"]),
                           bounds_min=d[f"b{i}_bounds_min"], bounds_max=d[f"b{i}_bounds_max"],
                           data_min=d[f"b{i}_data_min"], data_max=d[f"b{i}_data_max"]))
    return d, blocks


def single_block(d):
    p = d["particles"]
    return [dict(gid=0, particles=p, tets=d["tets"], vert_to_tet=d["vert_to_tet"], num_orig=len(p),
                 bounds_min=np.zeros(3, np.float32), bounds_max=np.ones(3, np.float32),
                 data_min=np.zeros(3, np.float32), data_max=np.ones(3, np.float32))]


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.fixture(scope="session")
def gpu_ctx():
    """A tessgpu context on cuda:0; the library is built in-tree first."""
    from tess2_gb300 import build
    build.build()
    from tess2_gb300.api import Context
    return Context(0)


WRITEGRID_CASES = ["c1_uniform4096_seed1", "mix2048_seed7", "blocks8_mix8192_seed3"]


def load_case_blocks(name):
    """(fixture dict, blocks, glo_num_idx) of a single-block or multi-block golden case."""
    if name.startswith("blocks"):
        d, blocks = load_blocks(name)
    else:
        d = load_single(name)
        blocks = single_block(d)
    return d, blocks, [int(x) for x in d["glo_num_idx"]]


def load_writegrid():
    z = np.load(os.path.join(GOLDEN, "writegrid.npz"))
    return {k: z[k] for k in z.files}
