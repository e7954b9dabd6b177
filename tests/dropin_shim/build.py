"""Builds the drop-in test library: tess2_gb300/dropin/*.cpp (the sources a
tess2 build compiles in place of src/dense.cpp and src/volume.cpp) with the
test driver, against the stand-in tess2 headers here and the single-rank
MPI/DIY stand-ins of oracle/ref_shim, linked to libtess2_gb300.so.  Test
infrastructure.  With tess_include (a tess2 checkout's include directory)
the drop-in sources are compiled against tess2's own headers instead (object
files only), which checks the signatures against the reference."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdropin_test.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
SRCS = [os.path.join(ROOT, "tess2_gb300", "dropin", f) for f in ("dense_gpu.cpp", "volume_gpu.cpp", "topology_gpu.cpp")]


def _flags(tess_include):
    return ["-std=gnu++14", "-O2", "-fPIC", "-I", tess_include, "-I", os.path.join(ROOT, "oracle", "ref_shim"),
            "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include")]


def build():
    os.makedirs(OUT, exist_ok=True)
    from tess2_gb300 import build as b
    so = b.build()
    cmd = (["g++"] + _flags(HERE) + ["-shared", "-o", LIB] + SRCS + [os.path.join(HERE, "driver.cpp")] +
           ["-L", os.path.dirname(so), "-ltess2_gb300", "-Wl,-rpath," + os.path.dirname(so),
            "-L", os.path.join(CUDA, "lib64"), "-lcudart"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


def compile_against(tess_include):
    """The drop-in sources against a tess2 checkout's own headers (objects only)."""
    os.makedirs(OUT, exist_ok=True)
    for src in SRCS:
        obj = os.path.join(OUT, os.path.basename(src) + ".ref.o")
        cmd = ["g++"] + _flags(tess_include) + ["-DTESS_NO_OPENMP", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
