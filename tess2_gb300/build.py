"""Builds libtess2_gb300.so (sm_103a) in-tree with nvcc, no cmake.

Per-file flags matter for results:
  geometry.cu, dtfe.cu   -fmad=false   the reference-order FP32 expressions and the
                                       DTFE error bounds assume no FMA contraction
  api.cu                 -Xcompiler -ffp-contract=off   host GridStepParams /
                                       BlockGridParams in the reference's FP32 order
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtess2_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    "geometry.cu": ["-fmad=false"],
    "dtfe.cu": ["-fmad=false"],
    "api.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "surrogate.cu": [],
    "unet.cu": [],
}


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "tess2_gb300.h"))
    jobs = []
    objs = []
    for unit, flags in UNITS.items():
        src = os.path.join(SRC, unit)
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([NVCC] + ARCH + COMMON + flags + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
