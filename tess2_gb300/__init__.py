"""tess2_gb300: GB300-native post-Delaunay geometry and density path of tess2.

The CUDA kernels and the C ABI live in csrc/ and build into
_build/libtess2_gb300.so (see build.py); api.py is the Python mirror of the
reference's calls; host.py prepares blocks (particles, ghost zones, Qhull
tets) on the host.
"""
from .api import (DENSE_CIC, DENSE_DTFE, DENSE_TESS, MODE_FP64, MODE_MIXED, Batch, Context, TessGpuError, lib,
                  library_path)

__all__ = ["DENSE_TESS", "DENSE_CIC", "DENSE_DTFE", "MODE_MIXED", "MODE_FP64", "Context", "Batch", "TessGpuError",
           "lib", "library_path"]
