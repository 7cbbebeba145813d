"""GB300 (sm_103a) implementation of NEMO's per-timestep ocean stencil path.

The compute path is the CUDA library built from ``../csrc`` (``libnemo_gpu.so``),
reached through its C ABI (``include/nemo_gpu.h``). This package holds the ctypes
binding of that ABI, a thin host mirror of the reference's Fortran interfaces
operating on device tensors, the build recipe and the synthetic GYRE case
generator used by the tests and the benchmark.
"""
from .build import build as build_library, library_path  # noqa: F401
from . import gyre  # noqa: F401
