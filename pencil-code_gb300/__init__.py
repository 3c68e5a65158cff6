"""GB300-native Pencil Code MHD timestep (sm_103a).

The compute path is libpcgb300.so (hand-written CUDA, C ABI in
include/pcgb300.h).  This package holds the build recipe, a ctypes binding,
a mirror of the reference's Fortran ``GPU`` module interface
(src/gpu_astaroth.f90), var.dat I/O, namelist parsing, initial conditions and
the ensemble / serving drivers.  There is no CPU fallback: every entry point
that computes calls the CUDA library and raises if it cannot be loaded.

Import it as ``importlib.import_module("pencil-code_gb300")``.
"""
from .build import build  # noqa: F401
from .lib import (Batch, Box, Params, PcgbError, autotune, default_params, diag_summary,  # noqa: F401
                  host_shape, launch_count, load, nfields)
