"""GB300-native staggered-grid elastic FDTD time loop (drop-in for the FastWaveED_GPU3D solver).

The compute path is libewfd.so (hand-written sm_103a CUDA behind a C ABI, include/ewfd.h);
this package holds its Python binding, the input generators and the legacy file contract.
"""
from . import fields
from .solver import EwfError, Solver, load_library, run_legacy

__all__ = ["fields", "EwfError", "Solver", "load_library", "run_legacy"]
