"""GB300 (sm_103a) implementation of RAM's bounce-averaged kinetic step.

``ramgpu.abi.RamGpu`` drives the CUDA library through its C ABI
(include/ramgpu.h); ``ramgpu.workload`` builds the synthetic grids, dipole
field tables and initial states the tests and the benchmark use.
"""
from . import workload  # noqa: F401
from .build import LIB_PATH, build_library  # noqa: F401

__all__ = ["workload", "build_library", "LIB_PATH"]
