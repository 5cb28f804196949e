"""GB300-native (sm_103a) matrix-free sum-factorization operators.

The compute path is the CUDA library ``libsfgpu.so`` (sources in ``csrc/``,
C ABI in ``include/sfgpu.h``); this package holds its build recipe and a
ctypes binding.  Importing the package does not load the library; calling
any operator does, and raises if it has not been built.
"""
from . import sfgpu  # noqa: F401
from .sfgpu import Operator, SFError  # noqa: F401

__all__ = ["sfgpu", "Operator", "SFError"]
