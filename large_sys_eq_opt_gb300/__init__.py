"""GB300-native (sm_103a) MUSCL-Hancock split step for the 2D Euler equations.

The compute path is libeuler2d.so: hand-written CUDA kernels (TMA-staged
fused x/y sweeps with a device-side CFL reduction) behind the C ABI in
include/euler2d.h.  ``euler2d`` is a thin ctypes binding of that ABI and
``cases`` mirrors the reference's case table.
"""
from . import cases  # noqa: F401

__all__ = ["cases", "euler2d", "build"]
