"""GB300-native visual-inertial bundle-adjustment back-end.

A drop-in for maplab's VIMapOptimizer / map_optimization::solve path and the
ceres_error_terms visual and inertial cost functions: hand-written sm_103a CUDA
kernels behind the C ABI of include/maplab_ba.h.
"""
from . import _native  # noqa: F401

__all__ = ["ba", "synth", "build"]
