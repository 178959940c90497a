"""GB300-native (sm_103a) implementation of canmom/rasteriser's per-frame hot path.

The compute path is librast (CUDA kernels behind a C ABI, include/rast.h); ``abi`` binds it and
``scenes`` generates the seeded synthetic workloads.
"""
from . import abi, scenes  # noqa: F401

__all__ = ["abi", "scenes"]
