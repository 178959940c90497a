"""GB300-native (sm_103a) implementation of canmom/rasteriser's per-frame hot path.

The compute path is librast (CUDA kernels behind a C ABI, include/rast.h); ``abi`` binds it and
``scenes`` generates the seeded synthetic workloads. Submodules load on first use, so importing
``scenes`` alone maps no native library.
"""
import importlib

__all__ = ["abi", "scenes"]


def __getattr__(name):
    if name in __all__:
        return importlib.import_module(f"{__name__}.{name}")
    raise AttributeError(name)
