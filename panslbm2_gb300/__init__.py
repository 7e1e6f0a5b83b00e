"""GB300-native implementation of PANSLBM2's lattice-Boltzmann topology-optimisation hot path.

The compute path is the CUDA library libpanslbm_gb300.so (C ABI: include/panslbm_gb300.h);
this package is its Python host binding. Importing the package does not load the library;
`LatticePair(...)` does, and raises if it has not been built.
"""
from . import _capi as capi  # noqa: F401
from .lattice import Desc, LatticePair, bc, phys, smooth_at, smooth_corner, smooth_line  # noqa: F401

__all__ = ["LatticePair", "Desc", "bc", "phys", "smooth_corner", "smooth_at", "smooth_line", "capi"]
