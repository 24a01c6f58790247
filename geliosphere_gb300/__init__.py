"""GB300-native (sm_103a) engine for Geliosphere's SDE hot path.

The product is the C-ABI library libgelio_cuda.so (include/gelio.h): the
per-particle trajectory integrators of the 1D F-p, 1D B-p, 2D SolarProp-like
and 2D Geliosphere models and the spectrum evaluation fused into them.  This
package holds its sources (csrc/), the in-tree build (build.py), the ctypes
mirror of the ABI (abi.py), a Python host API (engine.py) and the C++
drop-in host layer (host/) that mirrors the reference's Algorithm /
GpuModel / Results classes.
"""
from . import abi  # noqa: F401
from .engine import Engine, make_sim, spectra_dict  # noqa: F401

__all__ = ["abi", "Engine", "make_sim", "spectra_dict"]
