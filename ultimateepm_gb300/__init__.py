"""GB300-native (sm_103a) band-structure engine for UltimateEPM's per-k-point hot path.

The product is the native library ``lib/libuepm_gb300.so`` (C ABI: include/uepm_gb300.h) and the C++
adapter ``lib/libuepm_epp.so`` (the reference's uepm::pseudopotential classes, include/uepm/).
This package holds their sources (csrc/, adapter/), the in-tree build (build.py) and a ctypes mirror
of the reference's interface (api.py) for Python callers.
"""
from . import _native  # noqa: F401
from .api import BandStructure, Hamiltonian, Material, Materials, SymmetryPoints, generate_basis_vectors  # noqa: F401

__all__ = ["BandStructure", "Hamiltonian", "Material", "Materials", "SymmetryPoints", "generate_basis_vectors"]
