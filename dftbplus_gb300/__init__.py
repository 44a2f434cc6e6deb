"""GB300-native SCC-DFTB engine: the non-periodic Gamma-point SCC cycle, energy and forces.

The compute path is the CUDA library ``libdftbgpu.so`` (C-ABI in include/dftbgpu.h); this package
holds the host-side data formats (SKF tables, synthetic workloads) and the ctypes binding.
"""
from .model import Model, Species, PairTable  # noqa: F401
