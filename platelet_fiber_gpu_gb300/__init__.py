"""GB300-native coupled platelet / fibrin / lattice-Boltzmann step.

The product is the CUDA library `libpfgpu.so` built from `csrc/` and its C
ABI (include/pfgpu.h).  This package holds its build recipe, the ctypes
binding (`gpu`), the scene description (`scene`), mesh/topology preprocessing
(`mesh`), the synthetic workloads (`workloads`), the reference-format I/O
(`refio`) and the continuous-batching serving loop (`serving`).
"""

__version__ = "0.1.0"
