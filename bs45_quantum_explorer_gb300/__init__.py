"""GB300-native first-hit search for base sequences BS(n+1,n).

A drop-in for the reference solver's WZ_FIRSTHIT lane (src/solver/wz_match.cpp of
DanielGord0n/BS45_Quantum_Explorer): hand-written sm_103a CUDA kernels behind the C ABI in
include/bsfh.h (libbsfh.so), a C++ lane binary (bin/bs_firsthit) and this Python mirror.
"""
from .build import LIB, build_all, build_library  # noqa: F401

__version__ = "0.1.0"
