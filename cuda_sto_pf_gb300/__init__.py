"""GB300-native (sm_103a) time-stepping library for the CUDA_STO_PF phase-field model.

The compute path is libpfgb.so (hand-written CUDA, C ABI in include/pfgb.h).
This package holds its in-tree build (``build``), the ctypes binding
(``capi``), the Python mirror of the reference driver (``solver``), and the
synthetic microstructure generators of the workloads (``workloads``).
"""
from . import build, capi  # noqa: F401

__all__ = ["build", "capi"]
