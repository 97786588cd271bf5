"""GB300-native force-and-integrate engine for the Solaris N-body simulator.

The compute path is the in-tree CUDA library ``libsolaris_gb300.so``
(hand-written sm_103a kernels behind the C-ABI in include/solaris_gb300.h);
this package holds its ctypes binding (:mod:`.abi`, :mod:`.engine`), the
build recipe (:mod:`.build`) and the synthetic scenario generators
(:mod:`.scenarios`).
"""
from . import abi, scenarios  # noqa: F401

__all__ = ["abi", "scenarios"]
