"""GB300-native even-odd Wilson-clover solver: a drop-in for Chroma's clover system solvers.

The compute path is ``libgbclover.so`` (hand-written sm_103a CUDA behind a C ABI,
include/gbclover.h); this package holds its ctypes binding (``gbclover``), the
Chroma-shaped host interface (``syssolver``) and the sources of synthetic inputs.
"""
from . import gbclover  # noqa: F401
