"""GB300-native miniSOD2D hex convection/diffusion kernels.

The compute path is libmsod.so (hand-written sm_103a CUDA behind a C ABI,
include/msod.h).  This package is its Python host side: ctypes binding
(``capi``), the reference-shaped kernel calls over CUDA tensors
(``kernels``), host element setup / mesh / fields (``fem``) and the named
workloads (``workload``).
"""
from . import capi, fem  # noqa: F401
from .capi import MsodError, MsodLibraryMissing  # noqa: F401

__version__ = "1.0.0"


def load():
    """Load libmsod.so, failing loudly if it was not built."""
    return capi.lib()
