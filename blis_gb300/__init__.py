"""blis_gb300: GB300 (sm_103a) implementation of BLIS's dense hot path.

The product is the C-ABI shared library libblis_gb300.so (declared in
include/blis_gb300.h).  This package builds it (build.py), binds it
(_lib.py) and mirrors the reference's BLAS/typed entry points for Python
callers (blas.py) and device-resident torch tensors (dev.py).
"""
from . import _lib  # noqa: F401

__all__ = ["_lib"]
