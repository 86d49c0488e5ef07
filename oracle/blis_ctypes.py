"""ctypes access to the reference BLIS built by oracle/ref_blis.py (test infrastructure only).

The typed API of BLIS (frame/3/bli_l3_tapi_ex.h, frame/2/bli_l2_tapi.h,
frame/1/bli_l1v_tapi.h) on numpy arrays, for the oracle pins, the golden-fixture
generator and bench.py's CPU baseline.  Enum values are BLIS's
(frame/include/bli_type_defs.h:354-427): trans N 0x00 / T 0x08, uplo lower 0xC0 /
upper 0x60, side left 0 / right 1, diag non-unit 0x000 / unit 0x100.
"""
import ctypes as C
import os

import numpy as np

from oracle import ref_blis

_lib = None
_i64 = C.c_int64
NO_TRANSPOSE, TRANSPOSE = 0x00, 0x08
LOWER, UPPER = 0xC0, 0x60
LEFT, RIGHT = 0, 1
NONUNIT, UNIT = 0x000, 0x100


def available():
    return os.path.exists(ref_blis.lib_path())


def lib(build=False):
    """The reference libblis.so of this host's sub-configuration (built on request)."""
    global _lib
    if _lib is None:
        path = ref_blis.build() if build else ref_blis.lib_path()
        if not path or not os.path.exists(path):
            raise FileNotFoundError("reference BLIS not built (python -m oracle.ref_blis)")
        # RTLD_DEEPBIND: BLIS's calls into itself (bli_dgemm -> bli_dgemm_ex -> ...) must bind to
        # its own definitions even when a library exporting the same names (libblis_gb300.so)
        # is already loaded into the process's global scope
        L = C.CDLL(path, mode=os.RTLD_LOCAL | getattr(os, "RTLD_DEEPBIND", 0))
        L.bli_init()
        vp = C.c_void_p
        L.bli_dgemm.argtypes = [C.c_int, C.c_int, _i64, _i64, _i64, vp, vp, _i64, _i64, vp, _i64, _i64,
                                vp, vp, _i64, _i64]
        L.bli_dtrsm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i64, _i64, vp, vp, _i64, _i64, vp,
                                _i64, _i64]
        L.bli_dgemv.argtypes = [C.c_int, C.c_int, _i64, _i64, vp, vp, _i64, _i64, vp, _i64, vp, vp, _i64]
        L.bli_daxpyv.argtypes = [C.c_int, _i64, vp, vp, _i64, vp, _i64]
        L.bli_ddotv.argtypes = [C.c_int, C.c_int, _i64, vp, _i64, vp, _i64, vp]
        L.bli_thread_set_num_threads.argtypes = [_i64]
        L.bli_thread_get_num_threads.restype = _i64
        L.bli_arch_query_id.restype = C.c_int
        L.bli_arch_string.restype = C.c_char_p
        L.bli_arch_string.argtypes = [C.c_int]
        _lib = L
    return _lib


def arch_name():
    L = lib()
    return L.bli_arch_string(L.bli_arch_query_id()).decode()


def set_threads(n):
    lib().bli_thread_set_num_threads(int(n))


def _p(x):
    return x.ctypes.data_as(C.c_void_p)


def _d(v):
    return C.byref(C.c_double(v))


def _st(x):
    return x.strides[0] // x.itemsize, x.strides[1] // x.itemsize


def dgemm(transa, transb, alpha, a, b, beta, c):
    """C := alpha op(A) op(B) + beta C in place (bli_dgemm)."""
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    lib().bli_dgemm(transa, transb, m, n, k, _d(alpha), _p(a), *_st(a), _p(b), *_st(b), _d(beta), _p(c),
                    *_st(c))
    return c


def dtrsm(side, uplo, transa, diag, alpha, a, b):
    """B := alpha inv(op(A)) B (left) or alpha B inv(op(A)) (right), in place (bli_dtrsm)."""
    m, n = b.shape
    lib().bli_dtrsm(side, uplo, transa, diag, m, n, _d(alpha), _p(a), *_st(a), _p(b), *_st(b))
    return b


def dgemv(transa, alpha, a, x, beta, y, incx=1, incy=1):
    m, n = a.shape
    lib().bli_dgemv(transa, 0, m, n, _d(alpha), _p(a), *_st(a), _p(x), incx, _d(beta), _p(y), incy)
    return y


def daxpyv(alpha, x, y, incx=1, incy=1, n=None):
    n = x.size // abs(incx) if n is None else n
    lib().bli_daxpyv(0, n, _d(alpha), _p(x), incx, _p(y), incy)
    return y


def ddotv(x, y, incx=1, incy=1, n=None):
    n = x.size // abs(incx) if n is None else n
    rho = C.c_double(0.0)
    lib().bli_ddotv(0, 0, n, _p(x), incx, _p(y), incy, C.byref(rho))
    return rho.value
