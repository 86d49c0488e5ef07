"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, as the checker or the timed CPU baseline.  Arrays are numpy
arrays; strides are in elements, BLIS style (rs, cs).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

# BLIS enum encodings (frame/include/bli_type_defs.h)
NO_TRANSPOSE, TRANSPOSE = 0x00, 0x08
NO_CONJUGATE, CONJUGATE = 0x00, 0x10
LOWER, UPPER = 0xC0, 0x60
LEFT, RIGHT = 0, 1
NONUNIT_DIAG, UNIT_DIAG = 0x000, 0x100

_lib = None
_i64 = C.c_int64
_dp = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.orc_hash.restype = C.c_uint64
        L.orc_hash.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_fill_uniform.argtypes = [C.c_void_p, _i64, C.c_uint64, C.c_double, C.c_double]
        L.orc_fill_uniform_f.argtypes = [C.c_void_p, _i64, C.c_uint64, C.c_double, C.c_double]
        L.orc_fill_expspread.argtypes = [C.c_void_p, _i64, C.c_uint64, C.c_int, C.c_int]
        L.orc_fill_narrow_pow2.argtypes = [C.c_void_p, _i64, C.c_uint64]
        g = [C.c_int, C.c_int, _i64, _i64, _i64]
        L.orc_dgemm.argtypes = g + [C.c_double, C.c_void_p, _i64, _i64, C.c_void_p, _i64, _i64,
                                    C.c_double, C.c_void_p, _i64, _i64, C.c_int]
        L.orc_sgemm.argtypes = g + [C.c_float, C.c_void_p, _i64, _i64, C.c_void_p, _i64, _i64,
                                    C.c_float, C.c_void_p, _i64, _i64, C.c_int]
        L.orc_dtrsm.argtypes = [C.c_int] * 4 + [_i64, _i64, C.c_double, C.c_void_p, _i64, _i64,
                                                 C.c_void_p, _i64, _i64, C.c_int]
        L.orc_dtrmm.argtypes = [C.c_int] * 4 + [_i64, _i64, C.c_double, C.c_void_p, _i64, _i64,
                                                 C.c_void_p, _i64, _i64, C.c_int]
        L.orc_dsymm.argtypes = [C.c_int, C.c_int, _i64, _i64, C.c_double, C.c_void_p, _i64, _i64,
                                C.c_void_p, _i64, _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_int]
        L.orc_dgemmt.argtypes = [C.c_int] * 3 + [_i64, _i64, C.c_double, C.c_void_p, _i64, _i64,
                                                  C.c_void_p, _i64, _i64, C.c_double, C.c_void_p, _i64,
                                                  _i64, C.c_int]
        L.orc_zgemm.argtypes = [C.c_int, C.c_int, _i64, _i64, _i64, C.c_void_p, C.c_void_p, _i64, _i64,
                                C.c_void_p, _i64, _i64, C.c_void_p, C.c_void_p, _i64, _i64]
        L.orc_zherk.argtypes = [C.c_int, C.c_int, _i64, _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_double,
                                C.c_void_p, _i64, _i64]
        L.orc_zher2k.argtypes = [C.c_int, C.c_int, C.c_int, _i64, _i64, C.c_void_p, C.c_void_p, _i64, _i64,
                                 C.c_void_p, _i64, _i64, C.c_double, C.c_void_p, _i64, _i64]
        L.orc_zhemm.argtypes = [C.c_int] * 5 + [_i64, _i64, C.c_void_p, C.c_void_p, _i64, _i64, C.c_void_p, _i64,
                                                _i64, C.c_void_p, C.c_void_p, _i64, _i64]
        L.orc_dtrmm3.argtypes = [C.c_int] * 5 + [_i64, _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_void_p, _i64,
                                                 _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_int]
        L.orc_dsyr2k.argtypes = [C.c_int] * 3 + [_i64, _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_void_p,
                                                 _i64, _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_int]
        L.orc_dscalv.argtypes = [_i64, C.c_double, C.c_void_p, _i64]
        L.orc_dcopyv.argtypes = [_i64, C.c_void_p, _i64, C.c_void_p, _i64]
        L.orc_damaxv.argtypes = [_i64, C.c_void_p, _i64, C.c_void_p]
        L.orc_dger.argtypes = [_i64, _i64, C.c_double, C.c_void_p, _i64, C.c_void_p, _i64, C.c_void_p, _i64,
                               _i64]
        L.orc_dtrsv.argtypes = [C.c_int] * 3 + [_i64, C.c_double, C.c_void_p, _i64, _i64, C.c_void_p, _i64]
        L.orc_dgemv.argtypes = [C.c_int, C.c_int, _i64, _i64, C.c_double, C.c_void_p, _i64, _i64,
                                C.c_void_p, _i64, C.c_double, C.c_void_p, _i64]
        L.orc_daxpyv.argtypes = [C.c_int, _i64, C.c_double, C.c_void_p, _i64, C.c_void_p, _i64]
        L.orc_ddotv.argtypes = [C.c_int, C.c_int, _i64, C.c_void_p, _i64, C.c_void_p, _i64,
                                C.c_void_p]
        L.orc_dd_gemm_entries.argtypes = g + [C.c_double, C.c_void_p, _i64, _i64, C.c_void_p,
                                              _i64, _i64, C.c_double, C.c_void_p, _i64, _i64,
                                              _i64, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_int]
        L.orc_dd_dotv.argtypes = [_i64, C.c_void_p, _i64, C.c_void_p, _i64, C.c_void_p,
                                  C.c_void_p]
        L.orc_ozaki_kpart_limit.restype = _i64
        L.orc_ozaki_kpart_limit.argtypes = [C.c_int]
        L.orc_ozaki_split.argtypes = [_i64, _i64, C.c_void_p, _i64, _i64, C.c_int, C.c_void_p,
                                      C.c_void_p]
        L.orc_ozaki_crt_bits.restype = C.c_int
        L.orc_ozaki_crt_bits.argtypes = [C.c_int, _i64]
        L.orc_ozaki_crt_dgemm.restype = C.c_int
        L.orc_ozaki_crt_dgemm.argtypes = g + [C.c_double, C.c_void_p, _i64, _i64, C.c_void_p, _i64,
                                              _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_int,
                                              C.c_int]
        L.orc_ozaki_dgemm.restype = C.c_int
        L.orc_ozaki_dgemm.argtypes = g + [C.c_double, C.c_void_p, _i64, _i64, C.c_void_p, _i64,
                                          _i64, C.c_double, C.c_void_p, _i64, _i64, C.c_int,
                                          C.c_int]
        _lib = L
    return _lib


def _p(x):
    return x.ctypes.data_as(C.c_void_p)


def _strides(x):
    """(rs, cs) of a 2-D numpy array, in elements."""
    it = x.itemsize
    return x.strides[0] // it, x.strides[1] // it


def nthreads_default():
    return max(1, min(os.cpu_count() or 1, 64))


# ---------------------------------------------------------------- RNG
def uniform(shape, seed, lo=-1.0, hi=1.0, dtype=np.float64, order="F"):
    x = np.empty(shape, dtype=dtype, order=order)
    flat = x.reshape(-1, order="A")
    if dtype == np.float64:
        lib().orc_fill_uniform(_p(flat), flat.size, seed, lo, hi)
    else:
        lib().orc_fill_uniform_f(_p(flat), flat.size, seed, lo, hi)
    return x


def expspread(shape, seed, emin=-20, emax=20, order="F"):
    x = np.empty(shape, dtype=np.float64, order=order)
    flat = x.reshape(-1, order="A")
    lib().orc_fill_expspread(_p(flat), flat.size, seed, emin, emax)
    return x


def narrow_pow2(shape, seed, order="F"):
    x = np.empty(shape, dtype=np.float64, order=order)
    flat = x.reshape(-1, order="A")
    lib().orc_fill_narrow_pow2(_p(flat), flat.size, seed)
    return x


def hash64(seed, idx):
    return lib().orc_hash(seed, idx)


# ---------------------------------------------------------------- ops
def dgemm(transa, transb, alpha, a, b, beta, c, nthreads=None):
    """C := beta*C + alpha*op(A)*op(B) in place (BLIS semantics)."""
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    nt = nthreads or nthreads_default()
    fn = lib().orc_dgemm if c.dtype == np.float64 else lib().orc_sgemm
    fn(transa, transb, m, n, k, alpha, _p(a), *_strides(a), _p(b), *_strides(b), beta, _p(c),
       *_strides(c), nt)
    return c


sgemm = dgemm


def dtrsm(side, uplo, transa, diag, alpha, a, b, nthreads=None):
    m, n = b.shape
    lib().orc_dtrsm(side, uplo, transa, diag, m, n, alpha, _p(a), *_strides(a), _p(b),
                    *_strides(b), nthreads or nthreads_default())
    return b


def dtrmm(side, uplo, transa, diag, alpha, a, b, nthreads=None):
    m, n = b.shape
    lib().orc_dtrmm(side, uplo, transa, diag, m, n, alpha, _p(a), *_strides(a), _p(b),
                    *_strides(b), nthreads or nthreads_default())
    return b


def dsymm(side, uplo, alpha, a, b, beta, c, nthreads=None):
    m, n = c.shape
    lib().orc_dsymm(side, uplo, m, n, alpha, _p(a), *_strides(a), _p(b), *_strides(b), beta, _p(c),
                    *_strides(c), nthreads or nthreads_default())
    return c


def dgemmt(uplo, transa, transb, alpha, a, b, beta, c, nthreads=None):
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    lib().orc_dgemmt(uplo, transa, transb, m, k, alpha, _p(a), *_strides(a), _p(b), *_strides(b), beta,
                     _p(c), *_strides(c), nthreads or nthreads_default())
    return c


def zgemm(transa, transb, alpha, a, b, beta, c):
    """Complex gemm on complex128 arrays (strides in complex elements); trans_t 0x10 conjugates."""
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    al = np.array([alpha], dtype=np.complex128)
    be = np.array([beta], dtype=np.complex128)
    st = lambda x: (x.strides[0] // x.itemsize, x.strides[1] // x.itemsize)
    lib().orc_zgemm(transa, transb, m, n, k, _p(al), _p(a), *st(a), _p(b), *st(b), _p(be), _p(c), *st(c))
    return c


def _zst(x):
    return (x.strides[0] // x.itemsize, x.strides[1] // x.itemsize)


def zherk(uplo, transa, alpha, a, beta, c):
    """herk on complex128 arrays: the uplo triangle of C := alpha op(A) op(A)^H + beta C, the
    imaginary parts of C's diagonal zeroed (alpha, beta real)."""
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    lib().orc_zherk(uplo, transa, m, k, alpha, _p(a), *_zst(a), beta, _p(c), *_zst(c))
    return c


def zher2k(uplo, transa, transb, alpha, a, b, beta, c):
    """her2k on complex128 arrays (alpha complex, beta real)."""
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    al = np.array([alpha], dtype=np.complex128)
    lib().orc_zher2k(uplo, transa, transb, m, k, _p(al), _p(a), *_zst(a), _p(b), *_zst(b), beta, _p(c),
                     *_zst(c))
    return c


def zhemm(side, uplo, herm, conja, transb, alpha, a, b, beta, c):
    """hemm (herm=1) / complex symm (herm=0) on complex128 arrays."""
    m, n = c.shape
    al = np.array([alpha], dtype=np.complex128)
    be = np.array([beta], dtype=np.complex128)
    lib().orc_zhemm(side, uplo, herm, conja, transb, m, n, _p(al), _p(a), *_zst(a), _p(b), *_zst(b), _p(be),
                    _p(c), *_zst(c))
    return c


def dtrmm3(side, uplo, transa, diag, transb, alpha, a, b, beta, c, nthreads=None):
    m, n = c.shape
    lib().orc_dtrmm3(side, uplo, transa, diag, transb, m, n, alpha, _p(a), *_strides(a), _p(b), *_strides(b), beta,
                     _p(c), *_strides(c), nthreads or nthreads_default())
    return c


def dsyr2k(uplo, transa, transb, alpha, a, b, beta, c, nthreads=None):
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    lib().orc_dsyr2k(uplo, transa, transb, m, k, alpha, _p(a), *_strides(a), _p(b), *_strides(b), beta,
                     _p(c), *_strides(c), nthreads or nthreads_default())
    return c


def dscalv(alpha, x, n=None, incx=1):
    n = x.size if n is None else n
    lib().orc_dscalv(n, alpha, _p(x), incx)
    return x


def dcopyv(x, y, n=None, incx=1, incy=1):
    n = x.size if n is None else n
    lib().orc_dcopyv(n, _p(x), incx, _p(y), incy)
    return y


def damaxv(x, n=None, incx=1):
    n = x.size if n is None else n
    idx = C.c_int64(-1)
    lib().orc_damaxv(n, _p(x), incx, C.byref(idx))
    return idx.value


def dger(alpha, x, y, a, incx=1, incy=1):
    m, n = a.shape
    lib().orc_dger(m, n, alpha, _p(x), incx, _p(y), incy, _p(a), *_strides(a))
    return a


def dtrsv(uplo, transa, diag, alpha, a, x, incx=1):
    m = a.shape[0]
    lib().orc_dtrsv(uplo, transa, diag, m, alpha, _p(a), *_strides(a), _p(x), incx)
    return x


def dgemv(transa, alpha, a, x, beta, y, incx=1, incy=1):
    m, n = a.shape
    lib().orc_dgemv(transa, 0, m, n, alpha, _p(a), *_strides(a), _p(x), incx, beta, _p(y), incy)
    return y


def daxpyv(alpha, x, y, n=None, incx=1, incy=1):
    n = x.size if n is None else n
    lib().orc_daxpyv(0, n, alpha, _p(x), incx, _p(y), incy)
    return y


def ddotv(x, y, n=None, incx=1, incy=1):
    n = x.size if n is None else n
    rho = np.zeros(1)
    lib().orc_ddotv(0, 0, n, _p(x), incx, _p(y), incy, _p(rho))
    return float(rho[0])


def dd_gemm_entries(transa, transb, alpha, a, b, beta, c, ii, jj, nthreads=None):
    """Double-double value of (alpha*op(A)*op(B) + beta*C)[ii, jj] as (hi, lo)."""
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    ii = np.ascontiguousarray(ii, dtype=np.int64)
    jj = np.ascontiguousarray(jj, dtype=np.int64)
    hi = np.empty(ii.size)
    lo = np.empty(ii.size)
    lib().orc_dd_gemm_entries(transa, transb, m, n, k, alpha, _p(a), *_strides(a), _p(b),
                              *_strides(b), beta, _p(c), *_strides(c), ii.size, _p(ii), _p(jj),
                              _p(hi), _p(lo), nthreads or nthreads_default())
    return hi, lo


def dd_gemm_full(transa, transb, alpha, a, b, beta, c, nthreads=None):
    m, n = c.shape
    jj, ii = np.meshgrid(np.arange(n), np.arange(m))
    hi, lo = dd_gemm_entries(transa, transb, alpha, a, b, beta, c, ii.ravel(), jj.ravel(),
                             nthreads)
    return hi.reshape(m, n), lo.reshape(m, n)


def dd_dotv(x, y):
    hi = np.zeros(1)
    lo = np.zeros(1)
    lib().orc_dd_dotv(x.size, _p(x), 1, _p(y), 1, _p(hi), _p(lo))
    return float(hi[0]), float(lo[0])


def ozaki_kpart_limit(slices):
    return int(lib().orc_ozaki_kpart_limit(slices))


def ozaki_split(r, slices):
    """Split the rows of a 2-D array: returns (exps[rows], digits[slices, rows, k])."""
    rows, k = r.shape
    exps = np.empty(rows, dtype=np.int32)
    digits = np.empty((slices, rows, k), dtype=np.int16)
    lib().orc_ozaki_split(rows, k, _p(r), *_strides(r), slices, _p(exps), _p(digits))
    return exps, digits


def ozaki_dgemm(transa, transb, alpha, a, b, beta, c, slices, nthreads=None):
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    return lib().orc_ozaki_dgemm(transa, transb, m, n, k, alpha, _p(a), *_strides(a), _p(b),
                                 *_strides(b), beta, _p(c), *_strides(c), slices,
                                 nthreads or nthreads_default())


def ozaki_crt_bits(moduli, k):
    return lib().orc_ozaki_crt_bits(moduli, k)


def ozaki_crt_dgemm(transa, transb, alpha, a, b, beta, c, moduli, nthreads=None):
    """The CRT form's model: exact integer product of the scaled operands, one rounding."""
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    return lib().orc_ozaki_crt_dgemm(transa, transb, m, n, k, alpha, _p(a), *_strides(a), _p(b),
                                     *_strides(b), beta, _p(c), *_strides(c), moduli,
                                     nthreads or nthreads_default())


def componentwise_error(c, hi, lo):
    """max |c - (hi+lo)| / |hi+lo| over entries with a nonzero exact value."""
    d = np.abs((c - hi) - lo)
    den = np.abs(hi)
    mask = den > 0
    if not mask.any():
        return float(np.max(d)) if d.size else 0.0
    return float(np.max(d[mask] / den[mask]))
