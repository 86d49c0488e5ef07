"""Python mirror of the reference's BLAS-compat and typed-API entry points.

Each function calls the matching symbol of libblis_gb300.so through ctypes
with host (numpy) buffers, so a test reads like a call into BLIS's own
frame/compat layer: same names, same argument meaning (Fortran-style
leading dimensions, netlib increment rules, xerbla on bad arguments).
"""
import ctypes as C

import numpy as np

from . import _lib

NO_TRANSPOSE, TRANSPOSE, CONJ_NO_TRANSPOSE, CONJ_TRANSPOSE = 0x00, 0x08, 0x10, 0x18
NO_CONJUGATE, CONJUGATE = 0x00, 0x10
LOWER, UPPER = 0xC0, 0x60
LEFT, RIGHT = 0, 1
NONUNIT_DIAG, UNIT_DIAG = 0x000, 0x100
DGEMM_NATIVE, DGEMM_OZAKI, DGEMM_OZAKI_CRT = 0, 1, 2


def _i(v):
    return C.byref(C.c_int32(int(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


def _s(v):
    return C.byref(C.c_float(float(v)))


def _p(x):
    return None if x is None else x.ctypes.data_as(C.c_void_p)


def _c(ch):
    return ch.encode() if isinstance(ch, str) else ch


# ------------------------------------------------------------ Fortran BLAS
def dgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    _lib.load().dgemm_(_c(transa), _c(transb), _i(m), _i(n), _i(k), _d(alpha), _p(a), _i(lda),
                       _p(b), _i(ldb), _d(beta), _p(c), _i(ldc))


def sgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    _lib.load().sgemm_(_c(transa), _c(transb), _i(m), _i(n), _i(k), _s(alpha), _p(a), _i(lda),
                       _p(b), _i(ldb), _s(beta), _p(c), _i(ldc))


def dtrsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
    _lib.load().dtrsm_(_c(side), _c(uplo), _c(transa), _c(diag), _i(m), _i(n),
                       C.byref(C.c_double(alpha)), _p(a), _i(lda), _p(b), _i(ldb))


def strsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
    _lib.load().strsm_(_c(side), _c(uplo), _c(transa), _c(diag), _i(m), _i(n),
                       C.byref(C.c_float(alpha)), _p(a), _i(lda), _p(b), _i(ldb))


def _cscalar(v, dtype):
    return np.array([v], dtype=dtype)


def zgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    """Complex gemm on complex128 (zgemm_) or complex64 (cgemm_) Fortran-order arrays."""
    fn = _lib.load().zgemm_ if c.dtype == np.complex128 else _lib.load().cgemm_
    al, be = _cscalar(alpha, c.dtype), _cscalar(beta, c.dtype)
    fn(_c(transa), _c(transb), _i(m), _i(n), _i(k), _p(al), _p(a), _i(lda), _p(b), _i(ldb), _p(be), _p(c), _i(ldc))


cgemm = zgemm


def bli_zgemm(transa, transb, alpha, a, b, beta, c):
    """bli_zgemm / bli_cgemm by c's dtype; trans_t may carry the conjugation bit 0x10."""
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    fn = _lib.load().bli_zgemm if c.dtype == np.complex128 else _lib.load().bli_cgemm
    al, be = _cscalar(alpha, c.dtype), _cscalar(beta, c.dtype)
    fn(transa, transb, m, n, k, _p(al), _p(a), *_st(a), _p(b), *_st(b), _p(be), _p(c), *_st(c))


def ztrsm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
    """Complex trsm on complex128 (ztrsm_) or complex64 (ctrsm_) Fortran-order arrays, by b's dtype."""
    fn = _lib.load().ztrsm_ if b.dtype == np.complex128 else _lib.load().ctrsm_
    al = _cscalar(alpha, b.dtype)
    fn(_c(side), _c(uplo), _c(transa), _c(diag), _i(m), _i(n), _p(al), _p(a), _i(lda), _p(b), _i(ldb))


ctrsm = ztrsm


def ztrmm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
    """Complex trmm on complex128 (ztrmm_) or complex64 (ctrmm_) Fortran-order arrays, by b's dtype."""
    fn = _lib.load().ztrmm_ if b.dtype == np.complex128 else _lib.load().ctrmm_
    al = _cscalar(alpha, b.dtype)
    fn(_c(side), _c(uplo), _c(transa), _c(diag), _i(m), _i(n), _p(al), _p(a), _i(lda), _p(b), _i(ldb))


ctrmm = ztrmm


def zgemv(trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
    """zgemv_ / cgemv_ by y's dtype."""
    fn = _lib.load().zgemv_ if y.dtype == np.complex128 else _lib.load().cgemv_
    al, be = _cscalar(alpha, y.dtype), _cscalar(beta, y.dtype)
    fn(_c(trans), _i(m), _i(n), _p(al), _p(a), _i(lda), _p(x), _i(incx), _p(be), _p(y), _i(incy))


cgemv = zgemv


def _real_dtype(c):
    return np.float64 if c.dtype == np.complex128 else np.float32


def zherk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
    """zherk_ / cherk_ by c's dtype (alpha, beta real; trans 'N' or 'C')."""
    L = _lib.load()
    fn = L.zherk_ if c.dtype == np.complex128 else L.cherk_
    rt = _real_dtype(c)
    al, be = np.array([alpha], dtype=rt), np.array([beta], dtype=rt)
    fn(_c(uplo), _c(trans), _i(n), _i(k), _p(al), _p(a), _i(lda), _p(be), _p(c), _i(ldc))


cherk = zherk


def zher2k(uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    """zher2k_ / cher2k_ by c's dtype (alpha complex, beta real)."""
    L = _lib.load()
    fn = L.zher2k_ if c.dtype == np.complex128 else L.cher2k_
    al, be = _cscalar(alpha, c.dtype), np.array([beta], dtype=_real_dtype(c))
    fn(_c(uplo), _c(trans), _i(n), _i(k), _p(al), _p(a), _i(lda), _p(b), _i(ldb), _p(be), _p(c), _i(ldc))


cher2k = zher2k


def zsyrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
    """zsyrk_ / csyrk_ by c's dtype (alpha, beta complex; trans 'N' or 'T')."""
    L = _lib.load()
    fn = L.zsyrk_ if c.dtype == np.complex128 else L.csyrk_
    al, be = _cscalar(alpha, c.dtype), _cscalar(beta, c.dtype)
    fn(_c(uplo), _c(trans), _i(n), _i(k), _p(al), _p(a), _i(lda), _p(be), _p(c), _i(ldc))


csyrk = zsyrk


def zsyr2k(uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    """zsyr2k_ / csyr2k_ by c's dtype (alpha, beta complex; trans 'N' or 'T')."""
    L = _lib.load()
    fn = L.zsyr2k_ if c.dtype == np.complex128 else L.csyr2k_
    al, be = _cscalar(alpha, c.dtype), _cscalar(beta, c.dtype)
    fn(_c(uplo), _c(trans), _i(n), _i(k), _p(al), _p(a), _i(lda), _p(b), _i(ldb), _p(be), _p(c), _i(ldc))


csyr2k = zsyr2k


def zhemm(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc, herm=True):
    """zhemm_ / chemm_ (herm) or zsymm_ / csymm_ by c's dtype."""
    L = _lib.load()
    z = c.dtype == np.complex128
    fn = (L.zhemm_ if z else L.chemm_) if herm else (L.zsymm_ if z else L.csymm_)
    al, be = _cscalar(alpha, c.dtype), _cscalar(beta, c.dtype)
    fn(_c(side), _c(uplo), _i(m), _i(n), _p(al), _p(a), _i(lda), _p(b), _i(ldb), _p(be), _p(c), _i(ldc))


chemm = zhemm


def zsymm(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc):
    zhemm(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc, herm=False)


csymm = zsymm


def dsyr2k(uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    _lib.load().dsyr2k_(_c(uplo), _c(trans), _i(n), _i(k), _d(alpha), _p(a), _i(lda), _p(b), _i(ldb), _d(beta),
                        _p(c), _i(ldc))


def dscal(n, alpha, x, incx=1):
    _lib.load().dscal_(_i(n), _d(alpha), _p(x), _i(incx))


def dcopy(n, x, incx, y, incy):
    _lib.load().dcopy_(_i(n), _p(x), _i(incx), _p(y), _i(incy))


def idamax(n, x, incx=1):
    return int(_lib.load().idamax_(_i(n), _p(x), _i(incx)))


def dger(m, n, alpha, x, incx, y, incy, a, lda):
    _lib.load().dger_(_i(m), _i(n), _d(alpha), _p(x), _i(incx), _p(y), _i(incy), _p(a), _i(lda))


def dtrsv(uplo, trans, diag, m, a, lda, x, incx=1):
    _lib.load().dtrsv_(_c(uplo), _c(trans), _c(diag), _i(m), _p(a), _i(lda), _p(x), _i(incx))


def bli_dscalv(alpha, x, n=None, incx=1):
    n = x.size if n is None else n
    _lib.load().bli_dscalv(0, n, _d(alpha), _p(x), incx)


def bli_dcopyv(x, y, n=None, incx=1, incy=1):
    n = x.size if n is None else n
    _lib.load().bli_dcopyv(0, n, _p(x), incx, _p(y), incy)


def bli_damaxv(x, n=None, incx=1):
    n = x.size if n is None else n
    idx = C.c_int64(-1)
    _lib.load().bli_damaxv(n, _p(x), incx, C.byref(idx))
    return idx.value


def bli_dger(alpha, x, y, a, incx=1, incy=1):
    m, n = a.shape
    _lib.load().bli_dger(0, 0, m, n, _d(alpha), _p(x), incx, _p(y), incy, _p(a), *_st(a))


def bli_dtrsv(uplo, transa, diag, alpha, a, x, incx=1):
    m = a.shape[0]
    _lib.load().bli_dtrsv(uplo, transa, diag, m, _d(alpha), _p(a), *_st(a), _p(x), incx)


def dtrmm(side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb):
    _lib.load().dtrmm_(_c(side), _c(uplo), _c(transa), _c(diag), _i(m), _i(n), _d(alpha), _p(a), _i(lda),
                       _p(b), _i(ldb))


def dsymm(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc):
    _lib.load().dsymm_(_c(side), _c(uplo), _i(m), _i(n), _d(alpha), _p(a), _i(lda), _p(b), _i(ldb), _d(beta),
                       _p(c), _i(ldc))


def dsyrk(uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
    _lib.load().dsyrk_(_c(uplo), _c(trans), _i(n), _i(k), _d(alpha), _p(a), _i(lda), _d(beta), _p(c), _i(ldc))


def dgemmt(uplo, transa, transb, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    _lib.load().dgemmt_(_c(uplo), _c(transa), _c(transb), _i(n), _i(k), _d(alpha), _p(a), _i(lda), _p(b),
                        _i(ldb), _d(beta), _p(c), _i(ldc))


def dgemv(trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
    _lib.load().dgemv_(_c(trans), _i(m), _i(n), C.byref(C.c_double(alpha)), _p(a), _i(lda), _p(x),
                       _i(incx), C.byref(C.c_double(beta)), _p(y), _i(incy))


def daxpy(n, alpha, x, incx, y, incy):
    _lib.load().daxpy_(_i(n), C.byref(C.c_double(alpha)), _p(x), _i(incx), _p(y), _i(incy))


def ddot(n, x, incx, y, incy):
    return _lib.load().ddot_(_i(n), _p(x), _i(incx), _p(y), _i(incy))


def dgemm_batch(transa, transb, m, n, k, alpha, a_list, lda, b_list, ldb, beta, c_list, ldc,
                group_size, dtype=np.float64):
    """Grouped interface of frame/compat/extra/bla_gemm_batch.c: per-group
    parameter arrays plus flat per-problem pointer arrays."""
    g = len(group_size)
    ta = (C.c_char * g)(*[_c(t) for t in transa])
    tb = (C.c_char * g)(*[_c(t) for t in transb])
    ia = lambda v: (C.c_int32 * g)(*[int(x) for x in v])
    fty = C.c_double if dtype == np.float64 else C.c_float
    fa = lambda v: (fty * g)(*[float(x) for x in v])
    total = sum(group_size)
    pa = (C.c_void_p * total)(*[x.ctypes.data for x in a_list])
    pb = (C.c_void_p * total)(*[x.ctypes.data for x in b_list])
    pc = (C.c_void_p * total)(*[x.ctypes.data for x in c_list])
    fn = _lib.load().dgemm_batch_ if dtype == np.float64 else _lib.load().sgemm_batch_
    fn(ta, tb, ia(m), ia(n), ia(k), fa(alpha), pa, ia(lda), pb, ia(ldb), fa(beta), pc, ia(ldc),
       _i(g), ia(group_size))


# ------------------------------------------------------------ typed BLIS API
def _st(x):
    it = x.itemsize
    return x.strides[0] // it, x.strides[1] // it


def bli_dgemm(transa, transb, alpha, a, b, beta, c):
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    _lib.load().bli_dgemm(transa, transb, m, n, k, _d(alpha), _p(a), *_st(a), _p(b), *_st(b),
                          _d(beta), _p(c), *_st(c))


def bli_sgemm(transa, transb, alpha, a, b, beta, c):
    m, n = c.shape
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    _lib.load().bli_sgemm(transa, transb, m, n, k, _s(alpha), _p(a), *_st(a), _p(b), *_st(b),
                          _s(beta), _p(c), *_st(c))


def bli_dtrsm(side, uplo, transa, diag, alpha, a, b):
    m, n = b.shape
    _lib.load().bli_dtrsm(side, uplo, transa, diag, m, n, _d(alpha), _p(a), *_st(a), _p(b), *_st(b))


def bli_dtrmm(side, uplo, transa, diag, alpha, a, b):
    m, n = b.shape
    _lib.load().bli_dtrmm(side, uplo, transa, diag, m, n, _d(alpha), _p(a), *_st(a), _p(b), *_st(b))


def bli_dsymm(side, uplo, alpha, a, b, beta, c, transb=0):
    m, n = c.shape
    _lib.load().bli_dsymm(side, uplo, 0, transb, m, n, _d(alpha), _p(a), *_st(a), _p(b), *_st(b), _d(beta),
                          _p(c), *_st(c))


def bli_dsyrk(uplo, transa, alpha, a, beta, c):
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    _lib.load().bli_dsyrk(uplo, transa, m, k, _d(alpha), _p(a), *_st(a), _d(beta), _p(c), *_st(c))


def bli_dgemmt(uplo, transa, transb, alpha, a, b, beta, c):
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    _lib.load().bli_dgemmt(uplo, transa, transb, m, k, _d(alpha), _p(a), *_st(a), _p(b), *_st(b), _d(beta),
                           _p(c), *_st(c))


def bli_zherk(uplo, transa, alpha, a, beta, c):
    """bli_zherk / bli_cherk by c's dtype."""
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    L = _lib.load()
    fn = L.bli_zherk if c.dtype == np.complex128 else L.bli_cherk
    rt = _real_dtype(c)
    al, be = np.array([alpha], dtype=rt), np.array([beta], dtype=rt)
    fn(uplo, transa, m, k, _p(al), _p(a), *_st(a), _p(be), _p(c), *_st(c))


def bli_zher2k(uplo, transa, transb, alpha, a, b, beta, c):
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    L = _lib.load()
    fn = L.bli_zher2k if c.dtype == np.complex128 else L.bli_cher2k
    al, be = _cscalar(alpha, c.dtype), np.array([beta], dtype=_real_dtype(c))
    fn(uplo, transa, transb, m, k, _p(al), _p(a), *_st(a), _p(b), *_st(b), _p(be), _p(c), *_st(c))


def bli_zhemm(side, uplo, conja, transb, alpha, a, b, beta, c, herm=True):
    """bli_zhemm / bli_chemm (herm) or bli_zsymm / bli_csymm by c's dtype."""
    m, n = c.shape
    L = _lib.load()
    z = c.dtype == np.complex128
    fn = (L.bli_zhemm if z else L.bli_chemm) if herm else (L.bli_zsymm if z else L.bli_csymm)
    al, be = _cscalar(alpha, c.dtype), _cscalar(beta, c.dtype)
    fn(side, uplo, conja, transb, m, n, _p(al), _p(a), *_st(a), _p(b), *_st(b), _p(be), _p(c), *_st(c))


def bli_dtrmm3(side, uplo, transa, diag, transb, alpha, a, b, beta, c):
    """C := beta C + alpha op(A) op(B) (LEFT) or beta C + alpha op(B) op(A) (RIGHT), A triangular."""
    m, n = c.shape
    _lib.load().bli_dtrmm3(side, uplo, transa, diag, transb, m, n, _d(alpha), _p(a), *_st(a), _p(b), *_st(b),
                           _d(beta), _p(c), *_st(c))


def bli_dsyr2k(uplo, transa, transb, alpha, a, b, beta, c):
    m = c.shape[0]
    k = a.shape[0] if transa & TRANSPOSE else a.shape[1]
    _lib.load().bli_dsyr2k(uplo, transa, transb, m, k, _d(alpha), _p(a), *_st(a), _p(b), *_st(b), _d(beta), _p(c),
                           *_st(c))


def bli_dgemv(transa, alpha, a, x, beta, y, incx=1, incy=1):
    m, n = a.shape
    _lib.load().bli_dgemv(transa, 0, m, n, _d(alpha), _p(a), *_st(a), _p(x), incx, _d(beta), _p(y),
                          incy)


def bli_daxpyv(alpha, x, y, n=None, incx=1, incy=1):
    n = x.size if n is None else n
    _lib.load().bli_daxpyv(0, n, _d(alpha), _p(x), incx, _p(y), incy)


def bli_ddotv(x, y, n=None, incx=1, incy=1):
    n = x.size if n is None else n
    rho = np.zeros(1)
    _lib.load().bli_ddotv(0, 0, n, _p(x), incx, _p(y), incy, _p(rho))
    return float(rho[0])


# ------------------------------------------------------------ controls
SGEMM_FMA, SGEMM_SPLIT, SGEMM_AUTO = 0, 1, 2


def set_sgemm_mode(mode):
    return _lib.check(_lib.load().gb_set_sgemm_mode(mode), "gb_set_sgemm_mode")


def set_dgemm_mode(mode, slices=8):
    return _lib.check(_lib.load().gb_set_dgemm_mode(mode, slices), "gb_set_dgemm_mode")


def launch_count():
    return int(_lib.load().gb_launch_count())
