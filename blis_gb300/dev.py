"""Device-pointer bindings of the gb_ addon for torch tensors already in HBM.

Strides are taken from the tensors (BLIS (rs, cs) convention, elements) and
every call is issued on the tensor's current torch CUDA stream, so torch
CUDA events recorded on that stream bracket exactly the library's kernels.
"""
import ctypes as C

import torch

from . import _lib


_LEGACY_DEFAULT_STREAM = 1  # cudaStreamLegacy: a NULL handle would select the library's own stream


def _stream():
    h = torch.cuda.current_stream().cuda_stream
    return C.c_void_p(h if h else _LEGACY_DEFAULT_STREAM)


def _rc(t):
    return t.stride(0), t.stride(1)


def _k(trans, a):
    return a.shape[0] if trans & 0x08 else a.shape[1]


def dgemm(transa, transb, alpha, a, b, beta, c):
    m, n = c.shape
    rc = _lib.load().gb_dgemm_dev(transa, transb, m, n, _k(transa, a), alpha, a.data_ptr(), *_rc(a),
                                  b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c), _stream())
    return _lib.check(rc, "gb_dgemm_dev")


def dgemm_ozaki(transa, transb, alpha, a, b, beta, c, slices=8):
    m, n = c.shape
    rc = _lib.load().gb_dgemm_ozaki_dev(transa, transb, m, n, _k(transa, a), alpha, a.data_ptr(),
                                        *_rc(a), b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c),
                                        slices, _stream())
    return _lib.check(rc, "gb_dgemm_ozaki_dev")


def dgemm_ozaki_crt(transa, transb, alpha, a, b, beta, c, moduli=16):
    """The CRT form of the Ozaki product: `moduli` residue products."""
    m, n = c.shape
    rc = _lib.load().gb_dgemm_ozaki_crt_dev(transa, transb, m, n, _k(transa, a), alpha, a.data_ptr(),
                                            *_rc(a), b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c),
                                            moduli, _stream())
    return _lib.check(rc, "gb_dgemm_ozaki_crt_dev")


def sgemm(transa, transb, alpha, a, b, beta, c):
    m, n = c.shape
    rc = _lib.load().gb_sgemm_dev(transa, transb, m, n, _k(transa, a), alpha, a.data_ptr(), *_rc(a),
                                  b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c), _stream())
    return _lib.check(rc, "gb_sgemm_dev")


def bgemm(transa, transb, alpha, a, b, beta, c, config=None):
    """C (fp32) := alpha op(A) op(B) + beta C for bf16 tensors a, b; config
    None lets the library choose (selector or threshold rule)."""
    k = _k(transa, a)
    L = _lib.load()
    if config is None:
        rc = L.gb_bgemm_dev(transa, transb, c.shape[0], c.shape[1], k, alpha, a.data_ptr(), *_rc(a), b.data_ptr(),
                            *_rc(b), beta, c.data_ptr(), *_rc(c), _stream())
    else:
        rc = L.gb_gemm_config_dev(2, config, transa, transb, c.shape[0], c.shape[1], k, alpha, a.data_ptr(), *_rc(a),
                                  b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c), _stream())
    _lib.check(rc, "gb_bgemm_dev")


def dtrsm(side, uplo, transa, diag, alpha, a, b):
    m, n = b.shape
    rc = _lib.load().gb_dtrsm_dev(side, uplo, transa, diag, m, n, alpha, a.data_ptr(), *_rc(a),
                                  b.data_ptr(), *_rc(b), _stream())
    return _lib.check(rc, "gb_dtrsm_dev")


def dscalv(alpha, x, incx=1, n=None):
    n = x.numel() if n is None else n
    return _lib.check(_lib.load().gb_dscalv_dev(n, alpha, x.data_ptr(), incx, _stream()), "gb_dscalv_dev")


def dcopyv(x, y, incx=1, incy=1, n=None):
    n = x.numel() if n is None else n
    return _lib.check(_lib.load().gb_dcopyv_dev(n, x.data_ptr(), incx, y.data_ptr(), incy, _stream()),
                      "gb_dcopyv_dev")


def damaxv(x, index, incx=1, n=None):
    """0-based index of the first largest |x_i| (first NaN) into the int64 tensor `index`."""
    n = x.numel() if n is None else n
    return _lib.check(_lib.load().gb_damaxv_dev(n, x.data_ptr(), incx, index.data_ptr(), _stream()),
                      "gb_damaxv_dev")


def dger(alpha, x, y, a, incx=1, incy=1):
    m, n = a.shape
    return _lib.check(_lib.load().gb_dger_dev(m, n, alpha, x.data_ptr(), incx, y.data_ptr(), incy, a.data_ptr(),
                                              *_rc(a), _stream()), "gb_dger_dev")


def dtrsv(uplo, transa, diag, alpha, a, x, incx=1):
    m = a.shape[0]
    return _lib.check(_lib.load().gb_dtrsv_dev(uplo, transa, diag, m, alpha, a.data_ptr(), *_rc(a), x.data_ptr(),
                                               incx, _stream()), "gb_dtrsv_dev")


def dtrmm(side, uplo, transa, diag, alpha, a, b):
    m, n = b.shape
    rc = _lib.load().gb_dtrmm_dev(side, uplo, transa, diag, m, n, alpha, a.data_ptr(), *_rc(a),
                                  b.data_ptr(), *_rc(b), _stream())
    return _lib.check(rc, "gb_dtrmm_dev")


def dsymm(side, uplo, alpha, a, b, beta, c):
    m, n = c.shape
    rc = _lib.load().gb_dsymm_dev(side, uplo, m, n, alpha, a.data_ptr(), *_rc(a), b.data_ptr(), *_rc(b), beta,
                                  c.data_ptr(), *_rc(c), _stream())
    return _lib.check(rc, "gb_dsymm_dev")


def dsyrk(uplo, transa, alpha, a, beta, c):
    m = c.shape[0]
    rc = _lib.load().gb_dsyrk_dev(uplo, transa, m, _k(transa, a), alpha, a.data_ptr(), *_rc(a), beta,
                                  c.data_ptr(), *_rc(c), _stream())
    return _lib.check(rc, "gb_dsyrk_dev")


def dgemmt(uplo, transa, transb, alpha, a, b, beta, c):
    m = c.shape[0]
    rc = _lib.load().gb_dgemmt_dev(uplo, transa, transb, m, _k(transa, a), alpha, a.data_ptr(), *_rc(a),
                                   b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c), _stream())
    return _lib.check(rc, "gb_dgemmt_dev")


def dsyr2k(uplo, transa, transb, alpha, a, b, beta, c):
    m = c.shape[0]
    rc = _lib.load().gb_dsyr2k_dev(uplo, transa, transb, m, _k(transa, a), alpha, a.data_ptr(), *_rc(a),
                                   b.data_ptr(), *_rc(b), beta, c.data_ptr(), *_rc(c), _stream())
    return _lib.check(rc, "gb_dsyr2k_dev")


def daxpyv(alpha, x, y, incx=1, incy=1, n=None):
    n = x.numel() if n is None else n
    rc = _lib.load().gb_daxpyv_dev(n, alpha, x.data_ptr(), incx, y.data_ptr(), incy, _stream())
    return _lib.check(rc, "gb_daxpyv_dev")


def ddotv(x, y, rho, incx=1, incy=1, n=None):
    n = x.numel() if n is None else n
    rc = _lib.load().gb_ddotv_dev(n, x.data_ptr(), incx, y.data_ptr(), incy, rho.data_ptr(), _stream())
    return _lib.check(rc, "gb_ddotv_dev")


def dgemv(transa, alpha, a, x, beta, y, incx=1, incy=1):
    m, n = a.shape
    rc = _lib.load().gb_dgemv_dev(transa, m, n, alpha, a.data_ptr(), *_rc(a), x.data_ptr(), incx, beta,
                                  y.data_ptr(), incy, _stream())
    return _lib.check(rc, "gb_dgemv_dev")


RAND_UNIFORM, RAND_EXPSPREAD, RAND_NARROW_POW2 = 0, 1, 2


def randm(x, kind, seed, p0=-1.0, p1=1.0):
    """Fill a 2-D float64/float32 CUDA tensor in place with seeded values."""
    m, n = x.shape
    is_float = 1 if x.dtype == torch.float32 else 0
    rc = _lib.load().gb_randm_dev(kind, is_float, x.data_ptr(), m, n, *_rc(x), seed, p0, p1, _stream())
    return _lib.check(rc, "gb_randm_dev")


def colmajor(m, n, dtype=torch.float64):
    """An m x n CUDA tensor with column-major strides (1, m)."""
    return torch.empty((n, m), dtype=dtype, device="cuda").t()


def dd_gemm_entries(transa, transb, alpha, a, b, beta, c, ii, jj):
    """Double-double (hi, lo) of selected entries of alpha*op(A)*op(B) + beta*C."""
    k = _k(transa, a)
    hi = torch.empty(ii.numel(), dtype=torch.float64, device="cuda")
    lo = torch.empty_like(hi)
    cp = c.data_ptr() if c is not None else None
    crs, ccs = _rc(c) if c is not None else (1, 1)
    rc = _lib.load().gb_dd_gemm_entries_dev(transa, transb, k, alpha, a.data_ptr(), *_rc(a), b.data_ptr(),
                                            *_rc(b), beta, cp, crs, ccs, ii.numel(), ii.data_ptr(),
                                            jj.data_ptr(), hi.data_ptr(), lo.data_ptr(), _stream())
    _lib.check(rc, "gb_dd_gemm_entries_dev")
    return hi, lo


def componentwise_error(c_vals, hi, lo):
    """max |c - (hi + lo)| / |hi + lo| over entries with a nonzero exact value."""
    d = ((c_vals - hi) - lo).abs()
    den = hi.abs()
    mask = den > 0
    return float((d[mask] / den[mask]).max()) if bool(mask.any()) else float(d.max())


def set_kernel_timing(on):
    _lib.load().gb_set_kernel_timing(1 if on else 0)


def kernel_time_ms(prefix):
    n = C.c_int64(0)
    ms = _lib.load().gb_kernel_time_ms(prefix.encode(), C.byref(n))
    return ms, int(n.value)


class _TraceEntry(C.Structure):
    _fields_ = [("name", C.c_char * 40), ("start_ms", C.c_double), ("end_ms", C.c_double)]


def kernel_trace(max_entries=1 << 16):
    """The recorded launches (and the host pipeline's copies) as a timeline:
    [(name, start_ms, end_ms)] from the first record's start; forgets them."""
    buf = (_TraceEntry * max_entries)()
    n = _lib.load().gb_kernel_trace(C.cast(buf, C.c_void_p), max_entries)
    return [(buf[i].name.decode(), buf[i].start_ms, buf[i].end_ms) for i in range(n)]


def synchronize():
    return _lib.check(_lib.load().gb_synchronize(), "gb_synchronize")
