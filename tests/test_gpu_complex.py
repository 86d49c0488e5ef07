"""zgemm / cgemm on the GPU (gb_complex.cu: one real gemm on the block-real
form) against the CPU oracle's complex gemm and numpy: every trans /
conjugate-transpose pair, complex alpha and beta, beta = 0 with NaN in C,
k = 0, general strides, the Ozaki form for zgemm and the device entry."""
import numpy as np
import pytest

from blis_gb300 import _lib, blas
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

U64 = np.finfo(np.float64).eps
U32 = np.finfo(np.float32).eps


@pytest.fixture(autouse=True)
def native(gblib):
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    yield
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def _cplx(shape, seed, dtype=np.complex128, order="F"):
    x = po.uniform(shape, seed) + 1j * po.uniform(shape, seed + 100)
    return np.asarray(x, dtype=dtype, order=order)


def _op(x, t):
    y = x.T if t in ("T", "C") else x
    return np.conj(y) if t == "C" else y


def _bound(alpha, a_op, b_op, beta, c0, eps, k):
    # componentwise, |x| of a complex product bounded by (|re| + |im|) of each factor
    g = abs(alpha) * (np.abs(a_op) @ np.abs(b_op)) + abs(beta) * np.abs(c0)
    return 8 * (k + 4) * eps * g + 1e-300


@pytest.mark.parametrize("ta", ["N", "T", "C"])
@pytest.mark.parametrize("tb", ["N", "T", "C"])
@pytest.mark.parametrize("m,n,k", [(130, 70, 90), (1, 33, 17), (65, 1, 300)])
def test_zgemm_vs_oracle(ta, tb, m, n, k):
    a = _cplx((k, m) if ta != "N" else (m, k), 1)
    b = _cplx((n, k) if tb != "N" else (k, n), 2)
    c0 = _cplx((m, n), 3)
    alpha, beta = 0.75 - 0.5j, -1.0 + 0.25j
    c = c0.copy(order="F")
    blas.zgemm(ta, tb, m, n, k, alpha, a, a.shape[0], b, b.shape[0], beta, c, m)
    code = {"N": 0x00, "T": 0x08, "C": 0x18}
    ref = c0.copy(order="F")
    po.zgemm(code[ta], code[tb], alpha, a, b, beta, ref)
    assert np.all(np.abs(c - ref) <= _bound(alpha, _op(a, ta), _op(b, tb), beta, c0, U64, k))


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "T")])
def test_cgemm_single(ta, tb):
    m, n, k = 200, 150, 120
    a = _cplx((k, m) if ta != "N" else (m, k), 4, np.complex64)
    b = _cplx((n, k) if tb != "N" else (k, n), 5, np.complex64)
    c0 = _cplx((m, n), 6, np.complex64)
    alpha, beta = 1.5 + 0.5j, 0.5 - 0.5j
    c = c0.copy(order="F")
    blas.cgemm(ta, tb, m, n, k, alpha, a, a.shape[0], b, b.shape[0], beta, c, m)
    A, B, C0 = (x.astype(np.complex128) for x in (a, b, c0))
    ref = alpha * (_op(A, ta) @ _op(B, tb)) + beta * C0
    assert np.all(np.abs(c - ref) <= _bound(alpha, _op(A, ta), _op(B, tb), beta, C0, U32, k))


def test_zgemm_beta_zero_ignores_nan_and_k_zero():
    m, n, k = 64, 48, 40
    a = _cplx((m, k), 7)
    b = _cplx((k, n), 8)
    c = np.full((m, n), np.nan + 1j * np.nan, order="F")
    blas.zgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    assert np.isfinite(c).all()
    assert np.all(np.abs(c - a @ b) <= _bound(1.0, a, b, 0.0, np.zeros_like(c), U64, k))
    c0 = _cplx((m, n), 9)
    c = c0.copy(order="F")
    blas.zgemm("N", "N", m, n, 0, 1.0, a, m, b, 1, 2.0j, c, m)  # k = 0: C := beta C
    assert np.allclose(c, 2.0j * c0, rtol=0, atol=1e-15)


def test_zgemm_ozaki_and_typed_conj_no_transpose():
    m, n, k = 300, 260, 333
    a = _cplx((m, k), 10)
    b = _cplx((k, n), 11)
    c0 = _cplx((m, n), 12)
    ref = 1j * (a @ b) + 0.5 * c0
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    c = c0.copy(order="F")
    blas.zgemm("N", "N", m, n, k, 1j, a, m, b, k, 0.5, c, m)
    assert np.all(np.abs(c - ref) <= _bound(1j, a, b, 0.5, c0, U64, k))
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    # bli_zgemm with row-major operands and conj-no-transpose (0x10) on A
    ar = np.ascontiguousarray(a)
    br = np.ascontiguousarray(b)
    cr = np.ascontiguousarray(c0)
    blas.bli_zgemm(0x10, 0x00, 2.0, ar, br, -1.0, cr)
    ref = 2.0 * (np.conj(a) @ b) - c0
    assert np.all(np.abs(cr - ref) <= _bound(2.0, a, b, 1.0, c0, U64, k))


def test_zgemm_device_entry(gblib):
    import torch
    m, n, k = 257, 129, 65
    a = _cplx((m, k), 13)
    b = _cplx((k, n), 14)
    ad = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    bd = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    cd = torch.zeros((n, m), dtype=torch.complex128, device="cuda").t()
    al, be = _lib.DComplex(1.0, -1.0), _lib.DComplex(0.0, 0.0)
    assert gblib.gb_zgemm_dev(0, 0, m, n, k, al, ad.data_ptr(), 1, m, bd.data_ptr(), 1, k, be, cd.data_ptr(), 1, m,
                              None) == 0
    assert gblib.gb_synchronize() == 0
    ref = (1.0 - 1.0j) * (a @ b)
    assert np.all(np.abs(cd.cpu().numpy() - ref) <= _bound(1.0 - 1.0j, a, b, 0.0, ref, U64, k))


def test_per_call_ozaki_form_and_complex_host_alias(gblib):
    # gb_dgemm_ozaki: the Ozaki form for one call while the library stays native
    import ctypes as C
    m, n, k = 300, 200, 250
    a = po.expspread((m, k), 20, -10, 10)
    b = po.expspread((k, n), 21, -10, 10)
    c = np.zeros((m, n), order="F")
    al, be = C.c_double(1.0), C.c_double(0.0)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    gblib.gb_dgemm_ozaki(0, 0, m, n, k, C.byref(al), p(a), 1, m, p(b), 1, k, C.byref(be), p(c), 1, m, 7)
    ref = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, a, b, 0.0, ref, 7)
    assert np.array_equal(c, ref)
    nat = np.zeros((m, n), order="F")
    blas.dgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, nat, m)  # still the native form
    assert not np.array_equal(nat, ref)
    g = np.abs(a) @ np.abs(b)
    assert np.all(np.abs(nat - ref) <= 4 * (k + 2) * U64 * g)
    # gb_zgemm: the sandbox's complex alias
    z1 = _cplx((40, 30), 22)
    z2 = _cplx((30, 20), 23)
    zc = np.zeros((40, 20), dtype=np.complex128, order="F")
    one, zero = np.array([1.0 + 0j]), np.array([0j])
    gblib.gb_zgemm(0, 0, 40, 20, 30, p(one), p(z1), 1, 40, p(z2), 1, 30, p(zero), p(zc), 1, 40)
    assert np.all(np.abs(zc - z1 @ z2) <= _bound(1.0, z1, z2, 0.0, zc, U64, 30))


def _ztri(a, uplo, diag):
    t = np.tril(a) if uplo == "L" else np.triu(a)
    if diag == "U":
        t = t - np.diag(np.diag(t)) + np.eye(a.shape[0])
    return t


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("diag", ["N", "U"])
@pytest.mark.parametrize("m,n", [(150, 90), (65, 1), (1, 7)])
def test_ztrsm_residual(side, uplo, trans, diag, m, n):
    # the testsuite's trsm check: || op(A) X - alpha B || small against || B || (test_trsm.c residual)
    na = m if side == "L" else n
    a = _cplx((na, na), 30) / na + 2.0 * np.eye(na)
    a = np.asfortranarray(a)
    b0 = _cplx((m, n), 31)
    x = b0.copy(order="F")
    alpha = 0.5 + 1.5j
    blas.ztrsm(side, uplo, trans, diag, m, n, alpha, a, na, x, m)
    t = _op(_ztri(a, uplo, diag), trans)
    lhs = t @ x if side == "L" else x @ t
    assert np.linalg.norm(lhs - alpha * b0) <= 1e-13 * np.linalg.norm(alpha * b0)


def test_ztrsm_ozaki_updates_and_alpha_zero():
    m, n = 700, 300
    a = np.asfortranarray(_cplx((m, m), 32) / m + 3.0 * np.eye(m))
    b0 = _cplx((m, n), 33)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    x = b0.copy(order="F")
    blas.ztrsm("L", "L", "C", "N", m, n, 1.0, a, m, x, m)
    t = np.conj(np.tril(a)).T
    assert np.linalg.norm(t @ x - b0) <= 1e-13 * np.linalg.norm(b0)
    x[:] = np.nan  # alpha = 0: B := 0 without reading it
    blas.ztrsm("L", "L", "C", "N", m, n, 0.0, a, m, x, m)
    assert (x == 0).all()


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("diag", ["N", "U"])
@pytest.mark.parametrize("m,n", [(150, 90), (65, 1), (1, 7), (300, 260)])
def test_ctrsm_residual(side, uplo, trans, diag, m, n):
    # single complex: FP32 diagonal solves and cgemm updates, residual against FP32's epsilon
    na = m if side == "L" else n
    a = np.asfortranarray(_cplx((na, na), 34, np.complex64) / na + 2.0 * np.eye(na, dtype=np.complex64))
    b0 = _cplx((m, n), 35, np.complex64)
    x = b0.copy(order="F")
    alpha = np.complex64(0.5 + 1.5j)
    blas.ctrsm(side, uplo, trans, diag, m, n, alpha, a, na, x, m)
    t = _op(_ztri(a.astype(np.complex128), uplo, diag), trans)
    xd = x.astype(np.complex128)
    lhs = t @ xd if side == "L" else xd @ t
    rhs = complex(alpha) * b0.astype(np.complex128)
    assert np.linalg.norm(lhs - rhs) <= 64 * max(m, n) * U32 * np.linalg.norm(rhs)


def test_ctrsm_general_strides_and_alpha_zero():
    """gb_ctrsm_dev on a row-major A and a B with a leading dimension larger than m; then alpha =
    0 sets B to zero without reading it (NaN there stays out)."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    m, n, ldb = 520, 130, 530
    a = _cplx((m, m), 36, np.complex64) / m + 2.0 * np.eye(m, dtype=np.complex64)
    a_rm = np.ascontiguousarray(a)  # row-major: rs = m, cs = 1
    b0 = _cplx((m, n), 37, np.complex64)
    bbuf = np.zeros((ldb, n), dtype=np.complex64, order="F")
    bbuf[:m] = b0
    A = torch.from_numpy(a_rm.view(np.float32)).cuda()
    B = torch.from_numpy(np.ascontiguousarray(bbuf.T).view(np.float32)).cuda()
    one = _lib.SComplex(1.0, 0.0)
    assert L.gb_ctrsm_dev(0, 0xC0, 0x18, 0x100, m, n, one, A.data_ptr(), m, 1, B.data_ptr(), 1, ldb, None) == 0
    assert L.gb_synchronize() == 0
    x = B.cpu().numpy().view(np.complex64).T[:m].astype(np.complex128)
    t = np.conj(_ztri(a.astype(np.complex128), "L", "U")).T
    assert np.linalg.norm(t @ x - b0) <= 64 * m * U32 * np.linalg.norm(b0)
    assert (B.cpu().numpy().view(np.complex64).T[m:] == 0).all()  # rows past m untouched
    B.fill_(float("nan"))
    zero = _lib.SComplex(0.0, 0.0)
    assert L.gb_ctrsm_dev(0, 0xC0, 0, 0, m, n, zero, A.data_ptr(), m, 1, B.data_ptr(), 1, ldb, None) == 0
    assert L.gb_synchronize() == 0
    bz = B.cpu().numpy().view(np.complex64).T
    assert (bz[:m] == 0).all() and np.isnan(bz[m:]).all()


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("diag", ["N", "U"])
def test_complex_trmm_vs_numpy(dt, side, uplo, trans, diag):
    """ztrmm_ / ctrmm_: B := alpha op(tri(A)) B or alpha B op(tri(A)); the other triangle of A
    (NaN here) and, with a unit diagonal, A's diagonal are not read."""
    m, n = 150, 70
    na = m if side == "L" else n
    a = _cplx((na, na), 40, dt)
    other = np.triu(np.ones((na, na), bool), 1) if uplo == "L" else np.tril(np.ones((na, na), bool), -1)
    a[other] = np.nan
    if diag == "U":
        np.fill_diagonal(a, np.nan)
    b0 = _cplx((m, n), 41, dt)
    x = b0.copy(order="F")
    alpha = 0.5 - 1.25j
    blas.ztrmm(side, uplo, trans, diag, m, n, alpha, a, na, x, m)
    t = _op(_ztri(np.where(np.isnan(a), 0, a).astype(np.complex128), uplo, diag), trans)
    B0 = b0.astype(np.complex128)
    ref = alpha * (t @ B0 if side == "L" else B0 @ t)
    g = abs(alpha) * ((np.abs(t) @ np.abs(B0)) if side == "L" else (np.abs(B0) @ np.abs(t)))
    eps = U64 if dt == np.complex128 else U32
    assert np.all(np.abs(x.astype(np.complex128) - ref) <= 8 * (na + 4) * eps * g + 1e-300)


def test_complex_trmm_alpha_zero_ozaki_and_device_strides():
    torch = pytest.importorskip("torch")
    m, n = 300, 120
    a = _cplx((m, m), 42) + 2.0 * np.eye(m)
    x = np.full((m, n), np.nan, dtype=np.complex128, order="F")
    blas.ztrmm("L", "U", "N", "N", m, n, 0.0, a, m, x, m)  # alpha = 0: B := 0 without reading it
    assert (x == 0).all()
    b0 = _cplx((m, n), 43)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    x = b0.copy(order="F")
    blas.ztrmm("L", "L", "C", "N", m, n, 1.0, a, m, x, m)
    t = np.conj(np.tril(a)).T
    assert np.all(np.abs(x - t @ b0) <= 64 * U64 * (np.abs(t) @ np.abs(b0)))
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    L = _lib.load()
    ac = _cplx((n, n), 44, np.complex64)
    bc = _cplx((m, n), 45, np.complex64)
    A = torch.from_numpy(np.ascontiguousarray(ac.T).view(np.float32)).cuda()  # column-major A: rs 1, cs n
    B = torch.from_numpy(np.ascontiguousarray(bc).view(np.float32)).cuda()  # row-major B: rs n, cs 1
    al = _lib.SComplex(2.0, 0.0)
    assert L.gb_ctrmm_dev(1, 0x60, 0x08, 0x100, m, n, al, A.data_ptr(), 1, n, B.data_ptr(), n, 1, None) == 0
    assert L.gb_synchronize() == 0
    got = B.cpu().numpy().view(np.complex64).astype(np.complex128)
    t = _ztri(ac.astype(np.complex128), "U", "U").T
    ref = 2.0 * (bc.astype(np.complex128) @ t)
    assert np.all(np.abs(got - ref) <= 8 * (n + 4) * U32 * 2.0 * (np.abs(bc.astype(np.complex128)) @ np.abs(t)))


def _strided(v, inc, dt):
    """v laid out with increment inc (BLAS convention: a negative inc stores v from the far end)."""
    n = len(v)
    buf = np.full(1 + (n - 1) * abs(inc), np.nan, dtype=dt) if n else np.zeros(1, dt)
    idx = np.arange(n) * abs(inc)
    buf[idx if inc > 0 else idx[::-1]] = v
    return buf


def _unstrided(buf, n, inc):
    idx = np.arange(n) * abs(inc)
    return buf[idx if inc > 0 else idx[::-1]]


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
@pytest.mark.parametrize("m,n", [(300, 200), (3, 5000), (5000, 3), (1, 1)])
@pytest.mark.parametrize("incx,incy", [(1, 1), (-2, 3)])
def test_complex_gemv_vs_numpy(dt, trans, m, n, incx, incy):
    a = _cplx((m, n), 50, dt)
    ly, lx = (n, m) if trans != "N" else (m, n)
    xv = _cplx((lx,), 51, dt)
    y0 = _cplx((ly,), 52, dt)
    alpha, beta = 1.5 - 0.5j, -0.25 + 2.0j
    xb, yb = _strided(xv, incx, dt), _strided(y0, incy, dt)
    blas.zgemv(trans, m, n, alpha, a, m, xb, incx, beta, yb, incy)
    got = _unstrided(yb, ly, incy).astype(np.complex128)
    A, X, Y0 = a.astype(np.complex128), xv.astype(np.complex128), y0.astype(np.complex128)
    op = _op(A, trans)
    ref = alpha * (op @ X) + beta * Y0
    g = abs(alpha) * (np.abs(op) @ np.abs(X)) + abs(beta) * np.abs(Y0)
    eps = U64 if dt == np.complex128 else U32
    assert np.all(np.abs(got - ref) <= 8 * (lx + 4) * eps * g)
    if abs(incy) > 1:  # the gaps between y's elements are not written
        gaps = np.ones(len(yb), bool)
        gaps[np.arange(ly) * abs(incy)] = False
        assert np.all(np.isnan(yb[gaps]))


def test_complex_gemv_beta_zero_quirk_and_device_conj():
    torch = pytest.importorskip("torch")
    m, n = 400, 250
    a = _cplx((m, n), 53)
    xv = _cplx((n,), 54)
    y = np.full(m, np.nan, dtype=np.complex128)
    blas.zgemv("N", m, n, 1.0, a, m, xv, 1, 0.0, y, 1)  # beta = 0: y is not read
    assert np.all(np.abs(y - a @ xv) <= 8 * (n + 4) * U64 * (np.abs(a) @ np.abs(xv)))
    y0 = _cplx((m,), 55)
    y = y0.copy()
    blas.zgemv("N", m, 0, 1.0, a, m, xv, 1, 3.0, y, 1)  # nothing to add: y left as it is (netlib)
    assert np.array_equal(y, y0)
    # gb_cgemv_dev, A row-major (the warp-per-row kernel for op = N), conjugated x, conjugate-only A
    L = _lib.load()
    ac = _cplx((m, n), 56, np.complex64)
    xc = _cplx((n,), 57, np.complex64)
    yc = _cplx((m,), 58, np.complex64)
    A = torch.from_numpy(np.ascontiguousarray(ac).view(np.float32)).cuda()
    X = torch.from_numpy(xc.view(np.float32).copy()).cuda()
    Y = torch.from_numpy(yc.view(np.float32).copy()).cuda()
    assert L.gb_cgemv_dev(0x10, 0x10, m, n, _lib.SComplex(1.0, 1.0), A.data_ptr(), n, 1, X.data_ptr(), 1,
                          _lib.SComplex(0.5, 0.0), Y.data_ptr(), 1, None) == 0
    assert L.gb_synchronize() == 0
    got = Y.cpu().numpy().view(np.complex64).astype(np.complex128)
    A2, X2 = np.conj(ac.astype(np.complex128)), np.conj(xc.astype(np.complex128))
    ref = (1.0 + 1.0j) * (A2 @ X2) + 0.5 * yc.astype(np.complex128)
    g = np.sqrt(2) * (np.abs(A2) @ np.abs(X2)) + 0.5 * np.abs(yc)
    assert np.all(np.abs(got - ref) <= 8 * (n + 4) * U32 * g)
