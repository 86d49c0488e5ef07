"""zherk / cherk, zher2k / cher2k, zsyrk / csyrk, zsyr2k / csyr2k, zhemm /
chemm, zsymm / csymm and dsyr2k on
the GPU (gb_hermitian.cu, gb_level3x.cu) against the CPU oracle: the stored
triangle within the componentwise bound of the products, the other triangle
bit-for-bit untouched, the imaginary parts of C's diagonal zero after herk /
her2k, the BLAS early return, beta = 0 with NaN in C, C stored by rows (the
merge path), more than one 1024-column block, and the precision form
bit-identical to the Ozaki model on the block-real operands."""
import numpy as np
import pytest

from blis_gb300 import _lib, blas
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

U64 = np.finfo(np.float64).eps
U32 = np.finfo(np.float32).eps
CODE = {"N": 0x00, "T": 0x08, "C": 0x18}


@pytest.fixture(autouse=True)
def native(gblib):
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    yield
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def _cplx(shape, seed, dtype=np.complex128, order="F"):
    x = po.uniform(shape, seed) + 1j * po.uniform(shape, seed + 100)
    return np.asarray(x, dtype=dtype, order=order)


def _op(x, t):
    y = x.T if t & 0x08 else x
    return np.conj(y) if t & 0x10 else y


def _tri(lower, m):
    return np.tril(np.ones((m, m), bool)) if lower else np.triu(np.ones((m, m), bool))


def _check_triangle(c, ref, c0, bound, lower):
    t = _tri(lower, c.shape[0])
    assert np.all(np.abs(c - ref)[t] <= bound[t])
    assert np.array_equal(c[~t], c0[~t])  # the other triangle is not touched


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("m,k", [(130, 90), (1, 17), (2100, 64)])
def test_zherk_vs_oracle(uplo, trans, m, k):
    a = _cplx((k, m) if trans == "C" else (m, k), 1)
    c0 = _cplx((m, m), 2)
    alpha, beta = 0.75, -1.25
    c = c0.copy(order="F")
    blas.zherk(uplo, trans, m, k, alpha, a, a.shape[0], beta, c, m)
    ref = c0.copy(order="F")
    lower = uplo == "L"
    po.zherk(po.LOWER if lower else po.UPPER, CODE[trans], alpha, a, beta, ref)
    oa = np.abs(_op(a, CODE[trans]))
    bound = 8 * (k + 4) * U64 * (abs(alpha) * (oa @ oa.T) + abs(beta) * np.abs(c0)) + 1e-300
    _check_triangle(c, ref, c0, bound, lower)
    assert np.all(c.diagonal().imag == 0)


def test_cherk_single_and_row_major_c():
    m, k = 300, 200
    a = _cplx((m, k), 3, np.complex64)
    c0 = _cplx((m, m), 4, np.complex64)
    c = c0.copy(order="F")
    blas.cherk("L", "N", m, k, 1.5, a, m, 0.5, c, m)
    A = a.astype(np.complex128)
    ref = 1.5 * (A @ np.conj(A).T) + 0.5 * c0.astype(np.complex128)
    np.fill_diagonal(ref, ref.diagonal().real)
    bound = 8 * (k + 4) * U32 * (1.5 * (np.abs(A) @ np.abs(A).T) + 0.5 * np.abs(c0)) + 1e-30
    _check_triangle(c, ref, c0, bound, True)
    # dcomplex with C stored by rows: the panels go through the scratch panel and the merge
    a = _cplx((1500, 70), 5)
    c0 = _cplx((1500, 1500), 6, order="C")
    c = c0.copy(order="C")
    blas.bli_zherk(po.UPPER, 0x00, 2.0, a, 0.0, c)
    ref = np.zeros_like(c)
    po.zherk(po.UPPER, 0x00, 2.0, a, 0.0, ref)
    oa = np.abs(a)
    _check_triangle(c, ref, c0, 8 * 74 * U64 * 2.0 * (oa @ oa.T) + 1e-300, False)


def test_zherk_early_return_alpha_zero_and_beta_zero_nan():
    m, k = 200, 50
    a = _cplx((m, k), 7)
    c0 = _cplx((m, m), 8)
    # BLAS: alpha == 0 and beta == 1 returns without touching C (the diagonal keeps its imaginary part)
    c = c0.copy(order="F")
    blas.zherk("L", "N", m, k, 0.0, a, m, 1.0, c, m)
    assert np.array_equal(c, c0)
    # the typed API scales the triangle and zeroes the diagonal's imaginary parts
    c = c0.copy(order="F")
    blas.bli_zherk(po.LOWER, 0x00, 0.0, a, 2.0, c)
    ref = 2.0 * c0
    np.fill_diagonal(ref, ref.diagonal().real)
    _check_triangle(c, ref, c0, np.zeros(c.shape), True)
    # beta == 0: C is not read
    c = np.full((m, m), np.nan + 1j * np.nan, order="F")
    blas.zherk("U", "N", m, k, 1.0, a, m, 0.0, c, m)
    assert np.all(np.isfinite(c[_tri(False, m)]))


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "C"])
@pytest.mark.parametrize("m,k", [(130, 90), (1100, 33)])
def test_zher2k_vs_oracle(uplo, trans, m, k):
    a = _cplx((k, m) if trans == "C" else (m, k), 9)
    b = _cplx((k, m) if trans == "C" else (m, k), 10)
    c0 = _cplx((m, m), 11)
    alpha, beta = 0.5 - 1.5j, 0.25
    c = c0.copy(order="F")
    blas.zher2k(uplo, trans, m, k, alpha, a, a.shape[0], b, b.shape[0], beta, c, m)
    ref = c0.copy(order="F")
    lower = uplo == "L"
    t = CODE[trans]
    po.zher2k(po.LOWER if lower else po.UPPER, t, t, alpha, a, b, beta, ref)
    oa, ob = np.abs(_op(a, t)), np.abs(_op(b, t))
    g = 2 * abs(alpha) * (oa @ ob.T + ob @ oa.T) + abs(beta) * np.abs(c0)
    _check_triangle(c, ref, c0, 8 * (2 * k + 4) * U64 * g + 1e-300, lower)
    assert np.all(c.diagonal().imag == 0)


def test_bli_zher2k_mixed_trans_and_single():
    m, k = 257, 100
    a = _cplx((m, k), 12)
    b = _cplx((k, m), 13)
    c0 = _cplx((m, m), 14)
    c = c0.copy(order="F")
    blas.bli_zher2k(po.LOWER, 0x10, 0x18, 1.0 + 1.0j, a, b, -0.5, c)  # conj(A), B^H
    ref = c0.copy(order="F")
    po.zher2k(po.LOWER, 0x10, 0x18, 1.0 + 1.0j, a, b, -0.5, ref)
    oa, ob = np.abs(a), np.abs(b.T)
    g = 2 * np.sqrt(2) * (oa @ ob.T + ob @ oa.T) + 0.5 * np.abs(c0)
    _check_triangle(c, ref, c0, 8 * (2 * k + 4) * U64 * g, True)
    a32, b32, c32 = (x.astype(np.complex64) for x in (a, b.T.copy(order="F"), c0))
    c = c32.copy(order="F")
    blas.cher2k("U", "N", m, k, 2.0j, a32, m, b32, m, 1.0, c, m)
    A, B = a32.astype(np.complex128), b32.astype(np.complex128)
    ref = 2.0j * (A @ np.conj(B).T) - 2.0j * (B @ np.conj(A).T) + c32.astype(np.complex128)
    np.fill_diagonal(ref, ref.diagonal().real)
    g = 2 * (np.abs(A) @ np.abs(B).T + np.abs(B) @ np.abs(A).T) + np.abs(c32)
    _check_triangle(c, ref, c32, 8 * (2 * k + 4) * U32 * g + 1e-30, False)


def _full(a, lower, herm, conja):
    n = a.shape[0]
    t = _tri(lower, n)
    s = np.where(t, a, 0)
    o = s.T.copy()
    if herm:
        o = np.conj(o)
    f = s + o - np.diag(np.diag(s))
    if herm:
        f[np.diag_indices(n)] = a.diagonal().real
    return np.conj(f) if conja else f


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("herm", [True, False])
def test_zhemm_zsymm_vs_oracle(side, uplo, herm):
    m, n = 150, 90
    na = m if side == "L" else n
    a = _cplx((na, na), 15)
    b = _cplx((m, n), 16)
    c0 = _cplx((m, n), 17)
    alpha, beta = 1.25 - 0.5j, 0.5 + 0.5j
    c = c0.copy(order="F")
    blas.zhemm(side, uplo, m, n, alpha, a, na, b, m, beta, c, m, herm=herm)
    ref = c0.copy(order="F")
    po.zhemm(po.LEFT if side == "L" else po.RIGHT, po.LOWER if uplo == "L" else po.UPPER, int(herm), 0, 0x00,
             alpha, a, b, beta, ref)
    f = np.abs(_full(a, uplo == "L", herm, False))
    g = abs(alpha) * (f @ np.abs(b) if side == "L" else np.abs(b) @ f) + abs(beta) * np.abs(c0)
    assert np.all(np.abs(c - ref) <= 8 * (na + 4) * U64 * g)


def test_bli_zhemm_conj_transb_single_and_alpha_zero():
    m, n = 120, 200
    a = _cplx((n, n), 18)
    b = _cplx((n, m), 19)  # op(B) = B^H is m x n
    c0 = _cplx((m, n), 20)
    c = c0.copy(order="F")
    blas.bli_zhemm(po.RIGHT, po.UPPER, 0x10, 0x18, 0.5j, a, b, 1.0, c)
    ref = c0.copy(order="F")
    po.zhemm(po.RIGHT, po.UPPER, 1, 1, 0x18, 0.5j, a, b, 1.0, ref)
    f = np.abs(_full(a, False, True, True))
    g = 0.5 * (np.abs(b.T) @ f) + np.abs(c0)
    assert np.all(np.abs(c - ref) <= 8 * (n + 4) * U64 * g)
    # alpha = 0: C := beta C
    c = c0.copy(order="F")
    blas.zsymm("L", "L", m, n, 0.0, a, n, b, n, 2.0, c, m)
    assert np.array_equal(c, 2.0 * c0)
    # single precision symm
    a32 = _cplx((m, m), 21, np.complex64)
    b32 = _cplx((m, n), 22, np.complex64)
    c = np.zeros((m, n), dtype=np.complex64, order="F")
    blas.csymm("L", "L", m, n, 1.0, a32, m, b32, m, 0.0, c, m)
    f = _full(a32.astype(np.complex128), True, False, False)
    ref = f @ b32.astype(np.complex128)
    assert np.all(np.abs(c - ref) <= 8 * (m + 4) * U32 * (np.abs(f) @ np.abs(b32)) + 1e-30)


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("m,k", [(300, 200), (2100, 40)])
def test_dsyr2k_vs_oracle(uplo, trans, m, k):
    a = po.uniform((k, m) if trans == "T" else (m, k), 23)
    b = po.uniform((k, m) if trans == "T" else (m, k), 24)
    c0 = po.uniform((m, m), 25)
    c = c0.copy(order="F")
    blas.dsyr2k(uplo, trans, m, k, 0.5, a, a.shape[0], b, b.shape[0], -1.0, c, m)
    lower = uplo == "L"
    ref = c0.copy(order="F")
    t = po.TRANSPOSE if trans == "T" else po.NO_TRANSPOSE
    po.dsyr2k(po.LOWER if lower else po.UPPER, t, t, 0.5, a, b, -1.0, ref)
    oa = np.abs(a.T if trans == "T" else a)
    ob = np.abs(b.T if trans == "T" else b)
    g = 0.5 * (oa @ ob.T + ob @ oa.T) + np.abs(c0)
    _check_triangle(c, ref, c0, 4 * (k + 4) * U64 * g, lower)


def _block_real(x):
    """Xb (rows 2i, 2i+1 = [Re x_i, -Im x_i], [Im x_i, Re x_i]) and Yb = [Re X^H; Im X^H]."""
    m, k = x.shape
    xb = np.zeros((2 * m, 2 * k), order="F")
    xb[0::2, :k], xb[1::2, :k] = x.real, x.imag
    xb[0::2, k:], xb[1::2, k:] = -x.imag, x.real
    y = np.conj(x).T
    yb = np.asfortranarray(np.vstack([y.real, y.imag]))
    return xb, yb


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_zherk_ozaki_bit_identical_to_model(uplo):
    m, k = 1100, 64
    a = np.asfortranarray(po.expspread((m, k), 26, -8, 8) + 1j * po.expspread((m, k), 27, -8, 8))
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    c0 = _cplx((m, m), 28)
    c = c0.copy(order="F")
    blas.zherk(uplo, "N", m, k, 1.0, a, m, 0.0, c, m)
    xb, yb = _block_real(a)
    p = np.zeros((2 * m, m), order="F")
    po.ozaki_dgemm(0, 0, 1.0, xb, yb, 0.0, p, 7)
    model = p[0::2] + 1j * p[1::2]
    np.fill_diagonal(model, model.diagonal().real)
    t = _tri(uplo == "L", m)
    assert np.array_equal(c[t], model[t])
    assert np.array_equal(c[~t], c0[~t])


def test_ozaki_her2k_hemm_syr2k_within_bound():
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    m, k = 600, 300
    a = _cplx((m, k), 29)
    b = _cplx((m, k), 30)
    c0 = _cplx((m, m), 31)
    c = c0.copy(order="F")
    blas.zher2k("L", "N", m, k, 1.0 - 1.0j, a, m, b, m, 1.0, c, m)
    ref = c0.copy(order="F")
    po.zher2k(po.LOWER, 0, 0, 1.0 - 1.0j, a, b, 1.0, ref)
    g = 2 * np.sqrt(2) * (np.abs(a) @ np.abs(b).T + np.abs(b) @ np.abs(a).T) + np.abs(c0)
    _check_triangle(c, ref, c0, 8 * (2 * k + 4) * U64 * g, True)
    h = _cplx((m, m), 32)
    bb = _cplx((m, 250), 33)
    cc = np.zeros((m, 250), dtype=np.complex128, order="F")
    blas.zhemm("L", "U", m, 250, 1.0, h, m, bb, m, 0.0, cc, m)
    ref = np.zeros_like(cc)
    po.zhemm(po.LEFT, po.UPPER, 1, 0, 0, 1.0, h, bb, 0.0, ref)
    f = np.abs(_full(h, False, True, False))
    assert np.all(np.abs(cc - ref) <= 8 * (m + 4) * U64 * (f @ np.abs(bb)))
    ra, rb = po.uniform((m, k), 34), po.uniform((m, k), 35)
    rc0 = po.uniform((m, m), 36)
    rc = rc0.copy(order="F")
    blas.dsyr2k("U", "N", m, k, 1.0, ra, m, rb, m, 0.5, rc, m)
    ref = rc0.copy(order="F")
    po.dsyr2k(po.UPPER, 0, 0, 1.0, ra, rb, 0.5, ref)
    g = np.abs(ra) @ np.abs(rb).T + np.abs(rb) @ np.abs(ra).T + 0.5 * np.abs(rc0)
    _check_triangle(rc, ref, rc0, 4 * (k + 4) * U64 * g, False)


def test_device_entry_points(gblib):
    import torch
    m, k = 400, 120
    a = _cplx((m, k), 37)
    ad = torch.from_numpy(a.T.copy()).cuda().t()  # column-major on the device
    cd = torch.zeros((m, m), dtype=torch.complex128, device="cuda").t().contiguous().t()
    p = lambda t: t.data_ptr()
    assert gblib.gb_zherk_dev(po.LOWER, 0, m, k, 1.0, p(ad), 1, m, 0.0, p(cd), 1, m, None) == 0
    assert gblib.gb_synchronize() == 0
    c = cd.cpu().numpy()
    ref = np.zeros((m, m), dtype=np.complex128, order="F")
    po.zherk(po.LOWER, 0, 1.0, a, 0.0, ref)
    t = _tri(True, m)
    oa = np.abs(a)
    assert np.all(np.abs(c - ref)[t] <= (8 * (k + 4) * U64 * (oa @ oa.T))[t])
    one = _lib.DComplex(1.0, 0.0)
    assert gblib.gb_zher2k_dev(po.UPPER, 0, 0, m, k, one, p(ad), 1, m, p(ad), 1, m, 0.0, p(cd), 1, m, None) == 0
    assert gblib.gb_synchronize() == 0
    c2 = cd.cpu().numpy()
    assert np.all(np.abs(c2 - 2 * ref.conj().T)[~np.tri(m, k=-1, dtype=bool)]
                  <= (2 * 8 * (2 * k + 4) * U64 * (oa @ oa.T))[~np.tri(m, k=-1, dtype=bool)])
    assert gblib.gb_zherk_dev(po.LOWER, 0, -1, k, 1.0, p(ad), 1, m, 0.0, p(cd), 1, m, None) != 0
    _lib.load().gb_clear_last_error()


def test_zherk_ozaki_nonfinite_keeps_other_triangle():
    m, k = 700, 90
    a = _cplx((m, k), 45)
    a[300, 10] = np.nan
    c0 = _cplx((m, m), 46)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    c = c0.copy(order="F")
    blas.zherk("L", "N", m, k, 1.0, a, m, 1.0, c, m)
    t = _tri(True, m)
    assert np.array_equal(c[~t], c0[~t])
    assert np.all(c.diagonal().imag == 0)
    assert np.isnan(c[300, 0].real) and np.isnan(c[699, 300].real)
    ok = np.ones(m, bool)
    ok[300] = False
    sub = np.ix_(ok, ok)
    ref = c0.copy(order="F")
    po.zherk(po.LOWER, 0, 1.0, a, 1.0, ref)
    oa = np.abs(np.nan_to_num(a))
    bound = 8 * (k + 4) * U64 * ((oa @ oa.T) + np.abs(c0))
    d = np.abs(c - ref)[sub][t[sub]]
    assert np.all(d <= bound[sub][t[sub]])


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("two", [False, True])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("m,k", [(130, 90), (1, 17), (1100, 40)])
def test_complex_syrk_syr2k_vs_numpy(dt, two, uplo, trans, m, k):
    """C := alpha op(A) op(B)^T (+ alpha op(B) op(A)^T) + beta C on the stored triangle: complex
    alpha and beta, no conjugation anywhere, the diagonal keeps its imaginary parts."""
    a = _cplx((k, m) if trans == "T" else (m, k), 11, dt)
    b = _cplx(a.shape, 12, dt)
    c0 = _cplx((m, m), 13, dt)
    alpha, beta = 0.75 - 0.5j, -1.25 + 0.25j
    c = c0.copy(order="F")
    if two:
        blas.zsyr2k(uplo, trans, m, k, alpha, a, a.shape[0], b, b.shape[0], beta, c, m)
    else:
        blas.zsyrk(uplo, trans, m, k, alpha, a, a.shape[0], beta, c, m)
    A, B, C0 = (x.astype(np.complex128) for x in (a, b, c0))
    oa, ob = (A.T, B.T) if trans == "T" else (A, B)
    if two:
        ref = alpha * (oa @ ob.T) + alpha * (ob @ oa.T) + beta * C0
        g = 2 * abs(alpha) * (np.abs(oa) @ np.abs(ob).T) + abs(beta) * np.abs(C0)
    else:
        ref = alpha * (oa @ oa.T) + beta * C0
        g = abs(alpha) * (np.abs(oa) @ np.abs(oa).T) + abs(beta) * np.abs(C0)
    eps = U64 if dt == np.complex128 else U32
    _check_triangle(c.astype(np.complex128), ref, C0, 8 * (2 * k + 4) * eps * g + 1e-300, uplo == "L")
    if m > 1:
        assert np.any(c.diagonal().imag != 0)


def test_zsyrk_beta_forms_early_return_and_error_exit():
    m, k = 200, 50
    a = _cplx((m, k), 14)
    c0 = _cplx((m, m), 15)
    low = _tri(True, m)
    # beta = 0 with NaN in C: the stored triangle is written without reading it
    c = c0.copy(order="F")
    c[low] = np.nan
    blas.zsyrk("L", "N", m, k, 1.0, a, m, 0.0, c, m)
    assert np.all(np.isfinite(c[low]))
    ref = a @ a.T
    g = np.abs(a) @ np.abs(a).T
    assert np.all(np.abs(c - ref)[low] <= 8 * (k + 4) * U64 * g[low])
    # alpha = 0, beta = 1: the BLAS early return leaves C as it is
    c = c0.copy(order="F")
    blas.zsyrk("U", "T", m, k, 0.0, a, k, 1.0, c, m)
    assert np.array_equal(c, c0)
    # alpha = 0, complex beta: the triangle scaled, the rest untouched
    c = c0.copy(order="F")
    blas.zsyrk("U", "N", m, k, 0.0, a, m, 0.5 + 2.0j, c, m)
    up = _tri(False, m)
    assert np.allclose(c[up], (0.5 + 2.0j) * c0[up], rtol=4 * U64, atol=0)
    assert np.array_equal(c[~up], c0[~up])


def test_zsyr2k_ozaki_and_device_strides():
    """The precision form (double complex under the Ozaki mode) and gb_csyr2k_dev on a row-major
    C with transposed operands."""
    torch = pytest.importorskip("torch")
    m, k = 700, 300
    a = _cplx((m, k), 16)
    b = _cplx((m, k), 17)
    c0 = _cplx((m, m), 18)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    c = c0.copy(order="F")
    blas.zsyr2k("L", "N", m, k, 1.0 + 1.0j, a, m, b, m, 2.0 - 1.0j, c, m)
    ref = (1.0 + 1.0j) * (a @ b.T + b @ a.T) + (2.0 - 1.0j) * c0
    g = 2 * np.sqrt(2) * (np.abs(a) @ np.abs(b).T) + np.sqrt(5) * np.abs(c0)
    _check_triangle(c, ref, c0, 64 * U64 * g + 1e-300, True)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    L = _lib.load()
    n, kk = 260, 70
    at = _cplx((kk, n), 19, np.complex64)  # op(A) = A^T, A stored k x n column-major
    bt = _cplx((kk, n), 20, np.complex64)
    cr = _cplx((n, n), 21, np.complex64)
    A = torch.from_numpy(np.ascontiguousarray(at.T).view(np.float32)).cuda()  # column-major at: rs 1, cs kk
    B = torch.from_numpy(np.ascontiguousarray(bt.T).view(np.float32)).cuda()
    Cd = torch.from_numpy(np.ascontiguousarray(cr).view(np.float32)).cuda()  # row-major C: rs n, cs 1
    al, be = _lib.SComplex(0.5, 0.25), _lib.SComplex(-1.0, 0.0)
    assert L.gb_csyr2k_dev(0x60, 0x08, 0x08, n, kk, al, A.data_ptr(), 1, kk, B.data_ptr(), 1, kk, be,
                           Cd.data_ptr(), n, 1, None) == 0
    assert L.gb_synchronize() == 0
    got = Cd.cpu().numpy().view(np.complex64).astype(np.complex128)
    AT, BT, C0 = at.T.astype(np.complex128), bt.T.astype(np.complex128), cr.astype(np.complex128)
    ref = (0.5 + 0.25j) * (AT @ BT.T + BT @ AT.T) - C0
    g = 2 * (np.abs(AT) @ np.abs(BT).T) + np.abs(C0)
    _check_triangle(got, ref, C0, 8 * (2 * kk + 4) * U32 * g, False)
