"""The oracle's herk, her2k, hemm / complex symm and syr2k against numpy's
definitions of the operations: the stored triangle only, the other left as it
is, herk / her2k with the imaginary parts of C's diagonal zeroed (as BLIS's
bli_setid after gemmt, frame/3/bli_l3_oapi_ex.c:229-320), beta == 0 not
reading C, the Hermitian diagonal read as real
(ref_kernels/1m/bli_packm_cxc_diag_1er_ref.c:214-225)."""
import numpy as np
import pytest

from oracle import pyoracle as po


def _cplx(shape, seed):
    return np.asfortranarray(po.uniform(shape, seed) + 1j * po.uniform(shape, seed + 100))


def _op(x, t):
    y = x.T if t & 0x08 else x
    return np.conj(y) if t & 0x10 else y


def _tri(uplo, m):
    return np.tril(np.ones((m, m), bool)) if uplo == po.LOWER else np.triu(np.ones((m, m), bool))


@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("ta", [0x00, 0x18, 0x08, 0x10])
def test_oracle_zherk_definition(uplo, ta):
    m, k = 13, 9
    a = _cplx((k, m) if ta & 8 else (m, k), 1)
    c0 = _cplx((m, m), 2)
    c = c0.copy(order="F")
    po.zherk(uplo, ta, 0.75, a, -1.5, c)
    oa = _op(a, ta)
    full = 0.75 * (oa @ np.conj(oa).T) - 1.5 * c0
    np.fill_diagonal(full, full.diagonal().real)
    t = _tri(uplo, m)
    assert np.allclose(c[t], full[t], rtol=0, atol=1e-13)
    assert np.array_equal(c[~t], c0[~t])
    assert np.all(c.diagonal().imag == 0)
    c = np.full((m, m), np.nan + 1j * np.nan, order="F")
    po.zherk(uplo, ta, 1.0, a, 0.0, c)  # beta == 0: C is not read
    assert np.all(np.isfinite(c[t]))


@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("ta,tb", [(0x00, 0x00), (0x18, 0x18), (0x00, 0x10), (0x08, 0x18)])
def test_oracle_zher2k_definition(uplo, ta, tb):
    m, k = 12, 8
    a = _cplx((k, m) if ta & 8 else (m, k), 3)
    b = _cplx((k, m) if tb & 8 else (m, k), 4)
    c0 = _cplx((m, m), 5)
    c = c0.copy(order="F")
    al = 0.5 - 2.0j
    po.zher2k(uplo, ta, tb, al, a, b, 0.25, c)
    oa, ob = _op(a, ta), _op(b, tb)
    full = al * (oa @ np.conj(ob).T) + np.conj(al) * (ob @ np.conj(oa).T) + 0.25 * c0
    np.fill_diagonal(full, full.diagonal().real)
    t = _tri(uplo, m)
    assert np.allclose(c[t], full[t], rtol=0, atol=1e-13)
    assert np.array_equal(c[~t], c0[~t])


@pytest.mark.parametrize("side", [po.LEFT, po.RIGHT])
@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("herm,conja,tb", [(1, 0, 0x00), (0, 0, 0x00), (1, 1, 0x18), (0, 1, 0x08)])
def test_oracle_zhemm_definition(side, uplo, herm, conja, tb):
    m, n = 9, 6
    na = m if side == po.LEFT else n
    a = _cplx((na, na), 6)
    b = _cplx((n, m) if tb & 8 else (m, n), 7)
    c0 = _cplx((m, n), 8)
    # the full matrix from the stored triangle
    t = _tri(uplo, na)
    s = np.where(t, a, 0)
    other = np.where(t, a, 0).T
    if herm:
        other = np.conj(other)
    full = s + other - np.diag(np.diag(s))
    if herm:
        full[np.diag_indices(na)] = a.diagonal().real
    if conja:
        full = np.conj(full)
    c = c0.copy(order="F")
    al, be = 1.5 + 0.5j, -0.5 + 1.0j
    po.zhemm(side, uplo, herm, conja, tb, al, a, b, be, c)
    ref = al * (full @ _op(b, tb) if side == po.LEFT else _op(b, tb) @ full) + be * c0
    assert np.allclose(c, ref, rtol=0, atol=1e-13)


@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("ta,tb", [(po.NO_TRANSPOSE, po.NO_TRANSPOSE), (po.TRANSPOSE, po.TRANSPOSE),
                                   (po.NO_TRANSPOSE, po.TRANSPOSE)])
def test_oracle_dsyr2k_definition(uplo, ta, tb):
    m, k = 14, 10
    a = po.uniform((k, m) if ta else (m, k), 9)
    b = po.uniform((k, m) if tb else (m, k), 10)
    c0 = po.uniform((m, m), 11)
    c = c0.copy(order="F")
    po.dsyr2k(uplo, ta, tb, 0.5, a, b, 2.0, c, nthreads=1)
    oa = a.T if ta else a
    ob = b.T if tb else b
    full = 0.5 * (oa @ ob.T) + 0.5 * (ob @ oa.T) + 2.0 * c0
    t = _tri(uplo, m)
    assert np.allclose(c[t], full[t], rtol=0, atol=1e-13)
    assert np.array_equal(c[~t], c0[~t])


@pytest.mark.parametrize("side", [po.LEFT, po.RIGHT])
@pytest.mark.parametrize("uplo,ta,diag", [(po.LOWER, po.NO_TRANSPOSE, po.NONUNIT_DIAG),
                                          (po.UPPER, po.TRANSPOSE, po.UNIT_DIAG)])
@pytest.mark.parametrize("tb", [po.NO_TRANSPOSE, po.TRANSPOSE])
def test_oracle_dtrmm3_definition(side, uplo, ta, diag, tb):
    m, n = 12, 9
    na = m if side == po.LEFT else n
    a = po.uniform((na, na), 12)
    b = po.uniform((n, m) if tb else (m, n), 13)
    c0 = po.uniform((m, n), 14)
    t = np.tril(a) if uplo == po.LOWER else np.triu(a)
    if diag == po.UNIT_DIAG:
        t = t - np.diag(np.diag(t)) + np.eye(na)
    t = t.T if ta else t
    ob = b.T if tb else b
    c = c0.copy(order="F")
    po.dtrmm3(side, uplo, ta, diag, tb, -0.5, a, b, 2.0, c, nthreads=1)
    ref = -0.5 * (t @ ob if side == po.LEFT else ob @ t) + 2.0 * c0
    assert np.allclose(c, ref, rtol=0, atol=1e-13)
    c = np.full((m, n), np.nan, order="F")
    po.dtrmm3(side, uplo, ta, diag, tb, 0.0, a, b, 0.0, c, nthreads=1)  # alpha = beta = 0: C := 0
    assert (c == 0).all()
