"""The oracle's trmm, symm and gemmt (syrk) restatements against the
operations' definitions in numpy, and the triangle gemmt must leave alone."""
import numpy as np
import pytest

from oracle import pyoracle as po


def _tri(a, lower, unit):
    t = np.tril(a) if lower else np.triu(a)
    if unit:
        t = t - np.diag(np.diag(t)) + np.eye(a.shape[0])
    return t


@pytest.mark.parametrize("side", [po.LEFT, po.RIGHT])
@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("trans", [po.NO_TRANSPOSE, po.TRANSPOSE])
@pytest.mark.parametrize("diag", [po.NONUNIT_DIAG, po.UNIT_DIAG])
def test_oracle_trmm_definition(side, uplo, trans, diag):
    m, n = 29, 17
    na = m if side == po.LEFT else n
    a = po.uniform((na, na), 3)
    b0 = po.uniform((m, n), 4)
    b = b0.copy(order="F")
    po.dtrmm(side, uplo, trans, diag, -0.75, a, b)
    t = _tri(a, uplo == po.LOWER, diag == po.UNIT_DIAG)
    t = t.T if trans else t
    ref = -0.75 * (t @ b0 if side == po.LEFT else b0 @ t)
    assert np.allclose(b, ref, rtol=0, atol=1e-13)


@pytest.mark.parametrize("side", [po.LEFT, po.RIGHT])
@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
def test_oracle_symm_reads_one_triangle(side, uplo):
    m, n = 23, 31
    na = m if side == po.LEFT else n
    a = po.uniform((na, na), 5)
    full = np.tril(a) + np.tril(a, -1).T if uplo == po.LOWER else np.triu(a) + np.triu(a, 1).T
    junk = a.copy(order="F")  # the other triangle replaced by NaN: never read
    junk[np.triu_indices(na, 1) if uplo == po.LOWER else np.tril_indices(na, -1)] = np.nan
    b = po.uniform((m, n), 6)
    c0 = po.uniform((m, n), 7)
    c = c0.copy(order="F")
    po.dsymm(side, uplo, 1.5, junk, b, -2.0, c)
    ref = 1.5 * (full @ b if side == po.LEFT else b @ full) - 2.0 * c0
    assert np.allclose(c, ref, rtol=0, atol=1e-13)


@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("ta,tb", [(0, 0), (8, 8), (0, 8)])
def test_oracle_gemmt_triangle_only(uplo, ta, tb):
    m, k = 37, 11
    a = po.uniform((k, m) if ta else (m, k), 8)
    b = po.uniform((m, k) if tb else (k, m), 9)
    c0 = po.uniform((m, m), 10)
    c = c0.copy(order="F")
    po.dgemmt(uplo, ta, tb, 0.5, a, b, 0.25, c)
    full = 0.5 * ((a.T if ta else a) @ (b.T if tb else b)) + 0.25 * c0
    mask = np.tril(np.ones((m, m), bool)) if uplo == po.LOWER else np.triu(np.ones((m, m), bool))
    assert np.allclose(c[mask], full[mask], rtol=0, atol=1e-13)
    assert np.array_equal(c[~mask], c0[~mask])
