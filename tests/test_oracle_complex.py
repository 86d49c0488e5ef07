"""The oracle's complex gemm against numpy's complex product, with the
conjugation bit of trans_t (0x10) and BLAS 'C' (0x18)."""
import numpy as np
import pytest

from oracle import pyoracle as po


def _cplx(shape, seed):
    return np.asfortranarray(po.uniform(shape, seed) + 1j * po.uniform(shape, seed + 100))


def _op(x, t):
    y = x.T if t & 0x08 else x
    return np.conj(y) if t & 0x10 else y


@pytest.mark.parametrize("ta", [0x00, 0x08, 0x10, 0x18])
@pytest.mark.parametrize("tb", [0x00, 0x18])
def test_oracle_zgemm_definition(ta, tb):
    m, n, k = 11, 7, 9
    a = _cplx((k, m) if ta & 8 else (m, k), 1)
    b = _cplx((n, k) if tb & 8 else (k, n), 2)
    c0 = _cplx((m, n), 3)
    c = c0.copy(order="F")
    po.zgemm(ta, tb, 0.5 - 1.25j, a, b, 2.0 + 0.5j, c)
    ref = (0.5 - 1.25j) * (_op(a, ta) @ _op(b, tb)) + (2.0 + 0.5j) * c0
    assert np.allclose(c, ref, rtol=0, atol=1e-13)
    c = np.full((m, n), np.nan + 1j * np.nan, order="F")
    po.zgemm(ta, tb, 1.0, a, b, 0.0, c)  # beta == 0: C is not read
    assert np.allclose(c, _op(a, ta) @ _op(b, tb), rtol=0, atol=1e-13)
