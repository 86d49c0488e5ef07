"""The oracle's scalv, copyv, amaxv, ger and trsv restatements against the
operations' definitions, including the reference's amaxv NaN rule (the
first NaN wins, else the first largest |x_i|)."""
import numpy as np
import pytest

from oracle import pyoracle as po


def test_oracle_scalv_copyv():
    x0 = po.uniform((50,), 1)
    x = x0.copy()
    po.dscalv(2.5, x)
    assert np.array_equal(x, 2.5 * x0)
    x = np.full(50, np.nan)
    po.dscalv(0.0, x)  # alpha == 0 sets zeros, NaN or not
    assert (x == 0.0).all()
    x = x0.copy()
    po.dscalv(-1.0, x, n=25, incx=2)
    assert np.array_equal(x[::2], -x0[::2]) and np.array_equal(x[1::2], x0[1::2])
    y = np.zeros(50)
    po.dcopyv(x0, y, n=10, incx=5, incy=1)
    assert np.array_equal(y[:10], x0[::5]) and (y[10:] == 0).all()


@pytest.mark.parametrize("vals,expect", [
    ([1.0, -3.0, 3.0, 2.0], 1),                # ties keep the first
    ([1.0, np.nan, 5.0, np.nan], 1),           # the first NaN
    ([5.0, 1.0, np.nan], 2),
    ([-np.inf, 7.0, np.inf], 0),
    ([0.0, -0.0, 0.0], 0),
    ([], 0),
])
def test_oracle_amaxv_rule(vals, expect):
    x = np.array(vals, dtype=np.float64)
    assert po.damaxv(x) == expect


def test_oracle_ger_and_trsv():
    m, n = 13, 9
    a0 = po.uniform((m, n), 2)
    x = po.uniform((m,), 3)
    y = po.uniform((n,), 4)
    a = a0.copy(order="F")
    po.dger(0.5, x, y, a)
    assert np.allclose(a, a0 + 0.5 * np.outer(x, y), rtol=0, atol=1e-15)
    t = np.tril(po.uniform((m, m), 5)) + 3 * np.eye(m)
    t = np.asfortranarray(t)
    b = po.uniform((m,), 6)
    z = b.copy()
    po.dtrsv(po.LOWER, po.NO_TRANSPOSE, po.NONUNIT_DIAG, 1.0, t, z)
    assert np.allclose(t @ z, b, rtol=0, atol=1e-13)
