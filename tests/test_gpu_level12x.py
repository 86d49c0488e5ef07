"""dscal, dcopy, idamax, dger and dtrsv on the GPU (gb_level12x.cu) against
the CPU oracle: scal, copy, amax and ger bit for bit (the same one rounding
per element, the same index rule), trsv within the substitution's error
bound; strided, negative-increment and zero-increment cases as the
reference's loops define them."""
import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,inc", [(1000003, 1), (777, 3), (5, 1), (1, 1)])
@pytest.mark.parametrize("alpha", [2.5, 0.0, 1.0, -0.5])
def test_dscal_bit_exact(n, inc, alpha):
    x0 = po.uniform((n * inc,), 1)
    if alpha == 0.0:
        x0[::7] = np.nan  # alpha == 0 sets zeros without reading x
    x = x0.copy()
    blas.dscal(n, alpha, x, inc)
    ref = x0.copy()
    po.dscalv(alpha, ref, n=n, incx=inc)
    assert np.array_equal(x, ref, equal_nan=True)


def test_dscal_negative_and_zero_increment():
    x0 = po.uniform((30,), 2)
    x = x0.copy()
    blas.dscal(10, 3.0, x, -3)  # the same elements as incx = 3
    ref = x0.copy()
    ref[0:30:3] *= 3.0
    assert np.array_equal(x, ref)
    x = x0.copy()
    blas.bli_dscalv(0.5, x, n=4, incx=0)  # the reference scales x[0] four times
    assert x[0] == x0[0] * 0.5 * 0.5 * 0.5 * 0.5 and np.array_equal(x[1:], x0[1:])


@pytest.mark.parametrize("n,incx,incy", [(2000001, 1, 1), (1001, 2, 3), (1001, -2, 1), (7, 1, 0)])
def test_dcopy(n, incx, incy):
    x = po.uniform((n * abs(incx),), 3)
    y0 = po.uniform((max(1, n * abs(incy)),), 4)
    y = y0.copy()
    blas.dcopy(n, x, incx, y, incy)
    # BLAS negative increments start at the far end (frame/include/bli_blas_macro_defs.h:50-75)
    xs = x[(n - 1) * -incx::incx] if incx < 0 else x[::incx]
    ref = y0.copy()
    if incy == 0:
        ref[0] = xs[n - 1]
    else:
        ref[::incy][:n] = xs[:n]
    assert np.array_equal(y, ref)


@pytest.mark.parametrize("n,inc", [(3000017, 1), (100001, 3), (1, 1)])
def test_idamax_matches_oracle(n, inc):
    x = po.uniform((n * inc,), 5)
    x[(n // 3) * inc] = 7.0
    x[(2 * n // 3) * inc] = -7.0  # a tie: the first stays
    assert blas.idamax(n, x, inc) == po.damaxv(x, n=n, incx=inc) + 1
    assert blas.bli_damaxv(x, n=n, incx=inc) == po.damaxv(x, n=n, incx=inc)


def test_amaxv_nan_rule_and_infinities():
    n = 500000
    x = po.uniform((n,), 6)
    x[123456] = np.inf
    x[400000] = np.nan
    x[450000] = np.nan
    assert blas.bli_damaxv(x) == 400000 == po.damaxv(x)
    x[400000] = x[450000] = 0.0
    assert blas.bli_damaxv(x) == 123456 == po.damaxv(x)
    assert blas.bli_damaxv(np.zeros(9)) == 0


@pytest.mark.parametrize("m,n,incx,incy", [(4096, 3000, 1, 1), (333, 77, 2, -1), (1, 5, 1, 1), (7, 1, 1, 1)])
@pytest.mark.parametrize("alpha", [0.75, 0.0])
def test_dger_bit_exact(m, n, incx, incy, alpha):
    a0 = po.uniform((m, n), 7)
    x = po.uniform((m * abs(incx),), 8)
    y = po.uniform((n * abs(incy),), 9)
    a = np.asfortranarray(a0.copy())
    blas.dger(m, n, alpha, x, incx, y, incy, a, m)
    xs = x[(m - 1) * -incx::incx] if incx < 0 else x[::incx]
    ys = y[(n - 1) * -incy::incy] if incy < 0 else y[::incy]
    ref = np.asfortranarray(a0.copy())
    po.dger(alpha, np.ascontiguousarray(xs[:m]), np.ascontiguousarray(ys[:n]), ref)
    assert np.array_equal(a, ref)


def test_bli_dger_row_major():
    m, n = 257, 300
    a0 = po.uniform((m, n), 10, order="C")
    x = po.uniform((m,), 11)
    y = po.uniform((n,), 12)
    a = a0.copy(order="C")
    blas.bli_dger(-1.5, x, y, a)
    assert np.allclose(a, a0 - 1.5 * np.outer(x, y), rtol=0, atol=4 * H.EPS)


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
@pytest.mark.parametrize("m,inc", [(1000, 1), (129, -2), (1, 1)])
def test_dtrsv_residual(uplo, trans, diag, m, inc):
    a = np.asfortranarray(H.normalize(po.uniform((m, m), 13)) + 2.0 * np.eye(m))
    b = po.uniform((m,), 14)
    x = np.zeros(m * abs(inc))
    xv = x[(m - 1) * -inc::inc] if inc < 0 else x[::inc]
    xv[:m] = b
    blas.dtrsv(uplo, trans, diag, m, a, m, x, inc)
    sol = (x[(m - 1) * -inc::inc] if inc < 0 else x[::inc])[:m]
    t = np.tril(a) if uplo == "L" else np.triu(a)
    if diag == "U":
        t = t - np.diag(np.diag(t)) + np.eye(m)
    t = t.T if trans == "T" else t
    assert np.linalg.norm(t @ sol - b) <= 1e-13 * max(1.0, np.linalg.norm(b))
    ref = b.copy()
    po.dtrsv(po.LOWER if uplo == "L" else po.UPPER, 8 if trans == "T" else 0,
             po.UNIT_DIAG if diag == "U" else po.NONUNIT_DIAG, 1.0, a, ref)
    assert np.max(np.abs(sol - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_bli_dtrsv_alpha_and_device_forms(gblib):
    import torch
    m = 700
    a = np.asfortranarray(H.normalize(po.uniform((m, m), 15)) + 2.0 * np.eye(m))
    b = po.uniform((m,), 16)
    x = b.copy()
    blas.bli_dtrsv(blas.UPPER, blas.NO_TRANSPOSE, blas.NONUNIT_DIAG, -2.0, a, x)
    assert np.linalg.norm(np.triu(a) @ x + 2.0 * b) <= 1e-13 * np.linalg.norm(b)
    # device entry points on torch memory
    xd = torch.from_numpy(b.copy()).cuda()
    idx = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert gblib.gb_damaxv_dev(m, xd.data_ptr(), 1, idx.data_ptr(), None) == 0
    assert gblib.gb_dscalv_dev(m, 3.0, xd.data_ptr(), 1, None) == 0
    yd = torch.zeros(m, dtype=torch.float64, device="cuda")
    assert gblib.gb_dcopyv_dev(m, xd.data_ptr(), 1, yd.data_ptr(), 1, None) == 0
    assert gblib.gb_synchronize() == 0
    assert int(idx.item()) == po.damaxv(b)
    assert np.array_equal(yd.cpu().numpy(), 3.0 * b)
