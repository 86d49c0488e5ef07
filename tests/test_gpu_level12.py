"""axpyv / dotv / gemv on the GPU: the reference's own DDOT/DAXPY golden
vectors through ddot_/daxpy_ (negative increments included), the DMMCH grid
of dblat2 through dgemv_, and large seeded cases against the oracle."""
import json
import os

import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _gold():
    return json.load(open(os.path.join(GOLD, "dblat1_check2.json")))


def _stest(comp, true, size, sfac):
    sd = np.asarray(comp) - np.asarray(true)
    return np.all((np.abs(sfac * sd) + np.abs(size)) - np.abs(size) == 0)


@pytest.mark.parametrize("ki", range(4))
@pytest.mark.parametrize("kn", range(4))
def test_ddot_golden_dblat1(gblib, ki, kn):
    d = _gold()
    x = np.array(d["dx1"])
    y = np.array(d["dy1"])
    rho = blas.ddot(d["ns"][kn], x, d["incxs"][ki], y, d["incys"][ki])
    assert _stest([rho], [d["dt7"][kn + 4 * ki]], [d["ssize1"][kn]], d["sfac"])


@pytest.mark.parametrize("ki", range(4))
@pytest.mark.parametrize("kn", range(4))
def test_daxpy_golden_dblat1(gblib, ki, kn):
    d = _gold()
    x = np.array(d["dx1"])
    y = np.array(d["dy1"])
    blas.daxpy(d["ns"][kn], d["sa"], x, d["incxs"][ki], y, d["incys"][ki])
    my = abs(d["incys"][ki])
    leny = d["lens"][kn + 4 * (my - 1)]
    true = [d["dt8"][j + 7 * (kn + 4 * ki)] for j in range(leny)]
    ksize = min(2, kn + 1)
    size = d["ssize2"][14 * (ksize - 1): 14 * (ksize - 1) + leny]
    assert _stest(y[:leny], true, size, d["sfac"])


@pytest.mark.parametrize("n", [1, 2, 1000003, 4 << 20])
@pytest.mark.parametrize("inc", [(1, 1), (2, 3), (-3, 1)])
def test_daxpyv_ddotv_vs_oracle(gblib, n, inc):
    incx, incy = inc
    if n > 2000000 and inc != (1, 1):
        pytest.skip("large strided case covered at smaller n")
    x = po.uniform(n * abs(incx), 1).ravel()
    y = po.uniform(n * abs(incy), 2).ravel()

    # BLAS convention: element i of the traversal; a negative increment
    # starts from the far end of the buffer
    def idx(i, inc):
        return (i if inc > 0 else n - 1 - i) * abs(inc)

    ix = np.array([idx(i, incx) for i in range(n)]) if n < 100 else (
        np.arange(n) * incx if incx > 0 else (n - 1 - np.arange(n)) * -incx)
    iy = np.array([idx(i, incy) for i in range(n)]) if n < 100 else (
        np.arange(n) * incy if incy > 0 else (n - 1 - np.arange(n)) * -incy)
    xs = np.ascontiguousarray(x[ix])
    ys_ref = np.ascontiguousarray(y[iy])
    hi, lo = po.dd_dotv(xs, ys_ref)
    rho = blas.ddot(n, x, incx, y, incy)
    assert abs(rho - (hi + lo)) <= 2 * n * H.EPS * np.abs(xs * ys_ref).sum()
    po.daxpyv(0.75, xs, ys_ref)
    blas.daxpy(n, 0.75, x, incx, y, incy)
    assert np.array_equal(y[iy], ys_ref)  # axpy is elementwise with the same fma: bit exact


@pytest.mark.parametrize("trans", ["N", "T"])
def test_dgemv_dmmch_dblat2_grid(gblib, trans):
    p = json.load(open(os.path.join(GOLD, "blastest_params.json")))["dblat2"]
    gen = H.DBeg()
    worst = 0.0
    for m in p["n"]:
        for n in p["n"]:
            for incx in p["inc"]:
                for incy in p["inc"]:
                    for alpha in p["alpha"]:
                        for beta in p["beta"]:
                            a = H.dmake_ge(gen, m, n)
                            lx, ly = (m, n) if trans == "T" else (n, m)
                            x = np.array([gen() for _ in range(lx)])
                            y0 = np.array([gen() for _ in range(ly)])
                            xb = np.zeros(max(1, lx * abs(incx)))
                            yb = np.zeros(max(1, ly * abs(incy)))
                            # BLAS convention: negative inc traverses from the end
                            for i in range(lx):
                                xb[(i if incx > 0 else lx - 1 - i) * abs(incx)] = x[i]
                            for i in range(ly):
                                yb[(i if incy > 0 else ly - 1 - i) * abs(incy)] = y0[i]
                            ab = a if a.size else np.zeros((1, 1))
                            blas.dgemv(trans, m, n, alpha, ab, max(1, m), xb, incx, beta, yb, incy)
                            y = np.array([yb[(i if incy > 0 else ly - 1 - i) * abs(incy)] for i in range(ly)])
                            if ly and lx == 0:
                                assert np.array_equal(y, y0)  # netlib quirk: no update when x is empty
                                continue
                            if ly:
                                worst = max(worst, H.dmmch_ratio(alpha, H.op(a, 8 if trans == "T" else 0),
                                                                 x.reshape(-1, 1), beta, y0.reshape(-1, 1),
                                                                 y.reshape(-1, 1)))
    assert worst < p["thresh"]


@pytest.mark.parametrize("trans", [blas.NO_TRANSPOSE, blas.TRANSPOSE])
@pytest.mark.parametrize("order", ["F", "C"])
def test_bli_dgemv_large_vs_oracle(gblib, trans, order):
    m, n = 4099, 3001
    a = po.uniform((m, n), 1, order=order)
    lx, ly = (m, n) if trans else (n, m)
    x = po.uniform(lx, 2).ravel()
    y = po.uniform(ly, 3).ravel()
    ref = y.copy()
    po.dgemv(trans, 1.5, a, x, -0.5, ref)
    blas.bli_dgemv(trans, 1.5, a, x, -0.5, y)
    g = 1.5 * (np.abs(H.op(a, trans)) @ np.abs(x)) + 0.5 * np.abs(ref)
    assert np.all(np.abs(y - ref) <= 2 * lx * H.EPS * g)


def test_dgemv_beta_zero_ignores_nan(gblib):
    m, n = 300, 200
    a = po.uniform((m, n), 1)
    x = po.uniform(n, 2).ravel()
    y = np.full(m, np.nan)
    blas.dgemv("N", m, n, 1.0, a, m, x, 1, 0.0, y, 1)
    assert np.isfinite(y).all()


def test_dgemm_redirects_to_gemv_for_vectors(gblib):
    m, k = 513, 77
    a = po.uniform((m, k), 1)
    b = po.uniform((k, 1), 2)
    c = po.uniform((m, 1), 3)
    ref = np.asfortranarray(c.copy())
    po.dgemm(0, 0, 1.0, a, b, 1.0, ref)
    launches = blas.launch_count()
    blas.dgemm("N", "N", m, 1, k, 1.0, a, m, b, k, 1.0, c, m)
    assert blas.launch_count() > launches
    assert np.allclose(c, ref, rtol=1e-13, atol=1e-13)
