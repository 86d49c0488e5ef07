"""Native FP64 / FP32 GEMM on the GPU against the CPU oracle, through the
C ABI (BLAS, typed BLIS API and the device-pointer addon)."""
import json
import os

import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu

N, T = blas.NO_TRANSPOSE, blas.TRANSPOSE


@pytest.fixture(autouse=True)
def native(gblib):
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    yield


def storage(x, kind):
    """Copy x into row ('r'), column ('c') or general-stride ('g') storage."""
    if kind == "c":
        return np.array(x, order="F", copy=True)
    if kind == "r":
        return np.array(x, order="C", copy=True)
    big = np.full((2 * x.shape[0] + 1, 3 * x.shape[1] + 1), np.nan, order="F")
    v = big[1::2, 1::3][: x.shape[0], : x.shape[1]]
    v[...] = x
    return v


@pytest.mark.parametrize("m,n,k", [(100, 100, 100), (300, 200, 250), (129, 65, 33), (2, 7, 5), (500, 300, 400)])
@pytest.mark.parametrize("ta", [N, T])
@pytest.mark.parametrize("tb", [N, T])
@pytest.mark.parametrize("st", ["c", "r", "g"])
def test_bli_dgemm_testsuite_residual(m, n, k, ta, tb, st):
    a = H.normalize(po.uniform((k, m) if ta else (m, k), 1))
    b = H.normalize(po.uniform((n, k) if tb else (k, n), 2))
    c0 = H.normalize(po.uniform((m, n), 3))
    A, B, Cm = storage(a, st), storage(b, st), storage(c0, st)
    blas.bli_dgemm(ta, tb, 2.0, A, B, 1.2, Cm)
    assert H.gemm_residual(2.0, H.op(a, ta), H.op(b, tb), 1.2, c0, np.array(Cm)) < 1e-14
    if st == "g":
        # elements between the strided entries are untouched
        base = Cm.base if Cm.base is not None else Cm
        mask = np.ones(base.shape, bool)
        mask[1::2, 1::3][: m, : n] = False
        assert np.isnan(base[mask]).all()


@pytest.mark.parametrize("ta", ["N", "T"])
@pytest.mark.parametrize("tb", ["N", "T"])
@pytest.mark.parametrize("beta", [0.0, 1.0])
def test_dgemm_narrow_pow2_bit_exact(ta, tb, beta):
    m, n, k = 333, 257, 700
    a = po.narrow_pow2((k, m) if ta == "T" else (m, k), 5)
    b = po.narrow_pow2((n, k) if tb == "T" else (k, n), 6)
    c = po.narrow_pow2((m, n), 7)
    ref = np.asfortranarray(c.copy())
    po.dgemm(T if ta == "T" else N, T if tb == "T" else N, 1.0, a, b, beta, ref)
    blas.dgemm(ta, tb, m, n, k, 1.0, a, a.shape[0], b, b.shape[0], beta, c, m)
    assert np.array_equal(c, ref)


def test_dgemm_dmmch_grid_through_dgemm_():
    p = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "blastest_params.json")))["dblat3"]
    gen = H.DBeg()
    worst = 0.0
    for m in p["n"]:
        for n in p["n"]:
            for k in p["n"]:
                for ta in "NT":
                    for tb in "NT":
                        for alpha in p["alpha"]:
                            for beta in p["beta"]:
                                a = H.dmake_ge(gen, *((k, m) if ta == "T" else (m, k)))
                                b = H.dmake_ge(gen, *((n, k) if tb == "T" else (k, n)))
                                c0 = H.dmake_ge(gen, m, n)
                                c = np.asfortranarray(c0.copy()) if c0.size else np.zeros(1)
                                lda = max(1, a.shape[0])
                                ldb = max(1, b.shape[0])
                                blas.dgemm(ta, tb, m, n, k, alpha, a if a.size else np.zeros(1), lda,
                                           b if b.size else np.zeros(1), ldb, beta, c, max(1, m))
                                if c0.size:
                                    worst = max(worst, H.dmmch_ratio(alpha, H.op(a, 8 if ta == "T" else 0),
                                                                     H.op(b, 8 if tb == "T" else 0), beta, c0,
                                                                     c.reshape(m, n, order="F")))
    assert worst < p["thresh"]


def test_dgemm_special_scalars():
    m, n, k = 70, 50, 40
    a = po.uniform((m, k), 1)
    b = po.uniform((k, n), 2)
    c = np.full((m, n), np.nan, order="F")
    blas.dgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)  # beta == 0 ignores NaN in C
    ref = np.zeros((m, n), order="F")
    po.dgemm(0, 0, 1.0, a, b, 0.0, ref)
    assert np.isfinite(c).all() and np.allclose(c, ref, rtol=1e-13, atol=1e-13)
    a[3, 4] = np.nan
    c2 = po.uniform((m, n), 3)
    c2_ref = 0.5 * c2
    blas.dgemm("N", "N", m, n, k, 0.0, a, m, b, k, 0.5, c2, m)  # alpha == 0: C := beta*C, A unread
    assert np.array_equal(c2, c2_ref)
    c3 = po.uniform((m, n), 4)
    c3_ref = 2.0 * c3
    blas.dgemm("N", "N", m, n, 0, 1.0, a, m, b, 1, 2.0, c3, m)  # k == 0
    assert np.array_equal(c3, c3_ref)


def test_dgemm_leading_dimension_padding():
    m, n, k, lda, ldb, ldc = 65, 33, 47, 80, 60, 70
    abuf = po.uniform((lda, k), 1)
    bbuf = po.uniform((ldb, n), 2)
    cbuf = po.uniform((ldc, n), 3)
    c_ref = np.asfortranarray(cbuf.copy())
    po.dgemm(0, 0, 1.5, abuf[:m], bbuf[:k], 0.25, c_ref[:m])
    blas.dgemm("N", "N", m, n, k, 1.5, abuf, lda, bbuf, ldb, 0.25, cbuf, ldc)
    assert np.allclose(cbuf[:m], c_ref[:m], rtol=1e-13, atol=1e-13)
    assert np.array_equal(cbuf[m:], c_ref[m:])  # padding rows untouched


def test_dgemm_device_config1_vs_dd():
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    n = 1024
    a = po.uniform((n, n), 101)
    b = po.uniform((n, n), 102)
    c0 = po.uniform((n, n), 103)
    ta = torch.from_numpy(a.T.copy()).cuda().t()  # column-major on the device
    tb = torch.from_numpy(b.T.copy()).cuda().t()
    tc = torch.from_numpy(c0.T.copy()).cuda().t()
    dev.dgemm(N, N, 1.0, ta, tb, 0.5, tc)
    torch.cuda.synchronize()
    c = tc.cpu().numpy()
    rng = np.random.default_rng(0)
    ii = rng.integers(0, n, 4096)
    jj = rng.integers(0, n, 4096)
    hi, lo = po.dd_gemm_entries(0, 0, 1.0, a, b, 0.5, c0, ii, jj)
    g = (np.abs(a) @ np.abs(b) + 0.5 * np.abs(c0))[ii, jj]
    assert np.all(np.abs(c[ii, jj] - hi - lo) <= 2 * n * H.EPS * g)


# (256, 384, 128): whole 128 x 128 tiles and 16-deep k blocks, the aligned fast path
@pytest.mark.parametrize("m,n,k", [(100, 100, 100), (257, 129, 300), (256, 384, 128)])
@pytest.mark.parametrize("ta", [N, T])
@pytest.mark.parametrize("tb", [N, T])
def test_sgemm_testsuite_residual(m, n, k, ta, tb):
    f = np.float32
    a = H.normalize(po.uniform((k, m) if ta else (m, k), 1, dtype=f)).astype(f, order="F")
    b = H.normalize(po.uniform((n, k) if tb else (k, n), 2, dtype=f)).astype(f, order="F")
    c0 = H.normalize(po.uniform((m, n), 3, dtype=f)).astype(f, order="F")
    c = np.asfortranarray(c0.copy())
    blas.sgemm("T" if ta else "N", "T" if tb else "N", m, n, k, 2.0, a, a.shape[0], b, b.shape[0], 1.2, c, m)
    r = H.gemm_residual(2.0, H.op(a, ta).astype(np.float64), H.op(b, tb).astype(np.float64), 1.2,
                        c0.astype(np.float64), c.astype(np.float64))
    assert r < 1e-5


@pytest.mark.parametrize("m,n,k", [(200, 150, 300), (256, 128, 64)])
def test_sgemm_narrow_pow2_bit_exact(m, n, k):
    a = po.narrow_pow2((m, k), 8).astype(np.float32, order="F")
    b = po.narrow_pow2((k, n), 9).astype(np.float32, order="F")
    c = np.zeros((m, n), np.float32, order="F")
    blas.bli_sgemm(N, N, 1.0, a, b, 0.0, c)
    assert np.array_equal(c, (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32))


def test_cblas_row_major_dgemm(gblib):
    import ctypes as C
    m, n, k = 40, 30, 20
    a = po.uniform((m, k), 1, order="C")
    b = po.uniform((k, n), 2, order="C")
    c = np.zeros((m, n))
    gblib.cblas_dgemm(101, 111, 111, m, n, k, 1.0, a.ctypes.data_as(C.c_void_p), k,
                      b.ctypes.data_as(C.c_void_p), n, 0.0, c.ctypes.data_as(C.c_void_p), n)
    assert np.allclose(c, a @ b, rtol=1e-13, atol=1e-13)
