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
