"""Ozaki split-product DGEMM (tcgen05 slice products) against the CPU model.

The model in oracle/gb_oracle.c performs the same digit split, exact integer
level sums and FP64 recombination, so the GPU result must match it bit for
bit; the double-double oracle then bounds the error against native FP64.
"""
import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu

N, T = blas.NO_TRANSPOSE, blas.TRANSPOSE


@pytest.fixture(autouse=True, params=[2, 1], ids=["cta_pair", "one_cta"])
def engine(gblib, request):
    """Every test runs on both slice-GEMM engines (CTA pairs and single CTAs)."""
    assert gblib.gb_set_ozaki_ctas(request.param) == 0
    yield request.param
    gblib.gb_set_ozaki_ctas(0)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def _run_gpu(ta, tb, alpha, a, b, beta, c, slices):
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, slices)
    blas.bli_dgemm(ta, tb, alpha, a, b, beta, c)


@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 200, 1000), (17, 33, 5), (129, 257, 1100)])
@pytest.mark.parametrize("slices", [3, 8])
def test_ozaki_bit_exact_vs_model(m, n, k, slices):
    a = po.expspread((m, k), 1)
    b = po.expspread((k, n), 2)
    c0 = po.uniform((m, n), 3)
    ref = np.asfortranarray(c0.copy())
    po.ozaki_dgemm(N, N, 1.25, a, b, 0.5, ref, slices)
    c = np.asfortranarray(c0.copy())
    _run_gpu(N, N, 1.25, a, b, 0.5, c, slices)
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("ta", [N, T])
@pytest.mark.parametrize("tb", [N, T])
@pytest.mark.parametrize("rowmajor", [False, True])
def test_ozaki_transposes_and_layouts(ta, tb, rowmajor):
    m, n, k = 150, 90, 333
    order = "C" if rowmajor else "F"
    a = po.uniform((k, m) if ta else (m, k), 4, order=order)
    b = po.uniform((n, k) if tb else (k, n), 5, order=order)
    c0 = po.uniform((m, n), 6, order=order)
    ref = c0.copy(order=order)
    po.ozaki_dgemm(ta, tb, -0.75, a, b, 0.0, ref, 6)
    c = c0.copy(order=order)
    _run_gpu(ta, tb, -0.75, a, b, 0.0, c, 6)
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("slices,k", [(12, 12000), (8, 16384)])
def test_ozaki_k_partitions_bit_exact(slices, k):
    # the level with the most slice pairs needs more than one int32 k part
    assert po.ozaki_kpart_limit(slices) < k
    m, n = 64, 96
    a = po.expspread((m, k), 7)
    b = po.expspread((k, n), 8)
    ref = np.zeros((m, n), order="F")
    po.ozaki_dgemm(N, N, 1.0, a, b, 0.0, ref, slices)
    c = np.zeros((m, n), order="F")
    _run_gpu(N, N, 1.0, a, b, 0.0, c, slices)
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("ta,tb,order", [(N, N, "F"), (T, T, "F"), (N, T, "C"), (T, N, "C")])
def test_ozaki_long_k_split_layouts(ta, tb, order):
    # k above 4096 takes the row-maximum kernel and the tiled split instead of the fused split
    m, n, k = 70, 90, 5000
    a = po.expspread((k, m) if ta else (m, k), 9, order=order)
    b = po.expspread((n, k) if tb else (k, n), 10, order=order)
    c0 = po.uniform((m, n), 11, order=order)
    ref = c0.copy(order=order)
    po.ozaki_dgemm(ta, tb, 0.75, a, b, -1.0, ref, 7)
    c = c0.copy(order=order)
    _run_gpu(ta, tb, 0.75, a, b, -1.0, c, 7)
    assert np.array_equal(c, ref)


def test_ozaki_device_random_inputs_match_host_generator():
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    x = dev.colmajor(300, 70)
    dev.randm(x, dev.RAND_EXPSPREAD, 99, -20, 20)
    y = dev.colmajor(300, 70)
    dev.randm(y, dev.RAND_UNIFORM, 98, -1.0, 1.0)
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), po.expspread((300, 70), 99, -20, 20))
    assert np.array_equal(y.cpu().numpy(), po.uniform((300, 70), 98))


def test_ozaki_device_dd_evaluator_matches_cpu():
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    m, n, k = 200, 150, 3000
    a = po.expspread((m, k), 3)
    b = po.expspread((k, n), 4)
    c = po.uniform((m, n), 5)
    ii = np.arange(0, m * n, 97) % m
    jj = (np.arange(0, m * n, 97) // m) % n
    hi, lo = po.dd_gemm_entries(0, 0, 1.5, a, b, -0.5, c, ii, jj)
    ta = torch.from_numpy(a.T.copy()).cuda().t()
    tb = torch.from_numpy(b.T.copy()).cuda().t()
    tc = torch.from_numpy(c.T.copy()).cuda().t()
    dh, dl = dev.dd_gemm_entries(0, 0, 1.5, ta, tb, -0.5, tc, torch.from_numpy(ii).cuda(),
                                 torch.from_numpy(jj).cuda())
    g = 1.5 * (np.abs(a) @ np.abs(b))[ii, jj] + 0.5 * np.abs(c[ii, jj])
    # different summation orders: both are double-double accurate (~2^-100 of the gauge)
    assert np.all(np.abs((dh.cpu().numpy() - hi) + (dl.cpu().numpy() - lo)) <= 2.0 ** -96 * g)


def test_ozaki_error_not_worse_than_native():
    n = 1024
    a = po.expspread((n, n), 11)
    b = po.expspread((n, n), 12)
    c_oz = np.zeros((n, n), order="F")
    c_nat = np.zeros((n, n), order="F")
    _run_gpu(N, N, 1.0, a, b, 0.0, c_oz, 8)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    blas.bli_dgemm(N, N, 1.0, a, b, 0.0, c_nat)
    rng = np.random.default_rng(1)
    ii = rng.integers(0, n, 4096)
    jj = rng.integers(0, n, 4096)
    hi, lo = po.dd_gemm_entries(0, 0, 1.0, a, b, 0.0, c_oz, ii, jj)
    e_oz = po.componentwise_error(c_oz[ii, jj], hi, lo)
    e_nat = po.componentwise_error(c_nat[ii, jj], hi, lo)
    assert e_oz <= e_nat


def test_ozaki_nonfinite_falls_back_to_ieee():
    m, n, k = 40, 30, 20
    a = po.uniform((m, k), 1)
    b = po.uniform((k, n), 2)
    a[5, 3] = np.inf
    b[7, 9] = np.nan
    c = np.zeros((m, n), order="F")
    _run_gpu(N, N, 1.0, a, b, 0.0, c, 8)
    ref = np.zeros((m, n), order="F")
    po.dgemm(0, 0, 1.0, a, b, 0.0, ref)
    assert np.array_equal(np.isnan(c), np.isnan(ref))
    fin = np.isfinite(ref)
    assert np.allclose(c[fin], ref[fin], rtol=1e-13, atol=1e-13)


def test_ozaki_through_dgemm_blas_and_scalars():
    m, n, k = 96, 80, 640
    a = po.uniform((m, k), 21)
    b = po.uniform((k, n), 22)
    c = po.uniform((m, n), 23)
    ref = np.asfortranarray(c.copy())
    po.ozaki_dgemm(N, N, 2.0, a, b, 1.2, ref, 7)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    blas.dgemm("N", "N", m, n, k, 2.0, a, m, b, k, 1.2, c, m)
    assert np.array_equal(c, ref)
    # alpha == 0 and k == 0 keep the level-3 early exits
    c2 = po.uniform((m, n), 24)
    r2 = 3.0 * c2
    blas.dgemm("N", "N", m, n, k, 0.0, a, m, b, k, 3.0, c2, m)
    assert np.array_equal(c2, r2)


def test_ozaki_device_api_matches_model():
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    m, n, k = 512, 384, 2048
    a = po.expspread((m, k), 31)
    b = po.expspread((k, n), 32)
    ref = np.zeros((m, n), order="F")
    po.ozaki_dgemm(N, N, 1.0, a, b, 0.0, ref, 8)
    ta = torch.from_numpy(a.T.copy()).cuda().t()
    tb = torch.from_numpy(b.T.copy()).cuda().t()
    tc = torch.zeros((n, m), dtype=torch.float64, device="cuda").t()
    dev.dgemm_ozaki(N, N, 1.0, ta, tb, 0.0, tc, 8)
    torch.cuda.synchronize()
    assert np.array_equal(tc.cpu().numpy(), ref)


@pytest.mark.parametrize("ta,beta,pad,m", [(0, 0.0, 0, 2048), (1, 1.5, 3, 2048), (0, 0.5, 1, 2100)])
def test_ozaki_pipelined_host_path_bit_identical(ta, beta, pad, m):
    """dgemm_ on host buffers large enough for the pipelined path (op(A) in row
    blocks, op(B) and C in column blocks on copy streams, one slice GEMM per
    block of C) gives the bits of one device call on the same operands; m =
    2100 leaves a last row block of part of a tile."""
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    n, k = 2304, 2048
    a0 = po.expspread((k, m) if ta else (m, k), 41, -12, 12)
    b0 = po.expspread((k, n), 42, -12, 12)
    c0 = po.uniform((m, n), 43)
    lda, ldb, ldc = a0.shape[0] + pad, k + pad, m + pad
    a = np.zeros((lda, a0.shape[1]), order="F")
    a[: a0.shape[0]] = a0
    b = np.zeros((ldb, n), order="F")
    b[:k] = b0
    c = np.zeros((ldc, n), order="F")
    c[:m] = c0
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    try:
        blas.dgemm("T" if ta else "N", "N", m, n, k, -0.5, a, lda, b, ldb, beta, c, ldc)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    ad = torch.from_numpy(np.ascontiguousarray(a0.T)).cuda().t()
    bd = torch.from_numpy(np.ascontiguousarray(b0.T)).cuda().t()
    cd = torch.from_numpy(np.ascontiguousarray(c0.T)).cuda().t()
    dev.dgemm_ozaki(8 if ta else 0, 0, -0.5, ad, bd, beta, cd, 7)
    torch.cuda.synchronize()
    assert np.array_equal(c[:m], cd.cpu().numpy())
    assert np.all(c[m:] == 0.0)  # padding rows of C untouched


def test_ozaki_pipelined_host_path_row_major_a():
    """A row-major op(A) (no row-block copies) takes the column-block pipeline
    with op(A) staged whole: the same bits as one device call."""
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    m, n, k = 1024, 2304, 4096
    a = po.expspread((m, k), 51, -12, 12, order="C")
    b = po.expspread((k, n), 52, -12, 12)
    c0 = po.uniform((m, n), 53)
    c = np.asfortranarray(c0.copy())
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    try:
        blas.bli_dgemm(N, N, 0.75, a, b, 0.25, c)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    ad = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    bd = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    cd = torch.from_numpy(np.ascontiguousarray(c0.T)).cuda().t()
    dev.dgemm_ozaki(0, 0, 0.75, ad, bd, 0.25, cd, 7)
    torch.cuda.synchronize()
    assert np.array_equal(c, cd.cpu().numpy())
