"""The CRT form of the Ozaki products (residues modulo up to 16 pairwise coprime moduli on
the bf16 tensor cores, Chinese remainder reconstruction) against its CPU model.

The model (oracle/gb_oracle.c, orc_ozaki_crt_dgemm) scales the operands to the same t-bit
integers and forms their product exactly in 128-bit integers, with one rounding: the GPU,
which obtains the same integer product from the residue products by the Chinese remainder
theorem, must match it bit for bit.  The double-double oracle bounds its error against
native FP64.
"""
import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

N, T = blas.NO_TRANSPOSE, blas.TRANSPOSE


@pytest.fixture(autouse=True, params=[2, 1], ids=["cta_pair", "one_cta"])
def engine(gblib, request):
    assert gblib.gb_set_ozaki_ctas(request.param) == 0
    yield request.param
    gblib.gb_set_ozaki_ctas(0)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def _run_gpu(ta, tb, alpha, a, b, beta, c, moduli):
    blas.set_dgemm_mode(blas.DGEMM_OZAKI_CRT, moduli)
    try:
        blas.bli_dgemm(ta, tb, alpha, a, b, beta, c)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)


@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (300, 200, 1000), (17, 33, 5), (129, 257, 1100)])
@pytest.mark.parametrize("moduli", [6, 12, 16])
def test_crt_bit_exact_vs_model(m, n, k, moduli):
    a = po.expspread((m, k), 1)
    b = po.expspread((k, n), 2)
    c0 = po.uniform((m, n), 3)
    ref = np.asfortranarray(c0.copy())
    assert po.ozaki_crt_dgemm(N, N, 1.25, a, b, 0.5, ref, moduli) == 0
    c = np.asfortranarray(c0.copy())
    _run_gpu(N, N, 1.25, a, b, 0.5, c, moduli)
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("ta", [N, T])
@pytest.mark.parametrize("tb", [N, T])
@pytest.mark.parametrize("rowmajor", [False, True])
def test_crt_transposes_and_layouts(ta, tb, rowmajor):
    m, n, k = 150, 90, 333
    order = "C" if rowmajor else "F"
    a = po.uniform((k, m) if ta else (m, k), 4, order=order)
    b = po.uniform((n, k) if tb else (k, n), 5, order=order)
    c0 = po.uniform((m, n), 6, order=order)
    ref = c0.copy(order=order)
    po.ozaki_crt_dgemm(ta, tb, -0.75, a, b, 0.0, ref, 14)
    c = c0.copy(order=order)
    _run_gpu(ta, tb, -0.75, a, b, 0.0, c, 14)
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("k", [5000, 16384])
def test_crt_long_k_at_16_moduli(k):
    m, n = 70, 90
    a = po.expspread((m, k), 9)
    b = po.expspread((k, n), 10)
    c0 = po.uniform((m, n), 11)
    ref = np.asfortranarray(c0.copy())
    po.ozaki_crt_dgemm(N, N, 0.75, a, b, -1.0, ref, 16)
    c = np.asfortranarray(c0.copy())
    _run_gpu(N, N, 0.75, a, b, -1.0, c, 16)
    assert np.array_equal(c, ref)


def test_crt_error_not_worse_than_native_or_digits():
    """16 moduli at k = 1024 carry 57-bit operands: on exponent-spread inputs the error is at
    most the 7-slice digit form's (56-bit digits, and the dropped cross terms) and within a
    factor two of native FP64's, whose accumulation error is still small at this k (at
    k = 16384 native FP64's error grows past the CRT form's: the benchmark measures that)."""
    n = 1024
    a = po.expspread((n, n), 11)
    b = po.expspread((n, n), 12)
    c_crt = np.zeros((n, n), order="F")
    c_dig = np.zeros((n, n), order="F")
    c_nat = np.zeros((n, n), order="F")
    _run_gpu(N, N, 1.0, a, b, 0.0, c_crt, 16)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    blas.bli_dgemm(N, N, 1.0, a, b, 0.0, c_dig)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    blas.bli_dgemm(N, N, 1.0, a, b, 0.0, c_nat)
    rng = np.random.default_rng(1)
    ii = rng.integers(0, n, 4096)
    jj = rng.integers(0, n, 4096)
    hi, lo = po.dd_gemm_entries(0, 0, 1.0, a, b, 0.0, c_crt, ii, jj)
    e_crt = po.componentwise_error(c_crt[ii, jj], hi, lo)
    e_dig = po.componentwise_error(c_dig[ii, jj], hi, lo)
    e_nat = po.componentwise_error(c_nat[ii, jj], hi, lo)
    assert e_crt <= e_dig and e_crt <= 2 * e_nat, (e_crt, e_dig, e_nat)


def test_crt_nonfinite_falls_back_to_ieee():
    m, n, k = 40, 30, 20
    a = po.uniform((m, k), 1)
    b = po.uniform((k, n), 2)
    a[5, 3] = np.inf
    b[7, 9] = np.nan
    c = np.zeros((m, n), order="F")
    _run_gpu(N, N, 1.0, a, b, 0.0, c, 16)
    ref = np.zeros((m, n), order="F")
    po.dgemm(0, 0, 1.0, a, b, 0.0, ref)
    assert np.array_equal(np.isnan(c), np.isnan(ref))
    fin = np.isfinite(ref)
    assert np.allclose(c[fin], ref[fin], rtol=1e-13, atol=1e-13)


def test_crt_device_api_and_pipelined_host_path():
    """The device entry point and dgemm_ on host buffers large enough for the pipelined
    path (blocks of op(A), op(B) and C on copy streams) give the model's bits."""
    torch = pytest.importorskip("torch")
    from blis_gb300 import dev
    m, n, k = 2048, 2304, 2048
    a = po.expspread((m, k), 41, -12, 12)
    b = po.expspread((k, n), 42, -12, 12)
    c0 = po.uniform((m, n), 43)
    ref = np.asfortranarray(c0.copy())
    po.ozaki_crt_dgemm(N, N, -0.5, a, b, 1.5, ref, 16)
    ad = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()
    bd = torch.from_numpy(np.ascontiguousarray(b.T)).cuda().t()
    cd = torch.from_numpy(np.ascontiguousarray(c0.T)).cuda().t()
    dev.dgemm_ozaki_crt(N, N, -0.5, ad, bd, 1.5, cd, 16)
    torch.cuda.synchronize()
    assert np.array_equal(cd.cpu().numpy(), ref)
    c = np.asfortranarray(c0.copy())
    blas.set_dgemm_mode(blas.DGEMM_OZAKI_CRT, 16)
    try:
        blas.dgemm("N", "N", m, n, k, -0.5, a, m, b, k, 1.5, c, m)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    assert np.array_equal(c, ref)



@pytest.mark.parametrize("moduli", list(range(2, 17)))
def test_crt_every_moduli_count(moduli):
    # the model's bits at every moduli count (the int16 residue planes and the recombination's
    # weight tables), a partial tile of rows, op(B) transposed for odd counts
    m, n, k = 300, 70, 120
    a = po.expspread((m, k), 11)
    b = po.expspread((k, n), 12)
    tb = T if moduli % 2 else N
    bb = b.T.copy(order="F") if moduli % 2 else b
    c0 = po.uniform((m, n), 13)
    ref = np.asfortranarray(c0.copy())
    assert po.ozaki_crt_dgemm(N, tb, 0.5, a, bb, -1.0, ref, moduli) == 0
    c = np.asfortranarray(c0.copy())
    _run_gpu(N, tb, 0.5, a, bb, -1.0, c, moduli)
    assert np.array_equal(c, ref), moduli
