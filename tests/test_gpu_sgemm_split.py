"""SGEMM's split form on the bf16 tensor cores (gb_sgemm_split.cu) against the FP64 product.

The form splits op(A), op(B) straight from FP32 (each element widened exactly to FP64 as it
loads), forms their product as the Ozaki digit form with three slices (exact integer
accumulation) and rounds alpha P + beta C to FP32 once in the recombination.  With beta = 0
the model is exact: the oracle's digit-form product, times alpha in FP64, rounded to FP32.
Otherwise the result is checked against an FP64 product within the form's bound:
2^-(8s+1) (2^e_i |B_j|_1 + |A_i|_1 2^e_j) + 2^-(16s+2) k 2^(e_i+e_j) for the product (the
digits' representation error, no accumulation error) plus one FP32 rounding.
"""
import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
S = 3
U32 = float(np.finfo(np.float32).eps) / 2


@pytest.fixture(autouse=True)
def split_mode(gblib):
    blas.set_sgemm_mode(blas.SGEMM_SPLIT)
    yield
    blas.set_sgemm_mode(blas.SGEMM_AUTO)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k,spread", [(300, 200, 1000, False), (33, 517, 64, False), (1024, 1024, 2048, False),
                                          (200, 300, 5000, False), (260, 150, 700, True), (130, 270, 5000, True)])
def test_split_sgemm_bit_exact_beta0(ta, tb, m, n, k, spread):
    # k = 5000 takes the row-maximum kernel and the tiled split (k past the fused split's 4096);
    # spread: entries (1 + u) 2^e, e in [-30, 30], so rows lose their small entries' low bits
    if spread:
        a = po.expspread((k, m) if ta == "T" else (m, k), 1, -30, 30).astype(np.float32)
        b = po.expspread((n, k) if tb == "T" else (k, n), 2, -30, 30).astype(np.float32)
    else:
        a = po.uniform((k, m) if ta == "T" else (m, k), 1, dtype=np.float32)
        b = po.uniform((n, k) if tb == "T" else (k, n), 2, dtype=np.float32)
    c = np.zeros((m, n), dtype=np.float32, order="F")
    blas.sgemm(ta, tb, m, n, k, 0.75, a, a.shape[0], b, b.shape[0], 0.0, c, m)
    p = np.zeros((m, n), order="F")
    po.ozaki_dgemm(8 if ta == "T" else 0, 8 if tb == "T" else 0, 1.0, np.asfortranarray(a, dtype=np.float64),
                   np.asfortranarray(b, dtype=np.float64), 0.0, p, S)
    ref = (np.float64(0.75) * p).astype(np.float32)
    assert np.array_equal(c, ref)


def test_split_sgemm_alpha_beta_within_bound():
    m, n, k = 700, 650, 1500
    a = po.uniform((m, k), 3, dtype=np.float32)
    b = po.uniform((k, n), 4, dtype=np.float32)
    c0 = po.uniform((m, n), 5, dtype=np.float32)
    c = np.asfortranarray(c0.copy())
    blas.sgemm("N", "N", m, n, k, -1.5, a, m, b, k, 0.5, c, m)
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    exact = -1.5 * (a64 @ b64) + 0.5 * c0.astype(np.float64)
    ea = 2.0 ** (np.floor(np.log2(np.abs(a64).max(axis=1))) + 2)
    eb = 2.0 ** (np.floor(np.log2(np.abs(b64).max(axis=0))) + 2)
    pbound = 2.0 ** -(8 * S + 1) * (np.outer(ea, np.abs(b64).sum(0)) + np.outer(np.abs(a64).sum(1), eb)) \
        + 2.0 ** -(16 * S + 2) * k * np.outer(ea, eb)
    bound = 1.5 * pbound * (1 + 1e-12) + U32 * np.abs(exact) * (1 + 1e-6) + 1e-300
    assert np.all(np.abs(c.astype(np.float64) - exact) <= bound)


def test_split_sgemm_more_accurate_than_fma_at_large_k():
    """The measurement behind the default: at k = 8192 the split form's error against an FP64
    product is below the FP32 FMA kernel's."""
    m, n, k = 1024, 1024, 8192
    a = po.uniform((m, k), 6, dtype=np.float32)
    b = po.uniform((k, n), 7, dtype=np.float32)
    exact = a.astype(np.float64) @ b.astype(np.float64)
    c_split = np.zeros((m, n), dtype=np.float32, order="F")
    blas.sgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c_split, m)
    blas.set_sgemm_mode(blas.SGEMM_FMA)
    c_fma = np.zeros((m, n), dtype=np.float32, order="F")
    blas.sgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c_fma, m)
    e_split = np.abs(c_split - exact).max()
    e_fma = np.abs(c_fma - exact).max()
    assert e_split < e_fma, (e_split, e_fma)


def test_split_sgemm_nonfinite_propagates():
    m, n, k = 1024, 1024, 600
    a = po.uniform((m, k), 8, dtype=np.float32)
    b = po.uniform((k, n), 9, dtype=np.float32)
    a[10, 20] = np.inf
    b[30, 40] = np.nan
    c = np.zeros((m, n), dtype=np.float32, order="F")
    blas.sgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    ref = a.astype(np.float64) @ b.astype(np.float64)
    assert np.array_equal(np.isnan(c), np.isnan(ref))
    assert np.array_equal(np.isinf(c), np.isinf(ref))


@pytest.mark.parametrize("ta,tb", [(0, 0), (8, 8)])
def test_split_sgemm_general_strides_bit_exact(gblib, ta, tb):
    """The splits read op(A) and op(B) in the caller's memory: element strides other than one
    on both dimensions (a general-stride A, B and C), against the model."""
    torch = pytest.importorskip("torch")
    from blis_gb300 import _lib
    m, n, k = 300, 170, 700
    a = po.uniform((k, m) if ta else (m, k), 21, dtype=np.float32)
    b = po.uniform((n, k) if tb else (k, n), 22, dtype=np.float32)
    c0 = po.uniform((m, n), 23, dtype=np.float32)

    def strided(x, rs, cs):
        # x(i, j) at buf[i*rs + j*cs] of a device buffer
        buf = torch.zeros((x.shape[0] - 1) * rs + (x.shape[1] - 1) * cs + 1, dtype=torch.float32)
        idx = (np.arange(x.shape[0])[:, None] * rs + np.arange(x.shape[1])[None, :] * cs).ravel()
        buf[torch.from_numpy(idx)] = torch.from_numpy(np.ascontiguousarray(x).ravel())
        return buf.cuda(), idx

    A, _ = strided(a, 3, 3 * a.shape[0] + 5)
    B, _ = strided(b, 2 * b.shape[1] + 1, 2)
    C, cidx = strided(c0, 2, 2 * m + 3)
    L = _lib.load()
    assert L.gb_sgemm_dev(ta, tb, m, n, k, 1.5, A.data_ptr(), 3, 3 * a.shape[0] + 5, B.data_ptr(),
                          2 * b.shape[1] + 1, 2, 0.0, C.data_ptr(), 2, 2 * m + 3, None) == 0
    assert L.gb_synchronize() == 0
    got = C.cpu().numpy()[cidx].reshape(m, n)
    p = np.zeros((m, n), order="F")
    po.ozaki_dgemm(ta, tb, 1.0, np.asfortranarray(a, dtype=np.float64), np.asfortranarray(b, dtype=np.float64),
                   0.0, p, S)
    assert np.array_equal(got, (np.float64(1.5) * p).astype(np.float32))


def test_split_sgemm_k_beyond_one_part_bit_exact():
    """k = 50000 exceeds one exact k part at 3 slices (43648): the levels are summed over two
    parts and the recombination still rounds once, bit-exact against the model."""
    m, n, k = 70, 90, 50000
    a = po.uniform((m, k), 31, dtype=np.float32)
    b = po.uniform((k, n), 32, dtype=np.float32)
    assert k > po.ozaki_kpart_limit(S)
    c = np.zeros((m, n), dtype=np.float32, order="F")
    blas.sgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    p = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, np.asfortranarray(a, dtype=np.float64), np.asfortranarray(b, dtype=np.float64), 0.0,
                   p, S)
    assert np.array_equal(c, p.astype(np.float32))


def test_split_sgemm_alpha_zero_and_k_zero():
    """alpha = 0 (A and B not read: NaN there changes nothing) and k = 0 scale C by beta."""
    m, n, k = 40, 30, 20
    a = np.full((m, k), np.nan, dtype=np.float32, order="F")
    b = np.full((k, n), np.nan, dtype=np.float32, order="F")
    c0 = po.uniform((m, n), 33, dtype=np.float32)
    c = np.asfortranarray(c0.copy())
    blas.sgemm("N", "N", m, n, k, 0.0, a, m, b, k, 0.5, c, m)
    assert np.array_equal(c, (np.float32(0.5) * c0).astype(np.float32))
    c = np.asfortranarray(c0.copy())
    blas.sgemm("N", "N", m, n, 0, 2.0, a, m, b, 1, -1.0, c, m)
    assert np.array_equal(c, -c0)


@pytest.mark.parametrize("grid", ["4x2", "3x3"])
def test_split_sgemm_blocked_bit_exact(grid, monkeypatch):
    """The blocked form (row blocks of op(A), column blocks of op(B), two compute streams),
    forced at a size the model finishes quickly, with ragged last blocks: the same bits."""
    monkeypatch.setenv("GB_OZAKI_DEV_BLOCKS", grid)
    m, n, k = 2600, 1100, 700
    a = po.expspread((m, k), 51, -12, 12).astype(np.float32)
    b = po.uniform((k, n), 52, dtype=np.float32)
    c0 = po.uniform((m, n), 53, dtype=np.float32)
    c = np.asfortranarray(c0.copy())
    blas.sgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    p = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, np.asfortranarray(a, dtype=np.float64), np.asfortranarray(b, dtype=np.float64), 0.0,
                   p, S)
    assert np.array_equal(c, p.astype(np.float32))


def test_split_sgemm_blocked_nonfinite_with_beta(monkeypatch):
    """Blocks whose rows of op(A) or columns of op(B) hold an Inf or NaN take the FP32 pipe, the
    others the split form, and beta enters once everywhere."""
    monkeypatch.setenv("GB_OZAKI_DEV_BLOCKS", "4x2")
    m, n, k = 2600, 1100, 300
    a = po.uniform((m, k), 54, dtype=np.float32)
    b = po.uniform((k, n), 55, dtype=np.float32)
    c0 = po.uniform((m, n), 56, dtype=np.float32)
    a[m - 3, 5] = np.inf
    b[7, n - 2] = np.nan
    c = np.asfortranarray(c0.copy())
    blas.sgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.5, c, m)
    ref = a.astype(np.float64) @ b.astype(np.float64) + 0.5 * c0.astype(np.float64)
    assert np.array_equal(np.isnan(c), np.isnan(ref)) and np.array_equal(np.isinf(c), np.isinf(ref))
    fin = np.isfinite(ref)
    af = np.where(np.isfinite(a), np.abs(a), 0).astype(np.float64)
    bf = np.where(np.isfinite(b), np.abs(b), 0).astype(np.float64)
    gauge = af @ bf + 0.5 * np.abs(c0.astype(np.float64))
    assert np.all(np.abs(c[fin].astype(np.float64) - ref[fin]) <= 2 * (k + 2) * U32 * gauge[fin])
