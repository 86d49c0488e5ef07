"""dtrmm, dsymm, dsyrk and dgemmt on the GPU (gb_level3x.cu) against the CPU
oracle's restatements: the native form within the gemm error bound (a
DMMCH-style componentwise ratio), the Ozaki form of symm, syrk and gemmt
bit for bit against the Ozaki model of the full product (the same digits,
exponents and rounding per entry), and the triangle gemmt/syrk must not
touch left exactly as it was."""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def native(gblib):
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    yield
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def _tri(a, uplo, diag):
    t = np.tril(a) if uplo == "L" else np.triu(a)
    if diag == "U":
        t = t - np.diag(np.diag(t)) + np.eye(a.shape[0])
    return t


def _sym(a, uplo):
    return np.tril(a) + np.tril(a, -1).T if uplo == "L" else np.triu(a) + np.triu(a, 1).T


def _mask(m, uplo):
    return np.tril(np.ones((m, m), bool)) if uplo == "L" else np.triu(np.ones((m, m), bool))


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
@pytest.mark.parametrize("m,n", [(300, 200), (65, 1), (1, 7), (257, 129)])
def test_dtrmm_all_cases(side, uplo, trans, diag, m, n):
    na = m if side == "L" else n
    a = po.uniform((na, na), 11)
    b0 = po.uniform((m, n), 12)
    b = np.asfortranarray(b0.copy())
    blas.dtrmm(side, uplo, trans, diag, m, n, -1.5, a, na, b, m)
    t = _tri(a, uplo, diag)
    t = t.T if trans == "T" else t
    if side == "L":
        r = H.dmmch_ratio(-1.5, t, b0, 0.0, np.zeros_like(b0), b)
    else:
        r = H.dmmch_ratio(-1.5, b0, t, 0.0, np.zeros_like(b0), b)
    assert r < 2 * (na + 2)
    ref = np.asfortranarray(b0.copy())
    po.dtrmm(po.LEFT if side == "L" else po.RIGHT, po.LOWER if uplo == "L" else po.UPPER,
             8 if trans == "T" else 0, po.UNIT_DIAG if diag == "U" else po.NONUNIT_DIAG, -1.5, a, ref)
    assert np.max(np.abs(b - ref)) <= 4 * (na + 2) * H.EPS * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "T")])
def test_dtrmm_ozaki_many_columns_and_alpha_zero(uplo, trans):
    # 700 rows: the recursion splits into 64-row diagonal blocks and Ozaki gemm updates
    m, n = 700, 3000
    a = po.uniform((m, m), 13)
    b0 = po.uniform((m, n), 14)
    ref = np.asfortranarray(b0.copy())
    po.dtrmm(po.LEFT, po.LOWER if uplo == "L" else po.UPPER, 8 if trans == "T" else 0, po.NONUNIT_DIAG, 2.0,
             a, ref)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    b = np.asfortranarray(b0.copy())
    blas.dtrmm("L", uplo, trans, "N", m, n, 2.0, a, m, b, m)
    t = _tri(a, uplo, "N")
    assert H.dmmch_ratio(2.0, t.T if trans == "T" else t, b0, 0.0, np.zeros_like(b0), b) < 2 * (m + 2)
    assert np.max(np.abs(b - ref)) <= 1e-13 * np.max(np.abs(ref))
    b[:] = np.nan  # alpha = 0: B := 0 without reading it (or A)
    blas.dtrmm("L", uplo, trans, "N", m, n, 0.0, a, m, b, m)
    assert (b == 0.0).all()


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("m,n", [(200, 330), (1, 5), (129, 1)])
def test_dsymm_native_reads_one_triangle(side, uplo, m, n):
    na = m if side == "L" else n
    a = po.uniform((na, na), 15)
    junk = np.asfortranarray(a.copy())
    junk[np.triu_indices(na, 1) if uplo == "L" else np.tril_indices(na, -1)] = np.nan
    b = po.uniform((m, n), 16)
    c0 = po.uniform((m, n), 17)
    c = np.asfortranarray(c0.copy())
    blas.dsymm(side, uplo, m, n, 0.5, junk, na, b, m, -1.0, c, m)
    s = _sym(a, uplo)
    a_op, b_op = (s, b) if side == "L" else (b, s)
    assert np.isfinite(c).all()
    assert H.dmmch_ratio(0.5, a_op, b_op, -1.0, c0, c) < 2 * (na + 2)


@pytest.mark.parametrize("side", ["L", "R"])
def test_dsymm_ozaki_bit_exact_vs_model(side):
    m, n = 300, 257
    na = m if side == "L" else n
    a = po.expspread((na, na), 18, -10, 10)
    b = po.expspread((m, n), 19, -10, 10)
    c0 = po.uniform((m, n), 20)
    s = np.asfortranarray(_sym(a, "U"))
    ref = np.asfortranarray(c0.copy())
    if side == "L":
        po.ozaki_dgemm(0, 0, 1.25, s, b, 0.5, ref, 7)
    else:
        po.ozaki_dgemm(0, 0, 1.25, b, s, 0.5, ref, 7)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    c = np.asfortranarray(c0.copy())
    blas.dsymm(side, "U", m, n, 1.25, a, na, b, m, 0.5, c, m)
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,k", [(300, 200), (1100, 37), (1, 9)])
def test_dsyrk_native_triangle_and_untouched(uplo, trans, n, k):
    a = po.uniform((n, k) if trans == "N" else (k, n), 21)
    c0 = po.uniform((n, n), 22)
    c = np.asfortranarray(c0.copy())
    blas.dsyrk(uplo, trans, n, k, 0.75, a, a.shape[0], 1.5, c, n)
    a_op = a if trans == "N" else a.T
    msk = _mask(n, uplo)
    assert np.array_equal(c[~msk], c0[~msk])
    full = np.where(msk, c, 0.75 * (a_op @ a_op.T) + 1.5 * c0)  # the untouched part compares exactly
    assert H.dmmch_ratio(0.75, a_op, a_op.T, 1.5, c0, full) < 2 * (k + 2)
    ref = np.asfortranarray(c0.copy())
    po.dgemmt(po.LOWER if uplo == "L" else po.UPPER, 0 if trans == "N" else 8, 8 if trans == "N" else 0, 0.75,
              a, a, 1.5, ref)
    assert np.max(np.abs(c - ref)) <= 4 * (k + 2) * H.EPS * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T")])
def test_dgemmt_ozaki_bit_exact_vs_model(uplo, ta, tb):
    # 1300 rows: two 1024-column blocks, the second one short; slice GEMM row blocks at 1024
    m, k = 1300, 40
    a = po.expspread((k, m) if ta == "T" else (m, k), 23, -8, 8)
    b = po.expspread((m, k) if tb == "T" else (k, m), 24, -8, 8)
    c0 = po.uniform((m, m), 25)
    ref = np.asfortranarray(c0.copy())
    po.ozaki_dgemm(8 if ta == "T" else 0, 8 if tb == "T" else 0, -0.5, a, b, 2.0, ref, 5)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 5)
    c = np.asfortranarray(c0.copy())
    blas.dgemmt(uplo, ta, tb, m, k, -0.5, a, a.shape[0], b, b.shape[0], 2.0, c, m)
    msk = _mask(m, uplo)
    assert np.array_equal(c[msk], ref[msk])
    assert np.array_equal(c[~msk], c0[~msk])


def test_dsyrk_ozaki_beta_zero_ignores_nan_and_alpha_zero():
    n, k = 1100, 64
    a = po.expspread((n, k), 26, -6, 6)
    ref = np.zeros((n, n), order="F")
    po.ozaki_dgemm(0, 8, 1.0, a, a, 0.0, ref, 6)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 6)
    c = np.full((n, n), np.nan, order="F")
    blas.dsyrk("L", "N", n, k, 1.0, a, n, 0.0, c, n)
    msk = _mask(n, "L")
    assert np.array_equal(c[msk], ref[msk])
    assert np.isnan(c[~msk]).all()
    c0 = po.uniform((n, n), 27)
    c = np.asfortranarray(c0.copy())
    blas.dsyrk("U", "T", n, k, 0.0, a, k, 3.0, c, n)  # alpha = 0: the triangle is scaled by beta
    msk = _mask(n, "U")
    assert np.array_equal(c[msk], 3.0 * c0[msk])
    assert np.array_equal(c[~msk], c0[~msk])


def test_typed_api_general_strides():
    # bli_ entry points with row-major operands (rs = n, cs = 1)
    m, n, k = 150, 90, 60
    a = po.uniform((m, m), 28, order="C")
    b0 = po.uniform((m, n), 29, order="C")
    b = b0.copy(order="C")
    blas.bli_dtrmm(blas.LEFT, blas.UPPER, blas.NO_TRANSPOSE, blas.NONUNIT_DIAG, 1.0, a, b)
    assert H.dmmch_ratio(1.0, np.triu(a), b0, 0.0, np.zeros_like(b0), b) < 2 * (m + 2)
    c0 = po.uniform((m, n), 30, order="C")
    c = c0.copy(order="C")
    blas.bli_dsymm(blas.LEFT, blas.LOWER, 2.0, a, b0, 1.0, c)
    assert H.dmmch_ratio(2.0, _sym(a, "L"), b0, 1.0, c0, c) < 2 * (m + 2)
    x = po.uniform((k, m), 31, order="C")
    s0 = po.uniform((m, m), 32, order="C")
    s = s0.copy(order="C")
    blas.bli_dsyrk(blas.UPPER, blas.TRANSPOSE, 1.0, x, 0.0, s)
    msk = _mask(m, "U")
    assert np.array_equal(s[~msk], s0[~msk])
    full = np.where(msk, s, x.T @ x)
    assert H.dmmch_ratio(1.0, x.T, x, 0.0, np.zeros_like(s0), full) < 2 * (k + 2)
    y = po.uniform((m, k), 33, order="C")
    g = s0.copy(order="C")
    blas.bli_dgemmt(blas.LOWER, blas.NO_TRANSPOSE, blas.TRANSPOSE, -1.0, y, x.T.copy(order="C"), 0.5, g)
    msk = _mask(m, "L")
    assert np.array_equal(g[~msk], s0[~msk])
    full = np.where(msk, g, -(y @ x) + 0.5 * s0)
    assert H.dmmch_ratio(-1.0, y, x, 0.5, s0, full) < 2 * (k + 2)


def test_device_api_syrk_and_trmm(gblib):
    import torch
    n, k = 513, 77
    a = po.uniform((n, k), 34)
    ad = torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t()  # column-major on the device
    c0 = po.uniform((n, n), 35)
    cd = torch.from_numpy(np.ascontiguousarray(c0.T)).cuda().t()
    assert gblib.gb_dsyrk_dev(blas.LOWER, blas.NO_TRANSPOSE, n, k, 1.0, ad.data_ptr(), 1, n, -1.0,
                              cd.data_ptr(), 1, n, None) == 0
    assert gblib.gb_synchronize() == 0
    c = cd.cpu().numpy()
    msk = _mask(n, "L")
    assert np.array_equal(c[~msk], c0[~msk])
    full = np.where(msk, c, a @ a.T - c0)
    assert H.dmmch_ratio(1.0, a, a.T, -1.0, c0, full) < 2 * (k + 2)
    t = po.uniform((n, n), 36)
    td = torch.from_numpy(np.ascontiguousarray(t.T)).cuda().t()
    bd = torch.from_numpy(np.ascontiguousarray(c0.T)).cuda().t()
    assert gblib.gb_dtrmm_dev(blas.RIGHT, blas.LOWER, blas.TRANSPOSE, blas.UNIT_DIAG, n, n, 0.5, td.data_ptr(), 1,
                              n, bd.data_ptr(), 1, n, None) == 0
    assert gblib.gb_synchronize() == 0
    tri = _tri(t, "L", "U").T
    assert H.dmmch_ratio(0.5, c0, tri, 0.0, np.zeros_like(c0), bd.cpu().numpy()) < 2 * (n + 2)


@pytest.mark.parametrize("side,uplo,trans,diag", [("L", "L", "N", "N"), ("L", "U", "T", "U"),
                                                  ("R", "L", "N", "N"), ("R", "U", "N", "U")])
def test_dtrmm_ozaki_bit_identical_to_model(side, uplo, trans, diag):
    # the precision form is one Ozaki product on the triangle materialised with
    # zeros; the slice GEMM skips each tile row's all-zero k blocks, which add
    # nothing to the exact digit sums, so the result is the model's bit for bit
    m, n = 700, 530
    na = m if side == "L" else n
    a = po.expspread((na, na), 41, -12, 12)
    b0 = po.expspread((m, n), 42, -12, 12)
    t = _tri(a, uplo, diag)
    t = t.T if trans == "T" else t
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    b = np.asfortranarray(b0.copy())
    blas.dtrmm(side, uplo, trans, diag, m, n, -0.75, a, na, b, m)
    if side == "L":
        model = np.zeros((m, n), order="F")
        po.ozaki_dgemm(0, 0, -0.75, np.asfortranarray(t), b0, 0.0, model, 7)
    else:
        # B op(A) runs as op(A)^T B^T
        mt = np.zeros((n, m), order="F")
        po.ozaki_dgemm(0, 0, -0.75, np.asfortranarray(t.T), np.asfortranarray(b0.T), 0.0, mt, 7)
        model = mt.T
    assert np.array_equal(b, model)


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_dsyrk_ozaki_nonfinite_keeps_other_triangle(uplo):
    # the precision form writes C's triangle from one product; with an Inf in
    # A the gated IEEE fallback takes over, still on the triangle only
    m, k = 1300, 200
    a = po.uniform((m, k), 43)
    a[700, 50] = np.inf
    c0 = po.uniform((m, m), 44)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE, 8)
    nat = np.asfortranarray(c0.copy())
    blas.dsyrk(uplo, "N", m, k, 1.5, a, m, 0.5, nat, m)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    c = np.asfortranarray(c0.copy())
    blas.dsyrk(uplo, "N", m, k, 1.5, a, m, 0.5, c, m)
    t = np.tril(np.ones((m, m), bool)) if uplo == "L" else np.triu(np.ones((m, m), bool))
    assert np.array_equal(c[~t], c0[~t])
    assert np.array_equal(np.isfinite(c), np.isfinite(nat))
    f = np.isfinite(nat) & t
    oa = np.abs(np.where(np.isfinite(a), a, 0.0))
    bound = 8 * (k + 2) * H.EPS * (1.5 * (oa @ oa.T) + 0.5 * np.abs(c0))
    assert np.all(np.abs(c - nat)[f] <= bound[f])


@pytest.mark.parametrize("side,uplo,transa,diag,transb", [("L", "L", "N", "N", "N"), ("R", "U", "T", "U", "T"),
                                                          ("L", "U", "T", "N", "T"), ("R", "L", "N", "U", "N")])
@pytest.mark.parametrize("mode", ["native", "ozaki"])
def test_dtrmm3_vs_oracle(side, uplo, transa, diag, transb, mode):
    m, n = 700, 530
    na = m if side == "L" else n
    a = po.uniform((na, na), 47)
    b = po.uniform((n, m) if transb == "T" else (m, n), 48)
    c0 = po.uniform((m, n), 49)
    code = {"N": blas.NO_TRANSPOSE, "T": blas.TRANSPOSE}
    sd = blas.LEFT if side == "L" else blas.RIGHT
    ul = blas.LOWER if uplo == "L" else blas.UPPER
    dg = blas.UNIT_DIAG if diag == "U" else blas.NONUNIT_DIAG
    blas.set_dgemm_mode(blas.DGEMM_OZAKI if mode == "ozaki" else blas.DGEMM_NATIVE, 8)
    try:
        c = np.asfortranarray(c0.copy())
        b_before = b.copy()
        blas.bli_dtrmm3(sd, ul, code[transa], dg, code[transb], 1.5, a, b, -0.5, c)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE, 8)
    assert np.array_equal(b, b_before)  # B is not written
    ref = np.asfortranarray(c0.copy())
    po.dtrmm3(po.LEFT if side == "L" else po.RIGHT, po.LOWER if uplo == "L" else po.UPPER,
              po.TRANSPOSE if transa == "T" else po.NO_TRANSPOSE, po.UNIT_DIAG if diag == "U" else po.NONUNIT_DIAG,
              po.TRANSPOSE if transb == "T" else po.NO_TRANSPOSE, 1.5, a, b, -0.5, ref)
    t = np.abs(_tri(a, uplo, diag))
    t = t.T if transa == "T" else t
    ob = np.abs(b.T if transb == "T" else b)
    g = 1.5 * (t @ ob if side == "L" else ob @ t) + 0.5 * np.abs(c0)
    assert np.all(np.abs(c - ref) <= 4 * (na + 2) * H.EPS * g)
