"""Pins the CPU oracle before it is trusted as the parity checker (no GPU).

The oracle (oracle/gb_oracle.c) is checked against:
  * the reference's own DDOT/DAXPY known answers (dblat1 check2_ data);
  * exact answers on "narrow power of two" inputs (every product and partial
    sum is exact, so any correct implementation agrees bit for bit);
  * the DMMCH test ratio on DBEG matrices for the dblat3 N/ALPHA/BETA grid;
  * the testsuite residual and a double-double evaluation;
and the Ozaki split-product model against the double-double error oracle.
"""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from tests import helpers as H

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def _blas_ptr(vec, n, inc):
    """BLAS convention: element 0 of the traversal is at the base pointer
    (frame/include/bli_blas_macro_defs.h:50-75); return the index of element 0
    in BLIS convention for a negative increment."""
    return (n - 1) * (-inc) if inc < 0 else 0


def dblat1_cases():
    d = _load("dblat1_check2.json")
    for ki in range(4):
        incx, incy = d["incxs"][ki], d["incys"][ki]
        for kn in range(4):
            n = d["ns"][kn]
            yield d, ki, kn, n, incx, incy


def stest_ok(comp, true, size, sfac):
    sd = np.asarray(comp) - np.asarray(true)
    return np.all((np.abs(sfac * sd) + np.abs(size)) - np.abs(size) == 0)


@pytest.mark.parametrize("case", list(range(16)))
def test_oracle_ddot_golden(case):
    d, ki, kn, n, incx, incy = list(dblat1_cases())[case]
    x = np.array(d["dx1"])
    y = np.array(d["dy1"])
    # BLIS convention: start at the element-0 index with a signed stride
    x0 = _blas_ptr(x, n, incx)
    y0 = _blas_ptr(y, n, incy)
    rho = po.ddotv(x[x0:] if incx > 0 else x, y[y0:] if incy > 0 else y, n=0) if n == 0 else None
    if n > 0:
        xs = np.array([x[x0 + i * incx] for i in range(n)])
        ys = np.array([y[y0 + i * incy] for i in range(n)])
        rho = po.ddotv(xs, ys)
    true = d["dt7"][kn + 4 * ki]
    assert stest_ok([rho], [true], [d["ssize1"][kn]], d["sfac"])


@pytest.mark.parametrize("case", list(range(16)))
def test_oracle_daxpy_golden(case):
    d, ki, kn, n, incx, incy = list(dblat1_cases())[case]
    x = np.array(d["dx1"])
    y = np.array(d["dy1"])
    mx, my = abs(incx), abs(incy)
    leny = d["lens"][kn + 4 * (my - 1)]
    x0 = _blas_ptr(x, n, incx)
    y0 = _blas_ptr(y, n, incy)
    for i in range(n):
        y[y0 + i * incy] = np.float64(y[y0 + i * incy])  # in place below
    xs = np.array([x[x0 + i * incx] for i in range(n)]) if n else np.zeros(0)
    ys = np.array([y[y0 + i * incy] for i in range(n)]) if n else np.zeros(0)
    if n:
        po.daxpyv(d["sa"], xs, ys)
        for i in range(n):
            y[y0 + i * incy] = ys[i]
    true = [d["dt8"][j + 7 * (kn + 4 * ki)] for j in range(leny)]
    ksize = min(2, kn + 1)
    size = d["ssize2"][14 * (ksize - 1): 14 * (ksize - 1) + leny]
    assert stest_ok(y[:leny], true, size, d["sfac"])
    del mx


@pytest.mark.parametrize("ta", [po.NO_TRANSPOSE, po.TRANSPOSE])
@pytest.mark.parametrize("tb", [po.NO_TRANSPOSE, po.TRANSPOSE])
@pytest.mark.parametrize("beta", [0.0, 1.0])
def test_oracle_gemm_narrow_pow2_exact(ta, tb, beta):
    m, n, k = 37, 29, 300
    a = po.narrow_pow2((k, m) if ta else (m, k), 11)
    b = po.narrow_pow2((n, k) if tb else (k, n), 12)
    c = po.narrow_pow2((m, n), 13)
    exact = H.op(a, ta) @ H.op(b, tb) + beta * c  # all partial sums exact in FP64
    po.dgemm(ta, tb, 1.0, a, b, beta, c)
    assert np.array_equal(c, exact)


def test_oracle_gemm_beta0_ignores_nan():
    a = po.uniform((8, 5), 1)
    b = po.uniform((5, 6), 2)
    c = np.full((8, 6), np.nan, order="F")
    po.dgemm(0, 0, 1.0, a, b, 0.0, c)
    assert np.isfinite(c).all()
    c2 = np.full((8, 6), np.nan, order="F")
    po.dgemm(0, 0, 0.0, a, b, 0.0, c2)  # alpha == 0 and beta == 0: C := 0
    assert (c2 == 0).all()


def test_oracle_gemm_dmmch_grid():
    p = _load("blastest_params.json")["dblat3"]
    gen = H.DBeg()
    worst = 0.0
    for m in p["n"]:
        for n in p["n"]:
            for k in p["n"]:
                for ta in (0, 8):
                    for tb in (0, 8):
                        for alpha in p["alpha"]:
                            for beta in p["beta"]:
                                a = H.dmake_ge(gen, *((k, m) if ta else (m, k)))
                                b = H.dmake_ge(gen, *((n, k) if tb else (k, n)))
                                c0 = H.dmake_ge(gen, m, n)
                                c = np.asfortranarray(c0.copy())
                                if m and n:
                                    po.dgemm(ta, tb, alpha, a, b, beta, c)
                                worst = max(worst, H.dmmch_ratio(alpha, H.op(a, ta), H.op(b, tb), beta, c0, c))
    assert worst < p["thresh"]


def test_oracle_gemm_residual_and_dd():
    m, n, k = 200, 170, 150
    a = H.normalize(po.uniform((m, k), 1))
    b = H.normalize(po.uniform((k, n), 2))
    c0 = H.normalize(po.uniform((m, n), 3))
    c = np.asfortranarray(c0.copy())
    po.dgemm(0, 0, 2.0, a, b, 1.2, c)  # testsuite alpha/beta (test_gemm.c:213-214)
    assert H.gemm_residual(2.0, a, b, 1.2, c0, c) < 1e-14
    hi, lo = po.dd_gemm_full(0, 0, 2.0, a, b, 1.2, c0)
    g = 2.0 * (np.abs(a) @ np.abs(b)) + 1.2 * np.abs(c0)
    assert np.all(np.abs(c - hi - lo) <= 2 * k * H.EPS * g)


def test_oracle_sgemm_residual():
    m, n, k = 120, 90, 110
    a = H.normalize(po.uniform((m, k), 1, dtype=np.float32)).astype(np.float32, order="F")
    b = H.normalize(po.uniform((k, n), 2, dtype=np.float32)).astype(np.float32, order="F")
    c0 = H.normalize(po.uniform((m, n), 3, dtype=np.float32)).astype(np.float32, order="F")
    c = np.asfortranarray(c0.copy())
    po.sgemm(0, 0, 2.0, a, b, 1.2, c)
    r = H.gemm_residual(2.0, a.astype(np.float64), b.astype(np.float64), 1.2, c0.astype(np.float64),
                        c.astype(np.float64))
    assert r < 1e-5


@pytest.mark.parametrize("side", [po.LEFT, po.RIGHT])
@pytest.mark.parametrize("uplo", [po.LOWER, po.UPPER])
@pytest.mark.parametrize("trans", [po.NO_TRANSPOSE, po.TRANSPOSE])
@pytest.mark.parametrize("diag", [po.NONUNIT_DIAG, po.UNIT_DIAG])
def test_oracle_trsm_residual(side, uplo, trans, diag):
    m, n = 150, 90
    na = m if side == po.LEFT else n
    a = H.normalize(po.uniform((na, na), 4))
    a = np.asfortranarray(a + 2.0 * np.eye(na))  # testsuite loads the diagonal by 2
    tri = np.tril(a) if uplo == po.LOWER else np.triu(a)
    if diag == po.UNIT_DIAG:
        tri = tri - np.diag(np.diag(tri)) + np.eye(na)
    b0 = H.normalize(po.uniform((m, n), 5))
    x = np.asfortranarray(b0.copy())
    po.dtrsm(side, uplo, trans, diag, 2.0, a, x)
    assert H.trsm_residual(0 if side == po.LEFT else 1, 2.0, H.op(tri, trans), b0, x) < 1e-13


@pytest.mark.parametrize("trans", [po.NO_TRANSPOSE, po.TRANSPOSE])
def test_oracle_gemv_dmmch(trans):
    p = _load("blastest_params.json")["dblat2"]
    gen = H.DBeg()
    worst = 0.0
    for m in p["n"]:
        for n in p["n"]:
            for alpha in p["alpha"]:
                for beta in p["beta"]:
                    a = H.dmake_ge(gen, m, n)
                    ly, lx = (n, m) if trans else (m, n)
                    x = np.array([gen() for _ in range(lx)])
                    y0 = np.array([gen() for _ in range(ly)])
                    y = y0.copy()
                    if ly:
                        po.dgemv(trans, alpha, a, x if lx else np.zeros(1), beta, y)
                    worst = max(worst, H.dmmch_ratio(alpha, H.op(a, trans), x.reshape(-1, 1), beta,
                                                     y0.reshape(-1, 1), y.reshape(-1, 1)))
    assert worst < p["thresh"]


def test_dd_dotv_exactness():
    x = po.uniform(1000, 3).ravel()
    y = po.uniform(1000, 4).ravel()
    hi, lo = po.dd_dotv(x, y)
    from fractions import Fraction
    exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y))
    assert abs(Fraction(hi) + Fraction(lo) - exact) <= abs(exact) * Fraction(1, 2 ** 100)


@pytest.mark.parametrize("slices", [3, 5, 8])
def test_ozaki_model_error_bound(slices):
    m, n, k = 48, 40, 500
    a = po.expspread((m, k), 21)
    b = po.expspread((k, n), 22)
    c = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, a, b, 0.0, c, slices)
    hi, lo = po.dd_gemm_full(0, 0, 1.0, a, b, 0.0, c)
    # representation error per row: 2^-(8s+1) * 2^e_row; bound the product error
    ea = 2.0 ** (np.floor(np.log2(np.abs(a).max(axis=1))) + 2)
    eb = 2.0 ** (np.floor(np.log2(np.abs(b).max(axis=0))) + 2)
    u = 2.0 ** (-8 * slices - 1)
    bound = u * (ea[:, None] * (np.abs(b).sum(axis=0))[None, :] + (np.abs(a).sum(axis=1))[:, None] * eb[None, :])
    bound += (slices + 2) * H.EPS * np.abs(hi) + ea[:, None] * eb[None, :] * 2.0 ** (-8 * (slices + 1)) * k
    assert np.all(np.abs(c - hi - lo) <= bound)


def test_ozaki_model_beats_native_at_8_slices():
    m, n, k = 96, 96, 2000
    a = po.expspread((m, k), 31)
    b = po.expspread((k, n), 32)
    c = np.zeros((m, n), order="F")
    cn = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, a, b, 0.0, c, 8)
    po.dgemm(0, 0, 1.0, a, b, 0.0, cn)
    hi, lo = po.dd_gemm_full(0, 0, 1.0, a, b, 0.0, c)
    assert po.componentwise_error(c, hi, lo) <= po.componentwise_error(cn, hi, lo)


def test_ozaki_split_digits_exact():
    r = po.expspread((5, 64), 41)
    for s in (3, 8):
        exps, dig = po.ozaki_split(r, s)
        assert np.abs(dig).max() <= 128
        recon = sum(dig[p].astype(np.float64) * 2.0 ** (-8 * (p + 1)) for p in range(s))
        recon = recon * (2.0 ** exps.astype(np.float64))[:, None]
        tol = (2.0 ** exps.astype(np.float64))[:, None] * 2.0 ** (-8 * s - 1)
        assert np.all(np.abs(recon - r) <= tol)


def test_ozaki_kpart_limit():
    for npairs in range(1, 13):
        lim = po.ozaki_kpart_limit(npairs)
        assert lim % 64 == 0 and npairs * lim * 128 * 128 < 2 ** 31
        assert npairs * (lim + 64) * 128 * 128 >= 2 ** 31 - 1 or lim + 64 > 2 ** 31


def _digits_exact(x, e, s):
    """The digit rule restated with Python integers: X = floor(|x| 2^(F-e)),
    F = 8s+2; Y = X + sum_p 128 2^(F-8p) + 2; d_1 = Y >> (F-8) - 128,
    d_p = ((Y >> (F-8p)) & 255) - 128; the sign of x on every digit."""
    from fractions import Fraction
    F = 8 * s + 2
    out = []
    for v in x:
        X = int(Fraction(abs(float(v))) * Fraction(2) ** (F - int(e)))  # floor of a nonnegative value
        Y = X + sum(128 << (F - 8 * p) for p in range(1, s + 1)) + 2
        ds = [(Y >> (F - 8)) - 128] + [((Y >> (F - 8 * p)) & 255) - 128 for p in range(2, s + 1)]
        out.append([-d if v < 0 else d for d in ds])
    return np.array(out, dtype=np.int64).T


def test_ozaki_digits_match_integer_restatement():
    r = po.expspread((7, 200), 51)
    r[3, 5] = 0.0
    r[4, :] = po.uniform((1, 200), 52)
    # the row maximum just below half the row scale: the first digit reaches 128
    r[5, 0] = np.nextafter(2.0 ** 3, 0.0) * 0.5 * 1.999
    r[6, :] = 0.0
    r[6, 3] = 5e-320  # subnormal
    for s in (3, 7, 8, 12):
        exps, dig = po.ozaki_split(r, s)
        assert np.abs(dig).max() <= 128
        for i in range(r.shape[0]):
            ref = _digits_exact(r[i], exps[i], s)
            assert np.array_equal(dig[:, i, :].astype(np.int64), ref), (s, i)
    _, dig = po.ozaki_split(np.array([[0.999999]]), 3)
    assert dig[0, 0, 0] == 128  # U just below 1/2: 128 is the first digit


def test_ozaki_recombination_is_correctly_rounded():
    from fractions import Fraction
    m, n, k, s = 6, 5, 40, 4
    a = po.expspread((m, k), 61)
    b = po.expspread((k, n), 62)
    c = np.zeros((m, n), order="F")
    po.ozaki_dgemm(0, 0, 1.0, a, b, 0.0, c, s)
    ea, da = po.ozaki_split(np.asfortranarray(a), s)
    eb, db = po.ozaki_split(np.asfortranarray(b.T), s)
    for i in range(m):
        for j in range(n):
            tot = Fraction(0)
            for pa in range(1, s + 1):
                for pb in range(1, s + 2 - pa):
                    dot = int(np.dot(da[pa - 1, i].astype(np.int64), db[pb - 1, j].astype(np.int64)))
                    tot += Fraction(dot) * Fraction(2) ** (-8 * (pa + pb))
            exact = tot * Fraction(2) ** int(ea[i] + eb[j])
            assert c[i, j] == float(exact)  # Fraction -> float rounds to nearest even


def test_rng_matches_numpy_restatement():
    """The counter RNG is reproducible from its definition (used by the GPU
    input generator too)."""
    M = (1 << 64) - 1

    def mix(z):
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return z ^ (z >> 31)

    G = 0x9E3779B97F4A7C15
    for seed, idx in [(1, 0), (7, 12345), (2 ** 40 + 3, 99)]:
        h = mix((mix((seed + G) & M) + (idx + 1) * G) & M)
        assert h == po.hash64(seed, idx)
    x = po.uniform(10, 5).ravel()
    h = [mix((mix((5 + G) & M) + (i + 1) * G) & M) for i in range(10)]
    assert np.array_equal(x, np.array([-1.0 + 2.0 * ((v >> 11) * 2.0 ** -53) for v in h]))
