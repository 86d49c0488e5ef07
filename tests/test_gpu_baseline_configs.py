"""Parity at the benchmark configurations' full sizes (one GB300).

The smaller tests compare whole results with the CPU oracle; at these sizes a full
CPU product takes too long, so each check is a size-independent property the
reference's own tests use, evaluated exactly where it matters:

* gemm (DGEMM / SGEMM 8192^3, U[-1, 1]): 4096 sampled entries against the
  double-double evaluator, within the componentwise accumulation bound
  2k u (|A||B|)_ij (u of the arithmetic's precision);
* trsm (L/L/N/N, m = 8192, n = 4096, diagonal 8192 + |u|; Ozaki form at 16384^2 too):
  the testsuite residual ||B - op(A) X t|| / (||op(A)|| ||X t|| u) on a random
  combination t of the columns (testsuite/src/test_trsm.c:290-389), and for the
  Ozaki form a sampled componentwise backward error no larger than native FP64's;
* gemv 32768^2 (N and T): every entry of y against an FP64 product with the bound
  2n u (|A||x|)_i;
* axpyv / dotv at n = 2^28: axpyv bit for bit against the oracle's fused
  multiply-add per element, dotv against the double-double dot within 2n u |x|.|y|;
* the 4096-problem batch of log-uniform [16, 1024] shapes with random transposes,
  FP64 native, FP64 Ozaki (7 slices) and FP32: every problem with the testsuite
  gemm residual (testsuite/src/test_gemm.c:303-414).
"""
import ctypes as C
import math

import numpy as np
import pytest

from blis_gb300 import _lib, dev
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

EPS64 = np.finfo(np.float64).eps
EPS32 = float(np.finfo(np.float32).eps)


def _torch():
    return pytest.importorskip("torch")


def _sample(n_rows, n_cols, count=4096, seed=5):
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(seed)
    return (torch.randint(0, n_rows, (count,), generator=g).cuda(),
            torch.randint(0, n_cols, (count,), generator=g).cuda())


def _abs_gauge(A, B, ii, jj):
    """(|A||B|)_ij for the sampled entries, in FP64 (A, B column-major device tensors)."""
    torch = _torch()
    out = torch.empty(ii.numel(), dtype=torch.float64, device="cuda")
    for s in range(0, ii.numel(), 512):
        ra = A[ii[s:s + 512], :].double().abs()
        cb = B[:, jj[s:s + 512]].double().abs().t()
        out[s:s + 512] = (ra * cb).sum(dim=1)
    return out


@pytest.mark.parametrize("prec", ["d", "s"])
def test_gemm_8192_sampled_vs_double_double(gblib, prec):
    torch = _torch()
    n = 8192
    dt = torch.float64 if prec == "d" else torch.float32
    A, B, Cm = dev.colmajor(n, n, dt), dev.colmajor(n, n, dt), dev.colmajor(n, n, dt)
    dev.randm(A, dev.RAND_UNIFORM, 81)
    dev.randm(B, dev.RAND_UNIFORM, 82)
    Cm.zero_()
    (dev.dgemm if prec == "d" else dev.sgemm)(0, 0, 1.0, A, B, 0.0, Cm)
    torch.cuda.synchronize()
    ii, jj = _sample(n, n)
    Ad, Bd = (A, B) if prec == "d" else (A.double(), B.double())
    hi, lo = dev.dd_gemm_entries(0, 0, 1.0, Ad, Bd, 0.0, None, ii, jj)
    got = Cm[ii, jj].double()
    err = (got - hi - lo).abs()
    u = EPS64 if prec == "d" else EPS32
    bound = 2 * n * u * _abs_gauge(A, B, ii, jj)
    assert bool((err <= bound).all()), float((err / bound).max())


def _trsm_problem(m, n, seed, b_kind=dev.RAND_UNIFORM):
    torch = _torch()
    L = dev.colmajor(m, m)
    dev.randm(L, dev.RAND_UNIFORM, seed)
    L.copy_(torch.tril(L))
    L.diagonal().copy_(m + L.diagonal().abs())
    Bm = dev.colmajor(m, n)
    if b_kind == dev.RAND_EXPSPREAD:
        dev.randm(Bm, dev.RAND_EXPSPREAD, seed + 1, -20, 20)
    else:
        dev.randm(Bm, b_kind, seed + 1)
    return L, Bm


def _trsm_residual(L, B0, X, seed=7):
    """The testsuite's trsm residual: ||L (X t) - B0 t|| / (||L||_F ||X t|| eps) for random t."""
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(seed)
    t = (torch.rand(X.shape[1], generator=g, dtype=torch.float64) * 2 - 1).cuda()
    xt = X @ t
    r = L @ xt - B0 @ t
    return float(r.norm() / (L.norm() * xt.norm() * EPS64))


def _backward_error_sample(L, B0, X, cols):
    """max over sampled columns j and rows i of |L X_j - B0_j|_i / (|L| |X_j|)_i."""
    Xs = X[:, cols]
    r = (L @ Xs - B0[:, cols]).abs()
    g = L.abs() @ Xs.abs()
    return float((r / g).max())


@pytest.mark.parametrize("form", ["native", "ozaki"])
def test_dtrsm_8192x4096_testsuite_residual(gblib, form):
    torch = _torch()
    m, n = 8192, 4096
    L, Bm = _trsm_problem(m, n, 91)
    B0 = Bm.clone()
    L_ = _lib.load()
    if form == "ozaki":
        _lib.check(L_.gb_set_dgemm_mode(1, 7), "mode")
    try:
        dev.dtrsm(0, 0xC0, 0, 0, 1.0, L, Bm)
        torch.cuda.synchronize()
    finally:
        L_.gb_set_dgemm_mode(0, 8)
    res = _trsm_residual(L, B0, Bm)
    # testsuite thresholds for double: pass below 1e-14 relative (test_trsm.c), here in units of eps
    assert res < 1e-14 / EPS64, res


def test_dtrsm_16384_ozaki_backward_error_at_most_native(gblib):
    """The precision form of the 16384^2 solve with (1+u) 2^e right-hand sides: its sampled
    componentwise backward error is no larger than native FP64's (within 2x, the sample noise of
    two backward-stable solves at the roundoff level)."""
    torch = _torch()
    m = n = 16384
    L, Bm = _trsm_problem(m, n, 95, dev.RAND_EXPSPREAD)
    B0 = Bm.clone()
    Xn = Bm.clone()
    dev.dtrsm(0, 0xC0, 0, 0, 1.0, L, Xn)
    L_ = _lib.load()
    _lib.check(L_.gb_set_dgemm_mode(1, 7), "mode")
    try:
        dev.dtrsm(0, 0xC0, 0, 0, 1.0, L, Bm)
        torch.cuda.synchronize()
    finally:
        L_.gb_set_dgemm_mode(0, 8)
    g = torch.Generator(device="cpu").manual_seed(3)
    cols = torch.randint(0, n, (64,), generator=g).cuda()
    be_oz = _backward_error_sample(L, B0, Bm, cols)
    be_nat = _backward_error_sample(L, B0, Xn, cols)
    assert be_oz <= max(2 * be_nat, 8 * EPS64), (be_oz, be_nat)


@pytest.mark.parametrize("trans", [0, 8])
def test_dgemv_32768_every_entry(gblib, trans):
    torch = _torch()
    n = 32768
    A = dev.colmajor(n, n)
    dev.randm(A, dev.RAND_UNIFORM, 71)
    x = torch.empty(n, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    y0 = torch.empty(n, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    y = y0.clone()
    dev.dgemv(trans, 0.75, A, x, -0.5, y)
    torch.cuda.synchronize()
    op = A.t() if trans else A
    ref = 0.75 * (op @ x) - 0.5 * y0
    gauge = 0.75 * (op.abs() @ x.abs()) + 0.5 * y0.abs()
    assert bool(((y - ref).abs() <= 2 * (n + 2) * EPS64 * gauge).all())


def test_daxpyv_ddotv_2p28(gblib):
    torch = _torch()
    n = 1 << 28
    x = torch.empty(n, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    y = torch.empty(n, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    rho = torch.empty(1, dtype=torch.float64, device="cuda")
    dev.ddotv(x, y, rho)
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    torch.cuda.synchronize()
    hi, lo = po.dd_dotv(xh, yh)
    gauge = float(np.dot(np.abs(xh), np.abs(yh)))
    assert abs(float(rho.item()) - (hi + lo)) <= 2 * n * EPS64 * gauge
    dev.daxpyv(-0.3, x, y)
    torch.cuda.synchronize()
    ref = yh.copy()
    po.daxpyv(-0.3, xh, ref)
    assert np.array_equal(y.cpu().numpy(), ref)


def _gemm_residual_t(A, B, C0, Cn, alpha, beta, ta, tb, seed):
    """Testsuite gemm residual (test_gemm.c): ||C t - (beta C0 t + alpha op(A)(op(B) t))|| over
    (||op(A)|| ||op(B)|| ||t|| eps), in FP64 on the host."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(-1.0, 1.0, size=Cn.shape[1])
    oa = A.T if ta else A
    ob = B.T if tb else B
    v = Cn @ t
    z = alpha * (oa @ (ob @ t)) + beta * (C0 @ t)
    den = np.linalg.norm(oa) * np.linalg.norm(ob) * np.linalg.norm(t)
    return float(np.linalg.norm(v - z) / den) if den > 0 else 0.0


@pytest.mark.parametrize("dtype,name", [(0, "fp64"), (2, "fp64_ozaki_s7"), (1, "fp32")])
def test_batch_4096_every_problem_testsuite_residual(gblib, dtype, name):
    torch = _torch()
    from blis_gb300 import perf
    L_ = _lib.load()
    if dtype == 2:
        _lib.check(L_.gb_set_dgemm_mode(1, 7), "mode")
    try:
        probs, (A, B, Cc), _ = perf.batch_problems(4096, 4, 1 if dtype == 1 else 0)
        Ah, Bh = A.cpu().numpy().astype(np.float64), B.cpu().numpy().astype(np.float64)
        plan = C.c_void_p()
        _lib.check(L_.gb_batch_plan_create(C.addressof(probs), 4096, dtype, C.byref(plan)), "plan")
        try:
            _lib.check(L_.gb_batch_plan_run(plan, 1, C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                       "run")
            torch.cuda.synchronize()
        finally:
            L_.gb_batch_plan_destroy(plan)
    finally:
        L_.gb_set_dgemm_mode(0, 8)
    Ch = Cc.cpu().numpy().astype(np.float64)
    u = EPS32 if dtype == 1 else EPS64
    es = A.element_size()
    worst = 0.0
    oa = ob = oc = 0
    for i in range(4096):
        p = probs[i]
        m, n, k = p.m, p.n, p.k
        ta, tb = bool(p.transa & 8), bool(p.transb & 8)
        a = Ah[oa:oa + m * k].reshape((m, k) if not ta else (k, m), order="F")
        b = Bh[ob:ob + k * n].reshape((k, n) if not tb else (n, k), order="F")
        c = Ch[oc:oc + m * n].reshape((m, n), order="F")
        r = _gemm_residual_t(a, b, np.zeros((m, n)), c, 1.0, 0.0, ta, tb, i) / u
        worst = max(worst, r)
        oa += m * k
        ob += k * n
        oc += m * n
    assert es in (4, 8)
    # the testsuite passes a gemm below 1e-14 (double) / 1e-5 (float) relative; in units of u
    # both are a few tens
    assert worst < (1e-14 / EPS64 if dtype != 1 else 1e-5 / EPS32), worst
