"""The oracle pinned to the reference BLIS itself (CPU, no GPU).

tests/golden/blis_ref_outputs.npz holds outputs of the reference BLIS's typed API
(bli_dgemm, bli_dtrsm, bli_dgemv, bli_daxpyv, bli_ddotv), compiled from the
reference's sources by oracle/ref_blis.py and run by tests/golden/make_blis_golden.py
on the oracle's seeded inputs.  The oracle must reproduce them: bit for bit where the
arithmetic is exact in any order (the testsuite's narrow-power-of-two inputs with
alpha = 1 and beta in {0, 1}, frame/include/bli_cast_macro_defs.h:477-525; axpyv, one
fused multiply-add per element in both), and within the FP64 accumulation bound
elsewhere.  Where the reference build is present on this machine, the same checks run
live, and BLIS's own testsuite is run on the build to pin it in turn.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import pyoracle as po
from tests import blis_programs as bp

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "blis_ref_outputs.npz"))
EPS = np.finfo(np.float64).eps

import importlib.util  # noqa: E402
_spec = importlib.util.spec_from_file_location("make_blis_golden",
                                               os.path.join(HERE, "golden", "make_blis_golden.py"))
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)


def gemm_bound(k, alpha, a, b, beta, c, ta, tb):
    oa = a.T if ta else a
    ob = b.T if tb else b
    return 2 * (k + 2) * EPS * (abs(alpha) * (np.abs(oa) @ np.abs(ob)) + abs(beta) * np.abs(c))


@pytest.mark.parametrize("i", range(len(mg.GEMM)))
def test_oracle_gemm_matches_blis(i):
    m, n, k, ta, tb, al, be, g = mg.GEMM[i]
    s = 100 + 10 * i
    a = mg.gen(g, (k, m) if ta else (m, k), s)
    b = mg.gen(g, (n, k) if tb else (k, n), s + 1)
    c = mg.gen(g, (m, n), s + 2)
    c0 = c.copy(order="F")
    po.dgemm(ta, tb, al, a, b, be, c)
    ref = GOLD["gemm%d" % i]
    if g == "pow2" and al == 1.0 and be in (0.0, 1.0):
        assert np.array_equal(c, ref)
    else:
        assert np.all(np.abs(c - ref) <= gemm_bound(k, al, a, b, be, c0, ta, tb))


@pytest.mark.parametrize("i", range(len(mg.TRSM)))
def test_oracle_trsm_matches_blis(i):
    sd, up, t, dg = mg.TRSM[i]
    a, b = mg.trsm_inputs(sd, 32, 24, 300 + 10 * i)
    po.dtrsm(sd, up, t, dg, 0.75, a, b)
    ref = GOLD["trsm%d" % i]
    # both solve a diagonally dominant system (condition number about 1): the difference
    # of two backward-stable solutions is a few units of roundoff of the solution's size
    na = a.shape[0]
    assert np.linalg.norm(b - ref) <= 8 * na * EPS * np.linalg.norm(ref)


@pytest.mark.parametrize("i", range(len(mg.GEMV)))
def test_oracle_gemv_matches_blis(i):
    t, m, n, al, be, g = mg.GEMV[i]
    s = 500 + 10 * i
    a = mg.gen(g, (m, n), s)
    x = mg.gen(g, ((m if t else n),), s + 1)
    y = mg.gen(g, ((n if t else m),), s + 2)
    y0 = y.copy()
    po.dgemv(t, al, a, x, be, y)
    ref = GOLD["gemv%d" % i]
    if g == "pow2" and al == 1.0 and be in (0.0, 1.0):
        assert np.array_equal(y, ref)
    else:
        oa = a.T if t else a
        bound = 2 * (oa.shape[1] + 2) * EPS * (abs(al) * (np.abs(oa) @ np.abs(x)) + abs(be) * np.abs(y0))
        assert np.all(np.abs(y - ref) <= bound)


@pytest.mark.parametrize("i,g", [(0, "pow2"), (1, "uniform")])
def test_oracle_level1v_matches_blis(i, g):
    x = mg.gen(g, (mg.VEC_N,), 700 + i)
    y = mg.gen(g, (mg.VEC_N,), 710 + i)
    rho = po.ddotv(x, y)
    ref = float(GOLD["dotv%d" % i])
    if g == "pow2":
        assert rho == ref
    else:
        assert abs(rho - ref) <= 2 * mg.VEC_N * EPS * float(np.sum(np.abs(x) * np.abs(y)))
    po.daxpyv(0.625 if g == "pow2" else -0.3, x, y)
    assert np.array_equal(y, GOLD["axpyv%d" % i])


# ---------------------------------------------------------------- live reference build
def _blis():
    from oracle import blis_ctypes as bc
    if not bc.available():
        pytest.skip("reference BLIS not built on this machine (python -m oracle.ref_blis)")
    return bc


def test_live_blis_gemm_matches_oracle():
    bc = _blis()
    m, n, k = 200, 150, 300
    for g, al, be in (("pow2", 1.0, 1.0), ("uniform", 0.9, -0.4)):
        a = mg.gen(g, (m, k), 901)
        b = mg.gen(g, (k, n), 902)
        c = mg.gen(g, (m, n), 903)
        c1, c2 = c.copy(order="F"), c.copy(order="F")
        bc.dgemm(0, 0, al, a, b, be, c1)
        po.dgemm(0, 0, al, a, b, be, c2)
        if g == "pow2":
            assert np.array_equal(c1, c2)
        else:
            assert np.all(np.abs(c1 - c2) <= gemm_bound(k, al, a, b, be, c, 0, 0))


def test_live_blis_build_passes_its_testsuite():
    """The reference build itself passes BLIS's testsuite on the hot-path operations
    (both randomisations), so its outputs are a trustworthy pin."""
    _blis()
    from oracle import ref_blis
    exe = os.path.join(ref_blis.config_dir(), "bin", "test_libblis.x")
    with tempfile.TemporaryDirectory() as d:
        for rand in (0, 1):
            gen, opf = bp.write_testsuite_inputs(d, {"gemm", "trsm", "gemv", "axpyv", "dotv"}, "sdcz", rand,
                                                 sizes=(100, 200, 100))
            r = subprocess.run([exe, "-g", gen, "-o", opf], capture_output=True, text=True, timeout=600, cwd=d)
            assert r.returncode == 0
            res = bp.parse_testsuite(r.stdout)
            for dt in "sdcz":
                for op in ("gemm", "trsm", "gemv", "axpyv", "dotv"):
                    assert (dt, op) in res
            assert all(v["FAIL"] == 0 and v["PASS"] > 0 for v in res.values()), res
