"""BLIS's own host code on the GPU: the reference's testsuite and netlib BLAS tests, unchanged,
against the GPU-backed BLIS build (integration/build.py).

Two link orders are exercised:
  * seams: libgb300_blis.so ahead of a libblis built with the gb300 gemm sandbox.  BLIS's
    object, typed and BLAS front ends run as they are; gemm reaches the GPU through the
    sandbox bli_gemm_ex, trsm through the interposed bli_trsm_ex, gemv through bli_dgemv_ex,
    axpyv/dotv through the kernels registered in BLIS's context.  The glue library's exit
    report (GB300_BLIS_REPORT) shows the GPU calls and that none was forwarded to the CPU.
  * interposition: libblis_gb300.so ahead of plain libblis; the library's own BLAS front
    ends (argument checks, xerbla_ numbering) replace BLIS's.

Pass criteria are the programs' own: the testsuite's residual verdicts
(testsuite/src/test_gemm.c:303-414, test_trsm.c:290-389, test_gemv.c, test_axpyv.c,
test_dotv.c) with no FAIL, and the netlib programs' "PASSED THE COMPUTATIONAL TESTS" /
"PASSED THE TESTS OF ERROR-EXITS" (threshold 16, blastest/input/dblat3.in) or "PASS".
"""
import json
import os
import subprocess

import numpy as np
import pytest

from tests import blis_programs as bp

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PARAMS = json.load(open(os.path.join(HERE, "golden", "blastest_params.json")))


@pytest.fixture(scope="module")
def integ():
    from integration import build as ib
    p = ib.build()
    if p is None:
        pytest.skip("no BLIS sources on this machine (neither the reference tree nor its snapshot)")
    return p


def report_env():
    e = dict(os.environ)
    e["GB300_BLIS_REPORT"] = "1"
    return e


TS_CASES = [
    ("hot_path_d", ("gemm", "trsm", "gemv", "axpyv", "dotv"), "d"),
    ("gemm_sdcz", ("gemm",), "sdcz"),
    ("trsm_z", ("trsm",), "z"),
]


@pytest.mark.parametrize("rand", [0, 1], ids=["uniform", "narrow_pow2"])
@pytest.mark.parametrize("name,ops,dts", TS_CASES, ids=[c[0] for c in TS_CASES])
def test_blis_testsuite_through_seams(integ, tmp_path, name, ops, dts, rand):
    gen, opf = bp.write_testsuite_inputs(str(tmp_path), set(ops), dts, rand)
    r = subprocess.run([os.path.join(integ["bin"], "test_libblis.x"), "-g", gen, "-o", opf],
                       capture_output=True, text=True, env=report_env(), cwd=str(tmp_path), timeout=1200)
    assert r.returncode == 0, r.stderr[-2000:]
    res = bp.parse_testsuite(r.stdout)
    for dt in dts:
        for op in ops:
            assert (dt, op) in res, "no results for %s%s" % (dt, op)
            assert res[(dt, op)]["PASS"] > 0
            assert res[(dt, op)]["FAIL"] == 0, (dt, op, res[(dt, op)])
    rep = bp.parse_report(r.stderr)
    assert rep is not None, r.stderr[-2000:]
    assert rep["kernel_launches"] > 0
    if "gemm" in ops:
        assert rep["gemm_gpu"] > 0 and rep["gemm_cpu_forwarded"] == 0, rep
    if "trsm" in ops:
        assert rep["trsm_gpu"] > 0 and rep["trsm_cpu_forwarded"] == 0, rep
    if "gemv" in ops:
        assert rep["gemv_gpu"] > 0, rep
    if "axpyv" in ops:
        assert rep["axpyv_gpu"] > 0, rep
    if "dotv" in ops:
        assert rep["dotv_gpu"] > 0, rep


# routines whose calls reach the GPU in each link order
SEAM_ROUTINES = {
    "dblat1": ["DDOT", "DAXPY"], "dblat2": ["DGEMV"], "dblat3": ["DGEMM", "DTRSM"],
    "sblat3": ["SGEMM", "STRSM"], "zblat3": ["ZGEMM", "ZTRSM"], "cblat3": ["CGEMM", "CTRSM"],
}
INTERPOSED_ROUTINES = {
    "dblat1": ["DDOT", "DAXPY", "DCOPY", "DSCAL", "IDAMAX"],
    "dblat2": ["DGEMV", "DGER", "DTRSV"],
    "dblat3": ["DGEMM", "DSYMM", "DTRMM", "DTRSM", "DSYRK", "DSYR2K"],
    "sblat3": ["SGEMM", "STRSM"],
    "zblat3": ["ZGEMM", "ZHEMM", "ZSYMM", "ZTRMM", "ZTRSM", "ZHERK", "ZSYRK", "ZHER2K", "ZSYR2K"],
    "cblat3": ["CGEMM", "CHEMM", "CSYMM", "CTRMM", "CTRSM", "CHERK", "CSYRK", "CHER2K", "CSYR2K"],
}


def _check_blat(prog, routines, rc, summary, err):
    assert rc == 0, err[-2000:]
    res = bp.blat_results(summary)
    assert "_" not in res, summary[-3000:]
    for name, verdicts in res.items():
        assert "FAILED" not in verdicts and "FAIL" not in verdicts, (prog, name, summary[-3000:])
    for name in routines:
        assert name in res, (prog, name, summary[-3000:])
        if prog.endswith("1"):
            assert res[name] == {"PASS"}, (prog, name, res[name])
        else:
            assert res[name] == {"PASSED COMPUTATIONAL TESTS", "PASSED TESTS OF ERROR-EXITS"}, (prog, name, res[name])


@pytest.mark.parametrize("prog", sorted(SEAM_ROUTINES))
def test_blas_tests_through_seams(integ, tmp_path, prog):
    rc, summary, err = bp.run_blat(integ["bin"], prog, str(tmp_path), PARAMS, env=report_env())
    _check_blat(prog, SEAM_ROUTINES[prog], rc, summary, err)
    rep = bp.parse_report(err)
    assert rep is not None and rep["kernel_launches"] > 0, err[-2000:]
    assert rep["gemm_cpu_forwarded"] == 0, rep
    if prog == "dblat1":
        assert rep["axpyv_gpu"] > 0 and rep["dotv_gpu"] > 0, rep
    elif prog == "dblat2":
        assert rep["gemv_gpu"] > 0, rep
    else:
        assert rep["gemm_gpu"] > 0, rep
        assert rep["trsm_gpu"] > 0 and rep["trsm_cpu_forwarded"] == 0, rep


@pytest.mark.parametrize("prog", sorted(INTERPOSED_ROUTINES))
def test_blas_tests_interposed(integ, tmp_path, prog):
    rc, summary, err = bp.run_blat(integ["bin_interpose"], prog, str(tmp_path), PARAMS)
    _check_blat(prog, INTERPOSED_ROUTINES[prog], rc, summary, err)


@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (-0.75, 0.5)])
def test_obj_gemm_comp_prec_takes_ozaki(integ, tmp_path, alpha, beta):
    """A double obj_t gemm with bli_obj_set_comp_prec(BLIS_SINGLE_PREC, &c) through BLIS's
    bli_gemm and the sandbox: the result is the Ozaki model's, bit for bit, at the slice count
    the library chose (selector proposal raised by the verifier)."""
    from oracle import pyoracle as po
    m, n, k = 300, 260, 1100
    a = po.expspread((m, k), 31)
    b = po.expspread((k, n), 32)
    c = po.uniform((m, n), 33)
    inp = tmp_path / "in.bin"
    out = tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([m, n, k], dtype=np.int64).tofile(f)
        np.array([alpha, beta], dtype=np.float64).tofile(f)
        for x in (a, b, c):
            x.ravel(order="F").tofile(f)
    r = subprocess.run([integ["comp_prec"], str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    raw = open(out, "rb").read()
    slices = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    got = np.frombuffer(raw[4:], dtype=np.float64).reshape((m, n), order="F")
    assert 2 <= slices <= 12, slices
    ref = np.array(c, order="F", copy=True)
    po.ozaki_dgemm(0, 0, alpha, a, b, beta, ref, slices)
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))
