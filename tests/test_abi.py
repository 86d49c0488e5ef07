"""The C-ABI library: loads, exports every declared symbol, and handles
argument errors exactly like the reference's BLAS layer (xerbla numbering
of frame/compat/check/bla_*_check.h).  No GPU is touched: invalid calls
return before any device work."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from blis_gb300 import _lib, blas


def test_library_exports_every_declared_symbol(gblib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    syms = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    declared = _lib.declared_functions()
    assert len(declared) > 40
    missing = [d for d in declared if d not in syms]
    assert missing == []


def test_library_links_no_oracle(gblib):
    out = subprocess.run(["nm", "-D", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "orc_" not in out
    deps = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "gb_oracle" not in deps


def _last():
    code, msg = _lib.last_error()
    _lib.load().gb_clear_last_error()
    return code, msg


@pytest.mark.parametrize("args,info", [
    (("X", "N", 2, 2, 2, 2, 2, 2), 1),
    (("N", "X", 2, 2, 2, 2, 2, 2), 2),
    (("N", "N", -1, 2, 2, 2, 2, 2), 3),
    (("N", "N", 2, -1, 2, 2, 2, 2), 4),
    (("N", "N", 2, 2, -1, 2, 2, 2), 5),
    (("N", "N", 4, 2, 2, 3, 2, 4), 8),
    (("N", "N", 2, 2, 4, 2, 3, 2), 10),
    (("N", "N", 4, 2, 2, 4, 2, 3), 13),
    (("T", "N", 2, 2, 4, 3, 4, 2), 8),
])
def test_dgemm_argument_errors(gblib, capfd, args, info):
    ta, tb, m, n, k, lda, ldb, ldc = args
    a = np.zeros(64)
    c = np.full(64, 7.0)
    blas.dgemm(ta, tb, m, n, k, 1.0, a, lda, a, ldb, 0.0, c, ldc)
    out = capfd.readouterr().out
    assert "parameter number %2d had an illegal value" % info in out
    assert "DGEMM" in out
    assert (c == 7.0).all()  # untouched
    code, _ = _last()
    assert code == -1


def test_dtrsm_and_dgemv_argument_errors(gblib, capfd):
    a = np.zeros(16)
    blas.dtrsm("X", "L", "N", "N", 2, 2, 1.0, a, 2, a, 2)
    assert "parameter number  1" in capfd.readouterr().out
    blas.dtrsm("L", "L", "N", "N", 3, 2, 1.0, a, 2, a, 3)
    assert "parameter number  9" in capfd.readouterr().out
    blas.dgemv("N", 2, 2, 1.0, a, 2, a, 0, 0.0, a, 1)
    assert "parameter number  8" in capfd.readouterr().out
    blas.dgemv("N", 2, 2, 1.0, a, 1, a, 1, 0.0, a, 1)
    assert "parameter number  6" in capfd.readouterr().out
    _last()


def test_dgemm_batch_argument_error(gblib, capfd):
    x = np.zeros(16)
    blas.dgemm_batch(["N", "Q"], ["N", "N"], [2, 2], [2, 2], [2, 2], [1.0, 1.0], [x, x], [2, 2],
                     [x, x], [2, 2], [0.0, 0.0], [x, x], [2, 2], [1, 1])
    assert "parameter number  1" in capfd.readouterr().out
    _last()


def test_set_dgemm_mode_validation(gblib):
    L = _lib.load()
    assert L.gb_set_dgemm_mode(7, 8) != 0
    assert L.gb_set_dgemm_mode(1, 1) != 0
    assert L.gb_set_dgemm_mode(1, 8) == 0
    assert L.gb_set_dgemm_mode(0, 8) == 0
    _last()


def test_quick_returns_do_not_touch_device(gblib):
    # n <= 0 and alpha == 0 return before any device work (no GPU here)
    x = np.arange(4.0)
    y = np.arange(4.0)
    blas.daxpy(0, 2.0, x, 1, y, 1)
    blas.daxpy(4, 0.0, x, 1, y, 1)
    assert (y == np.arange(4.0)).all()
    c = np.ones(4)
    blas.dgemm("N", "N", 0, 2, 2, 1.0, x, 1, x, 2, 0.0, c, 1)
    assert (c == 1).all()


def test_declared_functions_parser():
    names = _lib.declared_functions()
    for n in ("dgemm_", "cblas_dgemm", "bli_dgemm", "gb_dgemm_ozaki_dev", "gb_batch_plan_run"):
        assert n in names
    assert C.sizeof(C.c_int32) == 4


def test_level3x_argument_errors(gblib, capfd):
    # frame/compat/check/bla_trmm_check.h, bla_hemm_check.h (symm), bla_syrk_check.h, bla_gemmt_check.h
    a = np.zeros(64)
    c = np.full(64, 7.0)
    blas.dtrmm("L", "X", "N", "N", 2, 2, 1.0, a, 2, c, 2)
    assert "DTRMM" in capfd.readouterr().out
    blas.dtrmm("R", "L", "N", "N", 2, 3, 1.0, a, 2, c, 2)  # lda < n on the right
    assert "parameter number  9" in capfd.readouterr().out
    blas.dsymm("L", "U", 3, 2, 1.0, a, 3, a, 3, 0.0, c, 2)  # ldc < m
    assert "parameter number 12" in capfd.readouterr().out
    blas.dsymm("Q", "U", 3, 2, 1.0, a, 3, a, 3, 0.0, c, 3)
    assert "parameter number  1" in capfd.readouterr().out
    blas.dsyrk("L", "X", 2, 2, 1.0, a, 2, 0.0, c, 2)
    assert "parameter number  2" in capfd.readouterr().out
    blas.dsyrk("L", "T", 2, 3, 1.0, a, 2, 0.0, c, 2)  # trans: lda < k
    assert "parameter number  7" in capfd.readouterr().out
    blas.dgemmt("U", "N", "N", 3, 2, 1.0, a, 3, a, 1, 0.0, c, 3)  # ldb < k
    assert "parameter number 10" in capfd.readouterr().out
    blas.dgemmt("U", "N", "N", -1, 2, 1.0, a, 3, a, 2, 0.0, c, 3)
    assert "DGEMMT" in capfd.readouterr().out
    assert (c == 7.0).all()
    _last()


def test_level12x_argument_errors(gblib, capfd):
    # frame/compat/check/bla_ger_check.h:37-68, bla_trmv_check.h:37-77 (trsv)
    a = np.full(64, 7.0)
    x = np.ones(8)
    blas.dger(2, 2, 1.0, x, 0, x, 1, a, 2)
    assert "parameter number  5" in capfd.readouterr().out
    blas.dger(3, 2, 1.0, x, 1, x, 1, a, 2)
    assert "parameter number  9" in capfd.readouterr().out
    blas.dtrsv("L", "N", "Z", 2, a, 2, x, 1)
    assert "parameter number  3" in capfd.readouterr().out
    blas.dtrsv("L", "N", "N", 2, a, 2, x, 0)
    assert "parameter number  8" in capfd.readouterr().out
    assert (a == 7.0).all() and (x == 1.0).all()
    # idamax_: n < 1 or incx <= 0 return 0 without touching the device
    assert blas.idamax(0, x, 1) == 0 and blas.idamax(4, x, 0) == 0 and blas.idamax(4, x, -1) == 0
    _last()


def test_hermitian_argument_errors(gblib, capfd):
    # frame/compat/check/bla_herk_check.h:37-77, bla_her2k_check.h:37-79, bla_hemm_check.h:37-79,
    # bla_syr2k_check.h:37-84
    a = np.zeros(64, dtype=np.complex128)
    c = np.full(64, 7.0 + 1.0j)
    blas.zherk("L", "T", 2, 2, 1.0, a, 2, 0.0, c, 2)  # herk takes N or C only
    assert "ZHERK" in capfd.readouterr().out
    blas.zherk("U", "C", 2, 3, 1.0, a, 2, 0.0, c, 2)  # trans C: lda < k
    assert "parameter number  7" in capfd.readouterr().out
    blas.zherk("U", "N", 3, 2, 1.0, a, 3, 0.0, c, 2)  # ldc < n
    assert "parameter number 10" in capfd.readouterr().out
    blas.zher2k("L", "N", 3, 2, 1.0, a, 3, a, 2, 0.0, c, 3)  # ldb < n
    assert "parameter number  9" in capfd.readouterr().out
    blas.zher2k("X", "N", 3, 2, 1.0, a, 3, a, 3, 0.0, c, 3)
    assert "ZHER2K" in capfd.readouterr().out
    blas.zhemm("R", "L", 2, 3, 1.0, a, 2, a, 2, 0.0, c, 2)  # right: lda < n
    assert "ZHEMM" in capfd.readouterr().out
    blas.zsymm("L", "L", 3, 2, 1.0, a, 3, a, 3, 0.0, c, 2)  # ldc < m
    assert "parameter number 12" in capfd.readouterr().out
    blas.cherk("L", "N", -1, 2, 1.0, a.astype(np.complex64), 2, 0.0, c.astype(np.complex64), 2)
    assert "CHERK" in capfd.readouterr().out
    d = np.zeros(64)
    blas.dsyr2k("L", "N", 3, 2, 1.0, d, 3, d, 2, 0.0, d, 3)
    assert "DSYR2K" in capfd.readouterr().out
    assert (c == 7.0 + 1.0j).all()
    _last()
