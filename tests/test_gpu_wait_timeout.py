"""A bounded device wait that runs out, in the form this pool allows.

The one-launch dtrsv (trsv_flags_kernel, gb_trsm.cu) passes each 64-row block of
x from CTA to CTA through flags; every wait on a flag is bounded by a budget of
%globaltimer nanoseconds.  The test hook gb_test_trsv_wait_fault makes the CTA
of one block skip its publish (a flag that nothing sets) and shortens the budget
to a few milliseconds.  The CTAs after it must give up, report DEV_WAIT_TIMEOUT
in the status word and stop the rest of the grid; the call returns normally with
GB_ERR_DEVICE, and the next call, with the hook off, is clean and correct.
Nothing traps, faults or waits without a bound.
"""
import ctypes as C
import time

import numpy as np
import pytest

from blis_gb300 import _lib, blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu

GB_ERR_DEVICE = -3


def _hook(L, block, ns):
    L.gb_test_trsv_wait_fault.restype = C.c_int
    L.gb_test_trsv_wait_fault.argtypes = [C.c_int64, C.c_int64]
    assert L.gb_test_trsv_wait_fault(block, ns) == 0


def _solve(m, seed):
    a = np.asfortranarray(H.normalize(po.uniform((m, m), seed)) + 2.0 * np.eye(m))
    b = po.uniform((m,), seed + 1)
    x = b.copy()
    blas.dtrsv("L", "N", "N", m, a, m, x, 1)
    return a, b, x


def test_withheld_flag_times_out_then_recovers(gblib):
    L = _lib.load()
    L.gb_clear_last_error()
    m = 1024  # 16 blocks of 64 rows
    try:
        _hook(L, 3, 5_000_000)  # block 3 never published; 5 ms budget
        t0 = time.perf_counter()
        _solve(m, 41)
        dt = time.perf_counter() - t0
        code, msg = _lib.last_error()
    finally:
        _hook(L, -1, 0)
    assert code == GB_ERR_DEVICE, (code, msg)
    assert "bounded wait timed out" in msg, msg
    assert dt < 2.0  # the shortened budget, not the default 2 s per wait
    # the next call is clean and correct
    L.gb_clear_last_error()
    a, b, x = _solve(m, 43)
    code, msg = _lib.last_error()
    assert code == 0, msg
    ref = b.copy()
    po.dtrsv(po.LOWER, 0, po.NONUNIT_DIAG, 1.0, a, ref)
    assert np.max(np.abs(x - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_hook_rejects_bad_budget(gblib):
    L = _lib.load()
    L.gb_test_trsv_wait_fault.restype = C.c_int
    L.gb_test_trsv_wait_fault.argtypes = [C.c_int64, C.c_int64]
    assert L.gb_test_trsv_wait_fault(0, 10) != 0          # below 0.1 ms
    assert L.gb_test_trsv_wait_fault(0, 10**11) != 0      # above 10 s
    assert L.gb_test_trsv_wait_fault(-1, 0) == 0
