"""STRSM on the GPU (gb_trsm.cu strsm_dev): the FP32 recursion over 64-row diagonal blocks (the
diagonal-solve kernel of dtrsm at FP32) with updates through sgemm's engine choice, against an
FP64 solution of the same FP32 problem with the testsuite's residual; the BLAS front end strsm_
on host buffers with its netlib argument checks."""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import _lib, blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu
EPS32 = float(np.finfo(np.float32).eps)


def _tri(m, lower, unit, seed):
    a = po.uniform((m, m), seed, dtype=np.float32)
    a = np.tril(a) if lower else np.triu(a)
    if unit:
        # a unit triangle with O(1) entries grows its solution exponentially; off-diagonal
        # entries of size 1/m keep it well conditioned (the diagonal itself is not read)
        a = (a / np.float32(m)).astype(np.float32)
    else:
        a = a + np.float32(m) * np.eye(m, dtype=np.float32)  # diagonally dominant, as the testsuite's
    return np.asfortranarray(a)


@pytest.mark.parametrize("side", [0, 1])
@pytest.mark.parametrize("uplo,trans", [(0xC0, 0), (0x60, 0), (0xC0, 8), (0x60, 8)])
@pytest.mark.parametrize("diag", [0, 1])
@pytest.mark.parametrize("m,n", [(200, 130), (1300, 1100)])
def test_strsm_dev_residual(gblib, side, uplo, trans, diag, m, n):
    torch = pytest.importorskip("torch")
    lower = uplo == 0xC0
    na = m if side == 0 else n
    a = _tri(na, lower, diag == 1, 11 + na)
    b0 = po.uniform((m, n), 12 + m, dtype=np.float32)
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # column-major storage
    B = torch.from_numpy(np.ascontiguousarray(b0.T)).cuda()
    L = _lib.load()
    rc = L.gb_strsm_dev(side, uplo, trans, 0x100 if diag else 0, m, n, 0.75, A.data_ptr(), 1, na, B.data_ptr(), 1,
                        m, None)
    assert rc == 0, _lib.last_error()
    assert L.gb_synchronize() == 0
    x = B.cpu().numpy().T.astype(np.float64)
    a_op = H.op(a.astype(np.float64), trans)
    if diag:
        np.fill_diagonal(a_op, 1.0)
    r = H.trsm_residual(side, 0.75, a_op, b0.astype(np.float64), x)
    scale = np.linalg.norm(a_op, 1) * np.linalg.norm(x) * max(m, n) * EPS32
    assert r <= 30 * scale, (r, scale)


def test_strsm_host_blas_and_checks(gblib):
    m, n = 150, 90
    a = _tri(m, True, False, 5)
    b0 = po.uniform((m, n), 6, dtype=np.float32)
    b = np.asfortranarray(b0.copy())
    blas.strsm("L", "L", "N", "N", m, n, 2.0, a, m, b, m)
    x = b.astype(np.float64)
    r = H.trsm_residual(0, 2.0, a.astype(np.float64), b0.astype(np.float64), x)
    assert r <= 30 * np.linalg.norm(a, 1) * np.linalg.norm(x) * m * EPS32
    # a bad argument goes to xerbla and leaves B alone
    b2 = np.asfortranarray(b0.copy())
    blas.strsm("L", "L", "N", "N", m, n, 2.0, a, m - 1, b2, m)  # lda < m: info 9
    assert np.array_equal(b2, b0)
    # alpha = 0: B := 0, A not read
    b3 = np.asfortranarray(b0.copy())
    blas.strsm("R", "U", "T", "U", m, n, 0.0, np.full((n, n), np.nan, dtype=np.float32, order="F"), n, b3, m)
    assert (b3 == 0).all()
