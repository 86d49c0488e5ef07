"""The device entry points' blocked Ozaki form (dgemm_ozaki_blocks, gb_ozaki.cu): op(A) in row
blocks and op(B) in column blocks split on a stream of their own, one slice GEMM with its
recombination per block of C, the block products on two compute streams.

Rows and columns are split independently, so on finite operands every block carries the bits of
the CPU models of the digit and CRT forms.  Inf/NaN gates the block products one by one on the
flags of their own row and column blocks: the blocks that meet one are computed natively (IEEE
propagation), the others stay in the Ozaki form, and beta is applied once either way.
"""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import _lib
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

# The default takes blocks from 8192 (digit form) or 16384 (CRT form); GB_OZAKI_DEV_BLOCKS fixes
# the grid here at a size the CPU models finish quickly.  m is not a multiple of the 256-row tile
# and n splits unevenly, so the last row and column blocks are ragged.
M, NN, K = 2600, 4100, 300


@pytest.fixture(autouse=True, params=["4x2", "8x3"])
def blocks(request, monkeypatch):
    monkeypatch.setenv("GB_OZAKI_DEV_BLOCKS", request.param)
    yield request.param


def _dev(x):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.asfortranarray(x).T.copy()).cuda()  # column-major storage


def _run(crt, count, ta, a, b, alpha, beta, c0, tb=False):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    A, B, Cd = _dev(a), _dev(b), _dev(c0)
    m, n = c0.shape
    k = a.shape[0] if ta else a.shape[1]
    fn = L.gb_dgemm_ozaki_crt_dev if crt else L.gb_dgemm_ozaki_dev
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_void_p, C.c_int64,
                   C.c_int64, C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p, C.c_int64, C.c_int64,
                   C.c_int, C.c_void_p]
    torch.cuda.synchronize()
    assert fn(8 if ta else 0, 8 if tb else 0, m, n, k, alpha, A.data_ptr(), 1, a.shape[0], B.data_ptr(), 1,
              b.shape[0], beta, Cd.data_ptr(), 1, m, count, None) == 0
    assert L.gb_synchronize() == 0
    return Cd.cpu().numpy().T


@pytest.mark.parametrize("crt,count,ta,tb", [(False, 5, False, False), (True, 12, False, True), (True, 16, True, False),
                                             (False, 7, True, True)])
def test_blocked_form_bit_exact_vs_model(gblib, crt, count, ta, tb):
    a = po.expspread((K, M) if ta else (M, K), 41)
    b = po.expspread((NN, K) if tb else (K, NN), 42)
    c0 = po.uniform((M, NN), 43)
    got = _run(crt, count, ta, a, b, 1.25, -0.5, c0, tb)
    ref = np.asfortranarray(c0.copy())
    if crt:
        po.ozaki_crt_dgemm(8 if ta else 0, 8 if tb else 0, 1.25, a, b, -0.5, ref, count)
    else:
        po.ozaki_dgemm(8 if ta else 0, 8 if tb else 0, 1.25, a, b, -0.5, ref, count)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("crt,count", [(False, 7), (True, 16)])
def test_blocked_form_nonfinite_blocks_with_beta(gblib, crt, count):
    """An Inf in the last row block of op(A) and a NaN in the last column block of op(B): those
    rows and columns follow IEEE arithmetic, every other entry is the Ozaki result of its block,
    and C0 enters once (beta = 0.5) in all of them."""
    a = po.uniform((M, K), 44)
    b = po.uniform((K, NN), 45)
    c0 = po.uniform((M, NN), 46)
    a[M - 5, 7] = np.inf
    b[11, NN - 3] = np.nan
    got = _run(crt, count, False, a, b, 1.0, 0.5, c0)
    ref = a @ b + 0.5 * c0
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.isinf(got), np.isinf(ref))
    fin = np.isfinite(ref)
    gauge = np.where(np.isfinite(a), np.abs(a), 0.0) @ np.where(np.isfinite(b), np.abs(b), 0.0) + 0.5 * np.abs(c0)
    assert np.all(np.abs(got[fin] - ref[fin]) <= 1e-12 * gauge[fin])
