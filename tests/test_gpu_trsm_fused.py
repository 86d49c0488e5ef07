"""The fused small update of the precision-form DTRSM (trsm_update_fused_kernel in
gb_ozaki.cu): the updates of at most 128 rows and depth 128 at the bottom of the
recursion run as one launch that splits both operands into digits (A's from the digit
images trsm_image_kernel builds once per solve, or by the CTA itself with
GB_TRSM_IMAGES=0), multiplies them on the tensor cores and recombines in place; where the
updated rows are a whole diagonal block, the same launch then solves that block (the
gemmtrsm shape; GB_TRSM_GEMMTRSM=0 keeps the separate diagonal solve).  It must give the
same bits as the four-launch form (split, slice GEMM, recombination, gated IEEE fallback)
and separate diagonal solves that GB_TRSM_FUSED=0 selects, on every side / triangle /
transposition, ragged sizes, one and two column groups, and every slice count the kernel
takes."""
import os

import numpy as np
import pytest

from blis_gb300 import blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def restore(gblib):
    yield
    os.environ.pop("GB_TRSM_FUSED", None)
    os.environ.pop("GB_TRSM_IMAGES", None)
    os.environ.pop("GB_TRSM_GEMMTRSM", None)
    blas.set_dgemm_mode(blas.DGEMM_NATIVE, 8)


def _solve(side, uplo, trans, diag, m, n, alpha, a, b0, slices, fused):
    os.environ["GB_TRSM_FUSED"] = "1" if fused else "0"
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, slices)
    x = np.asfortranarray(b0.copy())
    blas.dtrsm(side, uplo, trans, diag, m, n, alpha, a, a.shape[0], x, m)
    return x


def _problem(side, m, n, seed, spread=False):
    na = m if side == "L" else n
    if spread:
        # off-diagonal magnitudes spread over 2^-20 .. 2^1 times 1/(4 na) (diagonally dominant for
        # any diagonal setting), right-hand sides over 2^-20 .. 2^20
        a = po.expspread((na, na), seed, -20, 0) / (4 * na) + np.diag(1.0 + np.abs(po.uniform((na,), seed + 1)))
        b0 = po.expspread((m, n), seed + 2)
    else:
        a = H.normalize(po.uniform((na, na), seed)) + 2.0 * np.eye(na)
        b0 = H.normalize(po.uniform((m, n), seed + 2))
    return np.asfortranarray(a), np.asfortranarray(b0)


@pytest.mark.parametrize("side,uplo,trans", [("L", "L", "N"), ("L", "U", "N"), ("L", "L", "T"), ("L", "U", "T"),
                                             ("R", "L", "N"), ("R", "U", "T")])
@pytest.mark.parametrize("m,n", [(700, 77), (256, 300), (129, 33)])
def test_fused_updates_bit_identical(side, uplo, trans, m, n):
    a, b0 = _problem(side, m, n, 31)
    ref = _solve(side, uplo, trans, "N", m, n, -0.75, a, b0, 7, False)
    got = _solve(side, uplo, trans, "N", m, n, -0.75, a, b0, 7, True)
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))
    tri = np.tril(a) if uplo == "L" else np.triu(a)
    r = H.trsm_residual(0 if side == "L" else 1, -0.75, tri.T if trans == "T" else tri, b0, got)
    assert r < 1e-12


@pytest.mark.parametrize("slices", [2, 4, 6, 8])
def test_fused_updates_every_slice_count(slices):
    m, n = 520, 190
    a, b0 = _problem("L", m, n, 41, spread=True)
    ref = _solve("L", "L", "N", "U", m, n, 1.0, a, b0, slices, False)
    got = _solve("L", "L", "N", "U", m, n, 1.0, a, b0, slices, True)
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))


@pytest.mark.parametrize("side,uplo,trans", [("L", "L", "N"), ("L", "U", "N"), ("R", "U", "T")])
def test_fused_updates_without_gemmtrsm(side, uplo, trans):
    # fused updates, diagonal blocks solved by their own launches: the same bits
    m, n = 330, 140
    a, b0 = _problem(side, m, n, 81, spread=True)
    ref = _solve(side, uplo, trans, "N", m, n, 1.0, a, b0, 7, False)
    os.environ["GB_TRSM_GEMMTRSM"] = "0"
    got = _solve(side, uplo, trans, "N", m, n, 1.0, a, b0, 7, True)
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))


@pytest.mark.parametrize("side,uplo,trans", [("L", "L", "N"), ("L", "U", "T"), ("R", "L", "T")])
def test_fused_updates_without_images(side, uplo, trans):
    # each fused update splits its A block itself: the same bits again
    m, n = 448, 100
    a, b0 = _problem(side, m, n, 71, spread=True)
    ref = _solve(side, uplo, trans, "N", m, n, 2.0, a, b0, 7, False)
    os.environ["GB_TRSM_IMAGES"] = "0"
    got = _solve(side, uplo, trans, "N", m, n, 2.0, a, b0, 7, True)
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))


def test_fused_updates_two_column_groups():
    # 2600 right-hand sides: two column halves on two streams, each with its own fused updates
    m, n = 640, 2600
    a, b0 = _problem("L", m, n, 51, spread=True)
    ref = _solve("L", "L", "N", "N", m, n, 1.0, a, b0, 7, False)
    got = _solve("L", "L", "N", "N", m, n, 1.0, a, b0, 7, True)
    assert np.array_equal(got, ref), float(np.max(np.abs(got - ref)))
    # the residual relative to |B0 t| for the helper's random combination t of the columns
    t = np.random.default_rng(7).uniform(-1.0, 1.0, size=n)
    assert H.trsm_residual(0, 1.0, np.tril(a), b0, got) < 1e-13 * np.linalg.norm(b0 @ t)


def test_fused_updates_nonfinite_tile():
    # an Inf in the right-hand side reaches the updates below it: the fused tiles that meet it
    # take FP64 FMAs (the four-launch form sends the whole update to the IEEE kernel); the
    # non-finite pattern matches and the finite entries stay within rounding
    m, n = 384, 96
    a, b0 = _problem("L", m, n, 61)
    b0[5, 40] = np.inf
    ref = _solve("L", "L", "N", "N", m, n, 1.0, a, b0, 7, False)
    got = _solve("L", "L", "N", "N", m, n, 1.0, a, b0, 7, True)
    assert np.array_equal(np.isfinite(got), np.isfinite(ref))
    # the fused path sends only the 32-column tiles that meet the Inf to FP64 FMAs, the
    # four-launch path the whole update to the IEEE kernel: the other columns differ by the
    # Ozaki form's rounding against the native kernel's, normwise
    fin = np.isfinite(ref)
    assert np.max(np.abs(got[fin] - ref[fin])) <= 1e-13 * np.max(np.abs(ref[fin]))
