"""gemm_batch through the Ozaki form (GB_BATCH_FP64_OZAKI): three grouped
launches for all problems.  Level sums are exact integers and the rounding is
the same, so every problem must match the single-problem Ozaki call and the
CPU model bit for bit, whatever the tiling; Inf/NaN operands send the batch to
the native grouped launch."""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import _lib, blas
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

FP64, FP32, FP64_OZAKI = 0, 1, 2
GROUPED, LOOP = 0, 1


class Prob(C.Structure):
    _fields_ = [("transa", C.c_int), ("transb", C.c_int), ("m", C.c_int64), ("n", C.c_int64),
                ("k", C.c_int64), ("alpha", C.c_double), ("beta", C.c_double), ("a", C.c_void_p),
                ("lda", C.c_int64), ("b", C.c_void_p), ("ldb", C.c_int64), ("c", C.c_void_p),
                ("ldc", C.c_int64)]


def _shapes(seed, count, extra=()):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m, n, k = (int(round(np.exp(rng.uniform(0.0, np.log(400.0))))) for _ in range(3))
        out.append((m, n, k, int(rng.integers(2)), int(rng.integers(2)),
                    float(rng.choice([1.0, -0.5, 2.0])), float(rng.choice([0.0, 0.5]))))
    return out + list(extra)


class Batch:
    """Column-major device operands for a list of (m, n, k, ta, tb, alpha, beta)."""

    def __init__(self, shapes, seed):
        import torch
        self.torch = torch
        self.shapes = shapes
        self.host = []
        self.dev = []
        for i, (m, n, k, ta, tb, al, be) in enumerate(shapes):
            a = po.expspread((k, m) if ta else (m, k), seed + 3 * i, -10, 10)
            b = po.expspread((n, k) if tb else (k, n), seed + 3 * i + 1, -10, 10)
            c = po.uniform((m, n), seed + 3 * i + 2)
            self.host.append((a, b, c))
            self.dev.append(tuple(self._to_dev(x) for x in (a, b, c)))
        self.reset()

    def _to_dev(self, x):
        # column-major storage: the transpose of a row-major torch tensor
        return self.torch.from_numpy(np.ascontiguousarray(x.T)).cuda()

    def reset(self):
        for (a, b, c), (_, _, cd) in zip(self.host, self.dev):
            cd.copy_(self.torch.from_numpy(np.ascontiguousarray(c.T)))

    def problems(self):
        ps = (Prob * len(self.shapes))()
        for i, ((m, n, k, ta, tb, al, be), (a, b, c)) in enumerate(zip(self.shapes, self.dev)):
            ps[i] = Prob(8 * ta, 8 * tb, m, n, k, al, be, a.data_ptr(), max(1, a.shape[1]), b.data_ptr(),
                         max(1, b.shape[1]), c.data_ptr(), max(1, m))
        return ps

    def results(self):
        self.torch.cuda.synchronize()
        return [cd.cpu().numpy().T.copy() for (_, _, cd) in self.dev]


def _run_batch(gblib, batch, dtype, mode):
    batch.reset()
    ps = batch.problems()
    assert gblib.gb_gemm_batch_dev(C.addressof(ps), len(ps), dtype, mode, None) == 0
    return batch.results()


def _single_ozaki(gblib, batch, slices):
    batch.reset()
    for (m, n, k, ta, tb, al, be), (a, b, c) in zip(batch.shapes, batch.dev):
        if m == 0 or n == 0:
            continue
        rc = gblib.gb_dgemm_ozaki_dev(8 * ta, 8 * tb, m, n, k, al, a.data_ptr(), 1, max(1, a.shape[1]),
                                      b.data_ptr(), 1, max(1, b.shape[1]), be, c.data_ptr(), 1, max(1, m),
                                      slices, None)
        assert rc == 0
    return batch.results()


@pytest.mark.parametrize("slices", [5, 8])
def test_grouped_ozaki_bit_identical_to_single_calls_and_model(gblib, slices):
    # k = 0, alpha = 0 and m = 0 problems; k = 17000 exceeds one exact part at 8 slices; tall C
    # (fewer tiles as C^T: the grouped form runs op(B)^T op(A)^T, a partial last column half)
    extra = [(7, 9, 0, 0, 0, 1.0, 0.5), (5, 4, 30, 1, 0, 0.0, 0.5), (0, 3, 5, 0, 0, 1.0, 0.0),
             (5, 6, 17000, 0, 1, 1.0, 0.0), (300, 260, 1024, 1, 1, 1.0, 0.0),
             (1000, 40, 300, 1, 0, -0.5, 0.5), (600, 129, 70, 0, 1, 1.0, 0.0)]
    batch = Batch(_shapes(11, 40, extra), 1000)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, slices)
    try:
        grouped = _run_batch(gblib, batch, FP64_OZAKI, GROUPED)
        loop = _run_batch(gblib, batch, FP64_OZAKI, LOOP)
        single = _single_ozaki(gblib, batch, slices)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    for i, (g, l, s) in enumerate(zip(grouped, loop, single)):
        assert np.array_equal(g, s), i
        assert np.array_equal(l, s), i
    # the CPU model of the same arithmetic, on a subset (it is a scalar loop)
    for i in list(range(0, 40, 7)) + [41, 43, 44, 45, 46]:
        m, n, k, ta, tb, al, be = batch.shapes[i]
        a, b, c = batch.host[i]
        ref = np.asfortranarray(c.copy())
        po.ozaki_dgemm(8 * ta, 8 * tb, al, a, b, be, ref, slices)
        assert np.array_equal(grouped[i], ref), i


def test_grouped_ozaki_plan_graph_replay(gblib):
    batch = Batch(_shapes(12, 64), 2000)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    try:
        first = _run_batch(gblib, batch, FP64_OZAKI, GROUPED)
        ps = batch.problems()
        plan = C.c_void_p()
        assert gblib.gb_batch_plan_create(C.addressof(ps), len(ps), FP64_OZAKI, C.byref(plan)) == 0
        try:
            for use_graph in (1, 1, 0, 1):
                batch.reset()
                assert gblib.gb_batch_plan_run(plan, use_graph, None) == 0
                assert gblib.gb_synchronize() == 0
                for f, r in zip(first, batch.results()):
                    assert np.array_equal(f, r)
        finally:
            gblib.gb_batch_plan_destroy(plan)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def test_grouped_ozaki_nonfinite_goes_native(gblib):
    batch = Batch(_shapes(13, 24), 3000)
    a0 = batch.dev[5][0]
    a0.view(-1)[3] = float("inf")
    batch.host[5][0].reshape(-1, order="F")[3] = np.inf
    native = _run_batch(gblib, batch, FP64, GROUPED)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 6)
    try:
        oz = _run_batch(gblib, batch, FP64_OZAKI, GROUPED)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    assert _lib.last_error()[0] == 0
    for x, y in zip(native, oz):
        assert np.array_equal(x, y, equal_nan=True)
    assert not np.isfinite(oz[5]).all()


def test_dgemm_batch_blas_follows_ozaki_mode(gblib):
    shapes = _shapes(14, 12)
    rng = np.random.default_rng(4)
    data = []
    for (m, n, k, ta, tb, al, be) in shapes:
        a = po.expspread((k, m) if ta else (m, k), int(rng.integers(1 << 30)), -8, 8)
        b = po.expspread((n, k) if tb else (k, n), int(rng.integers(1 << 30)), -8, 8)
        c = po.uniform((m, n), int(rng.integers(1 << 30)))
        data.append((a, b, c))
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 7)
    try:
        cs = [np.asfortranarray(c.copy()) for (_, _, c) in data]
        blas.dgemm_batch(["T" if s[3] else "N" for s in shapes], ["T" if s[4] else "N" for s in shapes],
                         [s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes],
                         [s[5] for s in shapes], [d[0] for d in data], [d[0].shape[0] for d in data],
                         [d[1] for d in data], [d[1].shape[0] for d in data], [s[6] for s in shapes], cs,
                         [s[0] for s in shapes], [1] * len(shapes))
        # the CPU model of the Ozaki form (not dgemm_: it sends m == 1 or n == 1 to gemv,
        # frame/compat/bla_gemm.c:180-218, while the batch path runs every problem as a gemm,
        # frame/compat/extra/bla_gemm_batch.c:227)
        for (m, n, k, ta, tb, al, be), (a, b, c), got in zip(shapes, data, cs):
            ref = np.asfortranarray(c.copy())
            po.ozaki_dgemm(8 * ta, 8 * tb, al, a, b, be, ref, 7)
            assert np.array_equal(got, ref)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def test_grouped_ozaki_only_trivial_problems(gblib):
    # nothing for the grouped launches: k = 0 and alpha = 0 only, C := beta C
    batch = Batch([(4, 5, 0, 0, 0, 1.0, 0.5), (3, 3, 7, 1, 1, 0.0, 2.0)], 4000)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 0)
    try:
        got = _run_batch(gblib, batch, FP64_OZAKI, GROUPED)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    assert np.array_equal(got[0], 0.5 * batch.host[0][2])
    assert np.array_equal(got[1], 2.0 * batch.host[1][2])
