"""DTRSM (recursive blocked solve on the GPU) and grouped gemm_batch."""
import ctypes as C

import numpy as np
import pytest

from blis_gb300 import _lib, blas
from oracle import pyoracle as po
from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def native(gblib):
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    yield
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)


def _tri(a, uplo, diag):
    t = np.tril(a) if uplo == "L" else np.triu(a)
    if diag == "U":
        t = t - np.diag(np.diag(t)) + np.eye(a.shape[0])
    return t


@pytest.mark.parametrize("side", ["L", "R"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("diag", ["N", "U"])
@pytest.mark.parametrize("m,n", [(300, 200), (65, 1), (1, 7), (257, 129)])
def test_dtrsm_testsuite_residual(side, uplo, trans, diag, m, n):
    na = m if side == "L" else n
    a = np.asfortranarray(H.normalize(po.uniform((na, na), 4)) + 2.0 * np.eye(na))
    b0 = H.normalize(po.uniform((m, n), 5))
    x = np.asfortranarray(b0.copy())
    blas.dtrsm(side, uplo, trans, diag, m, n, 2.0, a, na, x, m)
    tri = _tri(a, uplo, diag)
    r = H.trsm_residual(0 if side == "L" else 1, 2.0, tri.T if trans == "T" else tri, b0, x)
    assert r < 1e-13


def test_dtrsm_config_shape_reduced_and_ozaki():
    # config-2 style: L lower, non-unit, diagonal = m + |u|
    m, n = 1536, 512
    L = np.tril(po.uniform((m, m), 7))
    L[np.diag_indices(m)] = m + np.abs(np.diag(L))
    L = np.asfortranarray(L)
    b0 = po.uniform((m, n), 8)
    ref = np.asfortranarray(b0.copy())
    po.dtrsm(po.LEFT, po.LOWER, 0, 0, 1.0, L, ref)
    for mode, slices in ((blas.DGEMM_NATIVE, 8), (blas.DGEMM_OZAKI, 8)):
        blas.set_dgemm_mode(mode, slices)
        x = np.asfortranarray(b0.copy())
        blas.dtrsm("L", "L", "N", "N", m, n, 1.0, L, m, x, m)
        assert np.max(np.abs(x - ref)) <= 1e-13 * np.max(np.abs(ref))


def test_dtrsm_alpha_zero():
    a = np.eye(5)
    b = np.full((5, 3), np.nan, order="F")
    blas.dtrsm("L", "L", "N", "N", 5, 3, 0.0, a, 5, b, 5)
    assert (b == 0).all()


def _problems(seed, count, dtype):
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(count):
        m, n, k = (int(round(np.exp(rng.uniform(np.log(16), np.log(300))))) for _ in range(3))
        ta, tb = rng.integers(0, 2, 2)
        a = po.uniform((k, m) if ta else (m, k), int(rng.integers(1 << 30)), dtype=dtype)
        b = po.uniform((n, k) if tb else (k, n), int(rng.integers(1 << 30)), dtype=dtype)
        c = po.uniform((m, n), int(rng.integers(1 << 30)), dtype=dtype)
        probs.append(("T" if ta else "N", "T" if tb else "N", m, n, k, a, b, c))
    return probs


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gemm_batch_blas_vs_oracle(dtype):
    probs = _problems(3, 40, dtype)
    # one group per problem, as the reference's batch test driver does
    ref = []
    for ta, tb, m, n, k, a, b, c in probs:
        r = np.asfortranarray(c.copy())
        po.dgemm(8 if ta == "T" else 0, 8 if tb == "T" else 0, 1.5, a, b, 0.5, r)
        ref.append(r)
    blas.dgemm_batch([p[0] for p in probs], [p[1] for p in probs], [p[2] for p in probs],
                     [p[3] for p in probs], [p[4] for p in probs], [1.5] * len(probs),
                     [p[5] for p in probs], [p[5].shape[0] for p in probs], [p[6] for p in probs],
                     [p[6].shape[0] for p in probs], [0.5] * len(probs), [p[7] for p in probs],
                     [p[2] for p in probs], [1] * len(probs), dtype=dtype)
    tol = 1e-12 if dtype == np.float64 else 2e-4
    for (ta, tb, m, n, k, a, b, c), r in zip(probs, ref):
        assert np.allclose(c, r, rtol=tol, atol=tol)


def test_grouped_equals_loop_and_graph_replay(gblib):
    torch = pytest.importorskip("torch")
    probs = _problems(5, 64, np.float64)
    tens = []
    descs = (_lib_problem * len(probs))()
    outs = []
    for i, (ta, tb, m, n, k, a, b, c) in enumerate(probs):
        A = torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()
        B = torch.from_numpy(np.asfortranarray(b).T.copy()).cuda()
        Cg = torch.from_numpy(np.asfortranarray(c).T.copy()).cuda()
        tens += [A, B, Cg]
        outs.append(Cg)
        descs[i] = _lib_problem(8 if ta == "T" else 0, 8 if tb == "T" else 0, m, n, k, 1.0, 0.0,
                                A.data_ptr(), a.shape[0], B.data_ptr(), b.shape[0], Cg.data_ptr(), m)
    L = _lib.load()
    L.gb_gemm_batch_dev.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_void_p]
    assert L.gb_gemm_batch_dev(C.addressof(descs), len(probs), 0, 0, None) == 0
    torch.cuda.synchronize()
    grouped = [o.clone() for o in outs]
    for o in outs:
        o.zero_()
    assert L.gb_gemm_batch_dev(C.addressof(descs), len(probs), 0, 1, None) == 0
    torch.cuda.synchronize()
    for g, o in zip(grouped, outs):
        assert torch.equal(g, o)
    plan = C.c_void_p()
    L.gb_batch_plan_create_ex.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    L.gb_batch_plan_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.gb_batch_plan_destroy.argtypes = [C.c_void_p]
    # policy 0 (every problem on the 128 x 128 engine, as the one-shot grouped call): an
    # autotuned plan may keep another policy, whose tiles sum in another order
    assert L.gb_batch_plan_create_ex(C.addressof(descs), len(probs), 0, 0, C.byref(plan)) == 0
    for _ in range(3):
        for o in outs:
            o.zero_()
        assert L.gb_batch_plan_run(plan, 1, None) == 0
        assert L.gb_synchronize() == 0
        for g, o in zip(grouped, outs):
            assert torch.equal(g, o)
    L.gb_batch_plan_destroy(plan)
    for (ta, tb, m, n, k, a, b, c), g in zip(probs, grouped):
        ref = np.zeros((m, n), order="F")
        po.dgemm(8 if ta == "T" else 0, 8 if tb == "T" else 0, 1.0, a, b, 0.0, ref)
        assert np.allclose(g.cpu().numpy().T, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("with_inf", [False, True])
def test_fp32_plan_split_form_edge_cases(gblib, with_inf):
    """FP32 plans through the split form (policy 3): larger problems, beta != 0,
    alpha = 0 over NaN operands, k = 0, m = 0, a k past the grouped form's range,
    with and without an Inf in op(A); the autotuned plan
    may pick the split form, and pinning SGEMM to the FP32 pipe takes policy 3
    out of its candidates."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    shapes = [(1100, 900, 1300, 1.0, 0.0), (700, 1024, 1500, -0.75, 0.5), (64, 48, 0, 1.0, 0.5),
              (0, 40, 30, 1.0, 0.0), (200, 100, 300, 0.0, 0.5), (300, 200, 250, 1.0, 0.0),
              (33, 17, 1000, 2.0, -1.0), (9, 12, 50000, 1.0, 0.25)]  # k past the grouped form: alone
    probs = []
    for i, (m, n, k, alpha, beta) in enumerate(shapes):
        ta, tb = int(rng.integers(0, 2)), int(rng.integers(0, 2))
        a = po.uniform((k, m) if ta else (m, k), 300 + i, dtype=np.float32)
        b = po.uniform((n, k) if tb else (k, n), 400 + i, dtype=np.float32)
        c = po.uniform((m, n), 500 + i, dtype=np.float32)
        if alpha == 0.0:
            a[:] = np.nan  # not read when alpha = 0
        if i == 5 and with_inf:
            a[3, 7] = np.inf  # the whole grouped part then runs on the FP32 pipe
        probs.append((ta, tb, m, n, k, alpha, beta, a, b, c))
    L = _lib.load()
    L.gb_batch_plan_create_ex.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    L.gb_batch_plan_run.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.gb_batch_plan_destroy.argtypes = [C.c_void_p]
    L.gb_batch_plan_policy.argtypes = [C.c_void_p]

    def run(policy):
        descs = (_lib_problem * len(probs))()
        keep, outs = [], []
        for i, (ta, tb, m, n, k, alpha, beta, a, b, c) in enumerate(probs):
            A = torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()
            B = torch.from_numpy(np.asfortranarray(b).T.copy()).cuda()
            Cg = torch.from_numpy(np.asfortranarray(c).T.copy()).cuda()
            keep += [A, B]
            outs.append(Cg)
            descs[i] = _lib_problem(8 * ta, 8 * tb, m, n, k, alpha, beta, A.data_ptr(), max(a.shape[0], 1),
                                    B.data_ptr(), max(b.shape[0], 1), Cg.data_ptr(), max(m, 1))
        torch.cuda.synchronize()
        plan = C.c_void_p()
        assert L.gb_batch_plan_create_ex(C.addressof(descs), len(probs), 1, policy, C.byref(plan)) == 0
        got_policy = L.gb_batch_plan_policy(plan)
        assert L.gb_batch_plan_run(plan, 1, None) == 0
        assert L.gb_synchronize() == 0
        L.gb_batch_plan_destroy(plan)
        return got_policy, [o.cpu().numpy().T for o in outs]

    pol3, res3 = run(3)
    assert pol3 == 3
    polt, rest = run(-1)
    assert polt in (0, 1, 2, 3)  # 1 and 2 when a selector model is in use
    assert gblib.gb_set_sgemm_mode(0) == 0  # GB_SGEMM_FMA
    try:
        pol0, res0 = run(-1)
    finally:
        assert gblib.gb_set_sgemm_mode(2) == 0  # GB_SGEMM_AUTO
    assert pol0 in (0, 1, 2)
    u = 2.0 ** -24
    for (ta, tb, m, n, k, alpha, beta, a, b, c), g3, gt, g0 in zip(probs, res3, rest, res0):
        A = (a.T if ta else a).astype(np.float64)
        B = (b.T if tb else b).astype(np.float64)
        c64 = c.astype(np.float64)
        if alpha == 0.0:
            ref, bound = beta * c64, np.abs(beta * c64) * u
        else:
            with np.errstate(invalid="ignore"):
                ref = alpha * (A @ B) + beta * c64
                bound = 2 * (k + 2) * u * (abs(alpha) * (np.abs(A) @ np.abs(B)) + abs(beta) * np.abs(c64))
        fin = np.isfinite(ref)
        for g in (g3, gt, g0):
            g = g.astype(np.float64)
            assert np.array_equal(np.isnan(g), np.isnan(ref)) and np.array_equal(np.isinf(g), np.isinf(ref))
            assert np.array_equal(g[~fin & ~np.isnan(ref)], ref[~fin & ~np.isnan(ref)])
            assert np.all(np.abs(g[fin] - ref[fin]) <= bound[fin])


def test_fp32_plan_split_form_bit_identical_to_sgemm_split(gblib):
    """Policy 3 runs every problem through the grouped Ozaki form on the FP32
    operands: per problem the same bits as the single-problem SGEMM split form
    (gb_sgemm_dev with GB_SGEMM_SPLIT), whatever the transposes, alpha, beta."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    probs = []
    for i in range(40):
        m, n, k = (int(round(np.exp(rng.uniform(np.log(8), np.log(700))))) for _ in range(3))
        ta, tb = (int(v) for v in rng.integers(0, 2, 2))
        alpha, beta = [(1.0, 0.0), (1.25, -0.5), (-2.0, 1.0), (0.5, 0.0)][i % 4]
        a = po.expspread((k, m) if ta else (m, k), 600 + i, -12, 12).astype(np.float32)
        b = po.expspread((n, k) if tb else (k, n), 700 + i, -12, 12).astype(np.float32)
        c = po.uniform((m, n), 800 + i, dtype=np.float32)
        probs.append((ta, tb, m, n, k, alpha, beta, a, b, c))
    L = _lib.load()
    dev = lambda x: torch.from_numpy(np.asfortranarray(x).T.copy()).cuda()
    descs = (_lib_problem * len(probs))()
    keep, outs, singles = [], [], []
    for i, (ta, tb, m, n, k, alpha, beta, a, b, c) in enumerate(probs):
        A, B, Cg, Cs = dev(a), dev(b), dev(c), dev(c)
        keep += [A, B]
        outs.append(Cg)
        singles.append(Cs)
        descs[i] = _lib_problem(8 * ta, 8 * tb, m, n, k, alpha, beta, A.data_ptr(), a.shape[0], B.data_ptr(),
                                b.shape[0], Cg.data_ptr(), m)
        assert gblib.gb_set_sgemm_mode(1) == 0  # GB_SGEMM_SPLIT
        try:
            assert L.gb_sgemm_dev(8 * ta, 8 * tb, m, n, k, alpha, A.data_ptr(), 1, a.shape[0], B.data_ptr(), 1,
                                  b.shape[0], beta, Cs.data_ptr(), 1, m, None) == 0
        finally:
            assert gblib.gb_set_sgemm_mode(2) == 0
    assert L.gb_synchronize() == 0
    torch.cuda.synchronize()
    plan = C.c_void_p()
    assert L.gb_batch_plan_create_ex(C.addressof(descs), len(probs), 1, 3, C.byref(plan)) == 0
    try:
        assert L.gb_batch_plan_run(plan, 1, None) == 0
        assert L.gb_synchronize() == 0
    finally:
        L.gb_batch_plan_destroy(plan)
    # and the CPU model of the same arithmetic: P by the digit form at 3 slices on the widened
    # operands, C = RN32(alpha P + beta C) (these alpha and beta make each step one rounding)
    bad_batch, bad_single = [], []
    for i, ((ta, tb, m, n, k, alpha, beta, a, b, c), g, r) in enumerate(zip(probs, outs, singles)):
        P = np.zeros((m, n), order="F")
        po.ozaki_dgemm(8 * ta, 8 * tb, 1.0, np.asfortranarray(a, dtype=np.float64),
                       np.asfortranarray(b, dtype=np.float64), 0.0, P, 3)
        t = alpha * P
        ref = (t if beta == 0.0 else beta * c.astype(np.float64) + t).astype(np.float32)
        if not np.array_equal(g.cpu().numpy().T, ref):
            bad_batch.append(i)
        if not np.array_equal(r.cpu().numpy().T, ref):
            bad_single.append(i)
    assert not bad_batch and not bad_single, (bad_batch, bad_single)
    for i, (g, r) in enumerate(zip(outs, singles)):
        assert torch.equal(g, r), i


class _lib_problem(C.Structure):
    _fields_ = [("transa", C.c_int), ("transb", C.c_int), ("m", C.c_int64), ("n", C.c_int64),
                ("k", C.c_int64), ("alpha", C.c_double), ("beta", C.c_double), ("a", C.c_void_p),
                ("lda", C.c_int64), ("b", C.c_void_p), ("ldb", C.c_int64), ("c", C.c_void_p),
                ("ldc", C.c_int64)]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_batch_with_selected_configs(gblib, dtype):
    """With the trained selector loaded, each problem of a batch gets its own
    configuration (128 x 128 grouped launch, or the grouped 64 x 64 engine with
    split-K and the grouped fold); results meet the testsuite residual, repeat
    bit for bit under graph replay, and some problems take each class."""
    torch = pytest.importorskip("torch")
    from blis_gb300 import selector as S
    rng = np.random.default_rng(9)
    probs = []
    for i in range(96):
        m, n = (int(rng.integers(8, 400)) for _ in range(2))
        k = int(rng.integers(8, 3000)) if i % 3 else 6000  # long k: split-K candidates
        if i % 24 == 0:
            m, n, k = 2048, 1536, 512  # large: the 128 x 128 engine's territory
        ta, tb = rng.integers(0, 2, 2)
        a = po.uniform((k, m) if ta else (m, k), 100 + 3 * i, dtype=dtype)
        b = po.uniform((n, k) if tb else (k, n), 101 + 3 * i, dtype=dtype)
        c = po.uniform((m, n), 102 + 3 * i, dtype=dtype)
        probs.append(("T" if ta else "N", "T" if tb else "N", m, n, k, a, b, c))
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    descs = (_lib_problem * len(probs))()
    keep, outs = [], []
    for i, (ta, tb, m, n, k, a, b, c) in enumerate(probs):
        A = torch.from_numpy(np.asfortranarray(a).T.copy()).cuda()
        B = torch.from_numpy(np.asfortranarray(b).T.copy()).cuda()
        Cg = torch.from_numpy(np.asfortranarray(c).T.copy()).cuda()
        keep += [A, B]
        outs.append(Cg)
        descs[i] = _lib_problem(8 if ta == "T" else 0, 8 if tb == "T" else 0, m, n, k, 1.25, -0.5, A.data_ptr(),
                                a.shape[0], B.data_ptr(), b.shape[0], Cg.data_ptr(), m)
    L = _lib.load()
    code = 0 if dtype == np.float64 else 1
    S.load_into_library()
    try:
        cfgs = []
        for (ta, tb, m, n, k, a, b, c) in probs:
            cfg, sl = C.c_int(), C.c_int()
            assert gblib.gb_selector_choose(code, m, n, k, int(ta == "T"), int(tb == "T"), 0, 0.0, 0.0,
                                            C.byref(cfg), C.byref(sl)) == 0
            cfgs.append(cfg.value)
        assert any(v >= 1 for v in cfgs)  # the grouped 64 x 64 launch is exercised
        c0 = [o.clone() for o in outs]
        results = {}
        # fixed policies (3: FP32 through SGEMM's split form), then the plan's own autotuning
        policies = (1, 2, 3, -1) if code == 1 else (1, 2, -1)
        for policy in policies:
            plan = C.c_void_p()
            assert L.gb_batch_plan_create_ex(C.addressof(descs), len(probs), code, policy, C.byref(plan)) == 0
            assert L.gb_batch_plan_policy(plan) in (((0, 1, 2, 3) if code == 1 else (0, 1, 2)) if policy < 0
                                                    else (policy,))
            first = None
            for rep in range(3):
                for o, z in zip(outs, c0):
                    o.copy_(z)
                torch.cuda.synchronize()  # the plan runs on the library's stream, not torch's
                assert L.gb_batch_plan_run(plan, 1, None) == 0
                assert L.gb_synchronize() == 0
                got = [o.clone() for o in outs]
                if first is None:
                    first = got
                else:
                    assert all(torch.equal(x, y) for x, y in zip(first, got))
            L.gb_batch_plan_destroy(plan)
            results[policy] = first
        # the autotuning ran the batch on scratch outputs: C itself was only written by the runs above
    finally:
        gblib.gb_set_gemm_autoselect(0)
        gblib.gb_selector_unload()
    # componentwise: |C - C_ref| <= 2 k u (|alpha| |A| |B| + |beta| |C0|) (operands are not
    # normalized as in the testsuite, so its absolute residual does not apply)
    u = 2.0 ** -53 if dtype == np.float64 else 2.0 ** -24
    checked = [results[1], results[2]] + ([results[3]] if code == 1 else [])
    for idx, (ta, tb, m, n, k, a, b, c) in enumerate(probs):
        A = H.op(a, 8 if ta == "T" else 0).astype(np.float64)
        B = H.op(b, 8 if tb == "T" else 0).astype(np.float64)
        ref = 1.25 * (A @ B) - 0.5 * c.astype(np.float64)
        bound = 2 * (k + 2) * u * (1.25 * (np.abs(A) @ np.abs(B)) + 0.5 * np.abs(c.astype(np.float64)))
        for res in checked:
            assert np.all(np.abs(res[idx].cpu().numpy().T.astype(np.float64) - ref) <= bound)


@pytest.mark.parametrize("n", [300, 20000, 40000, 120000])
@pytest.mark.parametrize("uplo,trans", [("L", "N"), ("U", "N"), ("L", "T")])
def test_dtrsm_many_right_hand_sides(uplo, trans, n):
    # on 152 SMs these n take the diagonal kernel with 8, 4, 2 and 1 lanes per right-hand side
    m = 200  # three full 64-row diagonal blocks and one of 8 rows
    a = np.asfortranarray(H.normalize(po.uniform((m, m), 14)) + 2.0 * np.eye(m))
    b0 = H.normalize(po.uniform((m, n), 15))
    x = np.asfortranarray(b0.copy())
    blas.dtrsm("L", uplo, trans, "N", m, n, 1.5, a, m, x, m)
    tri = _tri(a, uplo, "N")
    r = H.trsm_residual(0, 1.5, tri.T if trans == "T" else tri, b0, x)
    assert r < 1e-12


@pytest.mark.parametrize("side,uplo,trans", [("L", "L", "N"), ("L", "U", "T"), ("R", "U", "N"), ("R", "L", "T")])
def test_dtrsm_ozaki_two_column_groups(side, uplo, trans):
    # the precision form with at least 2048 right-hand sides solves two column
    # halves on two streams; every column must still match the oracle
    m, n = 700, 2600
    rows, cols = (m, n) if side == "L" else (n, m)
    na = m if side == "L" else m
    a = np.asfortranarray(H.normalize(po.uniform((na, na), 16)) + 2.0 * np.eye(na))
    b0 = H.normalize(po.uniform((rows, cols), 17))
    ref = np.asfortranarray(b0.copy())
    po.dtrsm(po.LEFT if side == "L" else po.RIGHT, po.LOWER if uplo == "L" else po.UPPER, 8 if trans == "T" else 0,
             po.NONUNIT_DIAG, -0.5, a, ref)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI, 8)
    try:
        x = np.asfortranarray(b0.copy())
        blas.dtrsm(side, uplo, trans, "N", rows, cols, -0.5, a, na, x, rows)
    finally:
        blas.set_dgemm_mode(blas.DGEMM_NATIVE, 8)
    tri = _tri(a, uplo, "N")
    r = H.trsm_residual(0 if side == "L" else 1, -0.5, tri.T if trans == "T" else tri, b0, x)
    assert r < 1e-12
    assert np.max(np.abs(x - ref)) <= 1e-12 * np.max(np.abs(ref))
