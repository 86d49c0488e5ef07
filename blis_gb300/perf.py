"""Throughput of the hot path's other configurations on one GPU.

bench.py measures the headline (emulated vs native DGEMM 16384^3); this
module measures the remaining workloads of the same path, device resident,
with CUDA events on the launching stream after warm-up, inputs larger than
L2 where the workload allows:

  dgemm_1024      C := A B + 0.5 C, m=n=k=1024, U[-1,1]          (FP64 pipe)
  dgemm_8192      native FP64 and Ozaki (7 slices), m=n=k=8192
  sgemm_8192      FP32, m=n=k=8192
  bgemm_8192      BF16 A, B, FP32 C, m=n=k=8192 (tensor cores)
  dtrsm_8192x4096 L/L/N/N, diag 8192+|u|, native and Ozaki updates (m^2 n flop)
  dgemv_32768     N and T, 8(mn + n + 2m) bytes                    (HBM)
  daxpyv_2^28     24 n bytes; ddotv_2^28: 16 n bytes                (HBM)
  dtrsm_16384     L/L/N/N, B entries (1+u) 2^e, e in [-20,20]: native and
                  Ozaki updates, sampled componentwise backward error
  level12x        dscal / dcopy / idamax at 2^28, dger 32768^2, dtrsv 16384
  complex         zgemm 4096^3 native / Ozaki, cgemm 4096^3 (8 mnk flop), ztrsm / ctrsm 4096^2,
                  zgemv / cgemv 16384^2
                  native / Ozaki updates (4 m^2 n flop)
  level3x         dtrmm 8192x4096 (m^2 n), dsyrk n=k=8192 (n^2 k), dsymm
                  8192x4096 (2 m^2 n): native FP64 and Ozaki (7 slices)
  batch_4096      4096 problems, m,n,k log-uniform in [16,1024], random
                  transposes: grouped launches (captured graph) vs a
                  per-problem launch loop, FP64 native, FP64 Ozaki (7
                  slices) and FP32
  e2e             dgemm_ 16384^3 (4096^3 with --small) in the CRT form (16
                  moduli) on pinned host buffers, per call: host time and
                  the timeline of its launches and copies (gb_kernel_trace)
                  for the fastest and the slowest of the calls

Usage: python -m blis_gb300.perf [--only name,...] [--json out.jsonl] [--batch-count N] [--small]
                                [--trsm-forms native,ozaki] [--forms native,ozaki]
(--small: 4096^3 GEMMs, 2048 x 10240 DTRSM, 2^25 vectors, 8192^2 GEMV, 4096-row level-3 extras,
for ncu captures)
"""
import argparse
import ctypes as C
import json
import math
import os

import numpy as np

from . import _lib, blas, dev

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = False  # --small: profiling sizes (inputs still larger than the 126 MB L2)
TRSM_FORMS = ("native", "ozaki")  # --trsm-forms: which DTRSM forms the trsm suites time
FORMS = ("native", "ozaki")  # --forms: which forms the level3x, hermitian and complex suites time
CRT_N = 0  # --crt-n: size of the crt suite's product (0: 16384, or 4096 with --small)


def _forms(pairs):
    """The (mode, name) pairs of the forms selected by --forms (mode 0 native, 1 Ozaki)."""
    return tuple(f for f in pairs if ("ozaki" if f[0] else "native") in FORMS)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream or 1)


def _timer(fn, reps=5, warmup=2):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def _mat(m, n, kind=dev.RAND_UNIFORM, seed=1, p0=-1.0, p1=1.0, dtype=None):
    import torch
    x = dev.colmajor(m, n, dtype or torch.float64)
    dev.randm(x, kind, seed, p0, p1)
    return x


def run_gemm(out):
    import torch
    pk, _ = peaks()
    a, b, c = _mat(1024, 1024, seed=1), _mat(1024, 1024, seed=2), _mat(1024, 1024, seed=3)
    ms = _timer(lambda: dev.dgemm(0, 0, 1.0, a, b, 0.5, c), reps=20)
    out.append({"workload": "dgemm_1024", "form": "native_fp64", "ms": ms, "tflops": 2 * 1024 ** 3 / ms / 1e9})
    n = 4096 if SMALL else 8192
    a, b, c = _mat(n, n, seed=4), _mat(n, n, seed=5), _mat(n, n, seed=6)
    ms = _timer(lambda: dev.dgemm(0, 0, 1.0, a, b, 0.0, c), reps=1, warmup=1)
    out.append({"workload": "dgemm_%d" % n, "form": "native_fp64", "ms": ms, "tflops": 2 * n ** 3 / ms / 1e9})
    ms = _timer(lambda: dev.dgemm_ozaki(0, 0, 1.0, a, b, 0.0, c, 7), reps=3)
    out.append({"workload": "dgemm_%d" % n, "form": "ozaki_s7", "ms": ms, "tflops": 2 * n ** 3 / ms / 1e9,
                "bf16_frac_of_measured_peak": 28 * 2 * n ** 3 / ms / 1e9 / pk.get("bf16_tflops", 1900.0)})
    ms = _timer(lambda: dev.dgemm_ozaki_crt(0, 0, 1.0, a, b, 0.0, c, 16), reps=3)
    out.append({"workload": "dgemm_%d" % n, "form": "ozaki_crt16", "ms": ms, "tflops": 2 * n ** 3 / ms / 1e9,
                "bf16_frac_of_measured_peak": 16 * 2 * n ** 3 / ms / 1e9 / pk.get("bf16_tflops", 1900.0)})
    del a, b, c
    fa, fb, fc = (_mat(n, n, seed=s, dtype=torch.float32) for s in (7, 8, 9))
    ms = _timer(lambda: dev.sgemm(0, 0, 1.0, fa, fb, 0.0, fc), reps=3)
    out.append({"workload": "sgemm_%d" % n, "form": "default_dispatch", "ms": ms, "tflops": 2 * n ** 3 / ms / 1e9})


def run_sgemm(out):
    """SGEMM 8192^3 on both engines (FP32 FMA kernel, split form on the bf16 tensor cores):
    time, and the max componentwise error of 4096 sampled entries against the double-double
    product of the same FP32 operands, in units of the FP32 gauge u32 (|A||B|)_ij."""
    import torch
    n = 4096 if SMALL else 8192
    fa, fb, fc = (_mat(n, n, seed=s, dtype=torch.float32) for s in (7, 8, 9))
    g = torch.Generator(device="cpu").manual_seed(3)
    ii = torch.randint(0, n, (4096,), generator=g).cuda()
    jj = torch.randint(0, n, (4096,), generator=g).cuda()
    da, db = fa.double(), fb.double()
    hi, lo = dev.dd_gemm_entries(0, 0, 1.0, da, db, 0.0, None, ii, jj)
    gauge = (da[ii, :].abs() * db[:, jj].abs().t()).sum(1)
    u32 = 2.0 ** -24
    for mode, name in ((blas.SGEMM_FMA, "ffma_fp32"), (blas.SGEMM_SPLIT, "split_bf16_s3")):
        blas.set_sgemm_mode(mode)
        ms = _timer(lambda: dev.sgemm(0, 0, 1.0, fa, fb, 0.0, fc), reps=3)
        err = ((fc[ii, jj].double() - hi - lo).abs() / gauge).max().item() / u32
        rec = {"workload": "sgemm_%d" % n, "form": name, "ms": ms, "tflops": 2 * n ** 3 / ms / 1e9,
               "max_err_in_u32_gauge": err}
        if mode == blas.SGEMM_SPLIT:
            # device time of each stage (the library's own events), mean of three calls
            dev.set_kernel_timing(True)
            dev.kernel_trace()
            for _ in range(3):
                dev.sgemm(0, 0, 1.0, fa, fb, 0.0, fc)
            dev.synchronize()
            stages = {}
            for nm, t0, t1 in dev.kernel_trace():
                stages[nm] = stages.get(nm, 0.0) + (t1 - t0) / 3
            dev.set_kernel_timing(False)
            rec["stage_ms"] = {k: round(v, 4) for k, v in stages.items()}
        out.append(rec)
    blas.set_sgemm_mode(blas.SGEMM_AUTO)


def run_bgemm(out):
    """BF16 GEMM 8192^3 (fp32 C) on the tensor-core kernel: op(A) = A^T (k
    contiguous, loaded by TMA in place) and op(A) = A (packed to k-major
    first); against the measured cuBLAS bf16 peak."""
    import torch
    pk, kind = peaks()
    n = 4096 if SMALL else 8192
    a = _mat(n, n, seed=41).to(torch.bfloat16)
    b = _mat(n, n, seed=42).to(torch.bfloat16)
    a, b = a.t().contiguous().t(), b.t().contiguous().t()  # column-major bf16
    c = dev.colmajor(n, n, torch.float32)
    for ta, name in ((8, "TN_tma_in_place"), (0, "NN_packed")):
        ms = _timer(lambda: dev.bgemm(ta, 0, 1.0, a, b, 0.0, c, config=0), reps=5)
        tf = 2 * n ** 3 / ms / 1e9
        out.append({"workload": "bgemm_%d" % n, "form": name, "ms": ms, "tflops": tf,
                    "frac_of_bf16_burst": tf / pk.get("bf16_tflops", 1900.0), "peak": "%s bf16_tflops" % kind})


def run_trsm(out):
    import torch
    m, n = (2048, 10240) if SMALL else (8192, 4096)  # small: fewer rows, more right-hand sides
    L = _mat(m, m, seed=11)
    L.copy_(torch.tril(L))
    d = torch.arange(m, device="cuda")
    L[d, d] = m + L[d, d].abs()
    b0 = _mat(m, n, seed=12)
    flops = float(m) * m * n
    for mode, cnt, name in ((0, 7, "native_fp64"), (1, 7, "ozaki_s7_updates"), (2, 16, "ozaki_crt16_updates")):
        if ("ozaki" if mode else "native") not in TRSM_FORMS:
            continue
        _lib.load().gb_set_dgemm_mode(mode, cnt)
        x = b0.clone()
        ms = _timer(lambda: (x.copy_(b0), dev.dtrsm(0, 0xC0, 0, 0, 1.0, L, x)), reps=1, warmup=1)
        copy_ms = _timer(lambda: x.copy_(b0), reps=3, warmup=1)
        out.append({"workload": "dtrsm_%dx%d" % (m, n), "form": name, "ms": ms - copy_ms,
                    "tflops": flops / (ms - copy_ms) / 1e9})
    _lib.load().gb_set_dgemm_mode(0, 8)


def run_strsm(out):
    """STRSM L/L/N/N 8192 x 4096 in FP32 (m^2 n flop): the FP32 recursion, its updates through
    sgemm's engine choice (the split form at size), against the same solve with every update on
    the FP32 FMA kernel."""
    import torch
    m, n = (2048, 10240) if SMALL else (8192, 4096)
    L = _mat(m, m, seed=11, dtype=torch.float32)
    L.copy_(torch.tril(L))
    d = torch.arange(m, device="cuda")
    L[d, d] = m + L[d, d].abs()
    b0 = _mat(m, n, seed=12, dtype=torch.float32)
    flops = float(m) * m * n
    lib = _lib.load()
    for mode, name in ((blas.SGEMM_AUTO, "updates_default_dispatch"), (blas.SGEMM_FMA, "updates_ffma")):
        blas.set_sgemm_mode(mode)
        x = b0.clone()
        st = _stream()

        def call():
            x.copy_(b0)
            _lib.check(lib.gb_strsm_dev(0, 0xC0, 0, 0, m, n, 1.0, L.data_ptr(), 1, m, x.data_ptr(), 1, m, st),
                       "gb_strsm_dev")
        ms = _timer(call, reps=3, warmup=1)
        copy_ms = _timer(lambda: x.copy_(b0), reps=3, warmup=1)
        out.append({"workload": "strsm_%dx%d" % (m, n), "form": name, "ms": ms - copy_ms,
                    "tflops": flops / (ms - copy_ms) / 1e9})
    blas.set_sgemm_mode(blas.SGEMM_AUTO)


def run_trsm_ozaki(out):
    """DTRSM L/L/N/N m = n = 16384: L as above (diagonal 16384+|u|), B with
    entries (1+u) 2^e, e in [-20, 20].  Native FP64 and Ozaki off-diagonal
    updates (7 slices; FP64 diagonal-block solves), each with its sampled
    componentwise backward error |B - L X|_ij / (|L||X| + |B|)_ij, numerator
    and denominator evaluated in double-double on the device."""
    import torch
    m = n = 16384
    L = _mat(m, m, seed=31)
    L.copy_(torch.tril(L))
    d = torch.arange(m, device="cuda")
    L[d, d] = m + L[d, d].abs()
    b0 = _mat(m, n, kind=dev.RAND_EXPSPREAD, seed=32, p0=-20, p1=20)
    g = torch.Generator(device="cpu").manual_seed(5)
    ii = torch.randint(0, m, (4096,), generator=g).cuda()
    jj = torch.randint(0, n, (4096,), generator=g).cuda()
    absL, absB = L.abs(), b0.abs()
    flops = float(m) * m * n
    for mode, cnt, name in ((0, 7, "native_fp64"), (1, 7, "ozaki_s7_updates"), (2, 16, "ozaki_crt16_updates")):
        if ("ozaki" if mode else "native") not in TRSM_FORMS:
            continue
        _lib.load().gb_set_dgemm_mode(mode, cnt)
        x = b0.clone()
        reps = 1 if mode == 0 else 3
        ms = _timer(lambda: (x.copy_(b0), dev.dtrsm(0, 0xC0, 0, 0, 1.0, L, x)), reps=reps, warmup=1)
        copy_ms = _timer(lambda: x.copy_(b0), reps=3, warmup=1)
        x.copy_(b0)
        dev.dtrsm(0, 0xC0, 0, 0, 1.0, L, x)
        rh, rl = dev.dd_gemm_entries(0, 0, 1.0, L, x, -1.0, b0, ii, jj)
        dh, dl = dev.dd_gemm_entries(0, 0, 1.0, absL, x.abs(), 1.0, absB, ii, jj)
        berr = float(((rh + rl).abs() / (dh + dl)).max())
        out.append({"workload": "dtrsm_16384x16384_expspread", "form": name, "ms": ms - copy_ms,
                    "tflops": flops / (ms - copy_ms) / 1e9, "max_componentwise_backward_err": berr,
                    "err_sample": "4096 random entries, double-double on the device"})
        del x
    _lib.load().gb_set_dgemm_mode(0, 8)


def run_level12(out):
    import torch
    pk, kind = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    n = 1 << (25 if SMALL else 28)
    x = torch.empty(n, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    y = torch.empty(n, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    rho = torch.zeros(1, dtype=torch.float64, device="cuda")
    ms = _timer(lambda: dev.daxpyv(0.5, x, y), reps=10)
    gbs = 24.0 * n / ms / 1e6
    out.append({"workload": "daxpyv_%d" % n, "ms": ms, "gbs": gbs, "hbm_frac": gbs / hbm, "peak": "%s hbm_gbs" % kind})
    ms = _timer(lambda: dev.ddotv(x, y, rho), reps=10)
    gbs = 16.0 * n / ms / 1e6
    out.append({"workload": "ddotv_%d" % n, "ms": ms, "gbs": gbs, "hbm_frac": gbs / hbm, "peak": "%s hbm_gbs" % kind})
    del x, y
    m = 8192 if SMALL else 32768
    a = _mat(m, m, seed=21)
    xv = torch.empty(m, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    yv = torch.empty(m, dtype=torch.float64, device="cuda").uniform_(-1, 1)
    for t, name in ((0, "N"), (8, "T")):
        ms = _timer(lambda: dev.dgemv(t, 1.0, a, xv, 0.5, yv), reps=5)
        gbs = 8.0 * (m * m + m + 2 * m) / ms / 1e6
        out.append({"workload": "dgemv_%d_%s" % (m, name), "ms": ms, "gbs": gbs, "hbm_frac": gbs / hbm,
                    "peak": "%s hbm_gbs" % kind})


class _Prob(C.Structure):
    _fields_ = [("transa", C.c_int), ("transb", C.c_int), ("m", C.c_int64), ("n", C.c_int64),
                ("k", C.c_int64), ("alpha", C.c_double), ("beta", C.c_double), ("a", C.c_void_p),
                ("lda", C.c_int64), ("b", C.c_void_p), ("ldb", C.c_int64), ("c", C.c_void_p),
                ("ldc", C.c_int64)]


def batch_problems(count, seed, dtype, lo=16, hi=1024):
    """The batching configuration: m, n, k log-uniform integers in [lo, hi],
    transposes random per operand, U[-1,1] entries; operands packed in one
    device arena per operand kind."""
    import torch
    rng = np.random.default_rng(seed)
    dims = np.round(np.exp(rng.uniform(math.log(lo), math.log(hi), size=(count, 3)))).astype(np.int64)
    tr = rng.integers(0, 2, size=(count, 2))
    tdt = torch.float64 if dtype == 0 else torch.float32
    na = int((dims[:, 0] * dims[:, 2]).sum())
    nb = int((dims[:, 2] * dims[:, 1]).sum())
    nc = int((dims[:, 0] * dims[:, 1]).sum())
    A = torch.empty(na, dtype=tdt, device="cuda").uniform_(-1, 1)
    B = torch.empty(nb, dtype=tdt, device="cuda").uniform_(-1, 1)
    Cc = torch.zeros(nc, dtype=tdt, device="cuda")
    es = A.element_size()
    probs = (_Prob * count)()
    oa = ob = oc = 0
    flops = 0.0
    for i in range(count):
        m, n, k = (int(v) for v in dims[i])
        ta, tb = int(tr[i, 0]), int(tr[i, 1])
        probs[i] = _Prob(8 * ta, 8 * tb, m, n, k, 1.0, 0.0, A.data_ptr() + oa * es, k if ta else m,
                         B.data_ptr() + ob * es, n if tb else k, Cc.data_ptr() + oc * es, m)
        oa += m * k
        ob += k * n
        oc += m * n
        flops += 2.0 * m * n * k
    return probs, (A, B, Cc), flops


BATCH_COUNT = 4096


def run_batch_ozaki(out):
    """The grouped Ozaki batch alone (7 slices), BATCH_COUNT problems: plan
    replay time and per-stage device times from the library's own events."""
    L = _lib.load()
    L.gb_set_dgemm_mode(1, 7)
    probs, keep, flops = batch_problems(BATCH_COUNT, 4, 0)
    plan = C.c_void_p()
    _lib.check(L.gb_batch_plan_create(C.addressof(probs), BATCH_COUNT, 2, C.byref(plan)), "plan")
    st = _stream()
    ms = _timer(lambda: _lib.check(L.gb_batch_plan_run(plan, 1, st), "run"), reps=3, warmup=2)
    dev.set_kernel_timing(True)
    for _ in range(3):
        _lib.check(L.gb_batch_plan_run(plan, 0, st), "run")
    stages = {}
    for pre in ("oz_split_batch", "ozaki_slice_gemm_batch", "oz_recombine_batch", "batch_grouped_dmma_gated"):
        stages[pre] = dev.kernel_time_ms(pre)[0] / 3
    dev.set_kernel_timing(False)
    L.gb_batch_plan_destroy(plan)
    L.gb_set_dgemm_mode(0, 8)
    out.append({"workload": "batch_%d_fp64_ozaki_s7" % BATCH_COUNT, "flops": flops, "grouped_graph_ms": ms,
                "grouped_tflops": flops / ms / 1e9, "stage_ms": stages})
    del keep


def run_batch(out):
    import torch
    L = _lib.load()
    for dtype, name in ((0, "fp64"), (2, "fp64_ozaki_s7"), (1, "fp32")):
        if dtype == 2:
            L.gb_set_dgemm_mode(1, 7)
        probs, keep, flops = batch_problems(4096, 4, 1 if dtype == 1 else 0)
        plan = C.c_void_p()
        _lib.check(L.gb_batch_plan_create(C.addressof(probs), 4096, dtype, C.byref(plan)), "plan")
        st = _stream()  # the library works on the stream the events are recorded on
        ms_g = _timer(lambda: _lib.check(L.gb_batch_plan_run(plan, 1, st), "run"), reps=3, warmup=1)
        rec = {"workload": "batch_4096_%s" % name, "flops": flops, "grouped_graph_ms": ms_g,
               "grouped_tflops": flops / ms_g / 1e9}
        if dtype == 2:
            # against the native grouped launch on the same operands
            c_oz = keep[2].clone()
            L.gb_batch_plan_destroy(plan)
            _lib.check(L.gb_batch_plan_create(C.addressof(probs), 4096, 0, C.byref(plan)), "plan")
            _lib.check(L.gb_batch_plan_run(plan, 0, st), "run")
            torch.cuda.synchronize()
            c_nat = keep[2]
            rec["max_abs_diff_vs_native"] = float((c_oz - c_nat).abs().max())
            rec["max_abs_c"] = float(c_nat.abs().max())
        ms_l = _timer(lambda: _lib.check(L.gb_gemm_batch_dev(C.addressof(probs), 4096, dtype, 1, st), "loop"),
                      reps=1, warmup=1)
        L.gb_batch_plan_destroy(plan)
        rec.update({"loop_ms": ms_l, "loop_tflops": flops / ms_l / 1e9, "speedup": ms_l / ms_g})
        if dtype in (0, 1):
            # the same batch with per-problem configurations from the trained selector
            from . import selector as S
            S.load_into_library()
            try:
                pol = {}
                # fixed policies (3: FP32 through the split form), then the plan's own autotuning
                for policy in ((1, 2, 3, -1) if dtype == 1 else (1, 2, -1)):
                    plan2 = C.c_void_p()
                    _lib.check(L.gb_batch_plan_create_ex(C.addressof(probs), 4096, dtype, policy, C.byref(plan2)),
                               "plan")
                    ms_p = _timer(lambda: _lib.check(L.gb_batch_plan_run(plan2, 1, st), "run"), reps=3, warmup=1)
                    pol[policy] = (ms_p, L.gb_batch_plan_policy(plan2))
                    L.gb_batch_plan_destroy(plan2)
            finally:
                L.gb_set_gemm_autoselect(0)
                L.gb_selector_unload()
            rec.update({"policy1_selected_tiles_ms": pol[1][0], "policy2_selected_tiles_splitk_ms": pol[2][0],
                        "autotuned_plan_ms": pol[-1][0], "autotuned_policy": pol[-1][1],
                        "autotuned_tflops": flops / pol[-1][0] / 1e9})
            if dtype == 1:
                rec["policy3_split_form_ms"] = pol[3][0]
        out.append(rec)
        L.gb_set_dgemm_mode(0, 8)
        del keep


def run_batch_large_fp32(out):
    """FP32 gemm_batch of 64 problems with m, n, k log-uniform in [1024, 4096]:
    the FP32-pipe grouped plan (policy 0) against the split form (policy 3:
    the grouped Ozaki form at 3 slices on the FP32 operands), and the plan's autotuned pick."""
    L = _lib.load()
    probs, keep, flops = batch_problems(64, 5, 1, lo=1024, hi=4096)
    st = _stream()
    rec = {"workload": "batch_64_fp32_1024_4096", "flops": flops}
    for policy, key in ((0, "policy0_ffma"), (3, "policy3_split_form"), (-1, "autotuned")):
        plan = C.c_void_p()
        _lib.check(L.gb_batch_plan_create_ex(C.addressof(probs), 64, 1, policy, C.byref(plan)), "plan")
        ms = _timer(lambda: _lib.check(L.gb_batch_plan_run(plan, 1, st), "run"), reps=3, warmup=1)
        rec[key + "_ms"] = ms
        rec[key + "_tflops"] = flops / ms / 1e9
        if policy < 0:
            rec["autotuned_policy"] = L.gb_batch_plan_policy(plan)
        L.gb_batch_plan_destroy(plan)
    out.append(rec)
    del keep


def run_level3x(out):
    """dtrmm L/L/N/N 8192 x 4096 (m^2 n flop), dsyrk L/N n = k = 8192 (n^2 k),
    dsymm L/L 8192 x 4096 (2 m^2 n), native FP64 and Ozaki s = 7; U[-1,1]."""
    m, n = (4096, 2048) if SMALL else (8192, 4096)
    A = _mat(m, m, seed=51)
    B = _mat(m, n, seed=52)
    C0 = _mat(m, n, seed=53)
    K = _mat(m, m, seed=54)
    S = _mat(m, m, seed=55)
    for mode, name in _forms(((0, "native_fp64"), (1, "ozaki_s7"))):
        _lib.load().gb_set_dgemm_mode(mode, 7)
        reps = 1 if mode == 0 else 3
        x = B.clone()
        ms = _timer(lambda: (x.copy_(B), dev.dtrmm(0, 0xC0, 0, 0, 1.0, A, x)), reps=reps, warmup=1)
        copy_ms = _timer(lambda: x.copy_(B), reps=3, warmup=1)
        out.append({"workload": "dtrmm_%dx%d" % (m, n), "form": name, "ms": ms - copy_ms,
                    "tflops": float(m) * m * n / (ms - copy_ms) / 1e9})
        ms = _timer(lambda: dev.dsyrk(0xC0, 0, 1.0, K, 0.5, S), reps=reps, warmup=1)
        out.append({"workload": "dsyrk_%d_k%d" % (m, m), "form": name, "ms": ms,
                    "tflops": float(m) * m * m / ms / 1e9})
        c = C0.clone()
        ms = _timer(lambda: dev.dsymm(0, 0xC0, 1.0, A, B, 0.5, c), reps=reps, warmup=1)
        out.append({"workload": "dsymm_%dx%d" % (m, n), "form": name, "ms": ms,
                    "tflops": 2.0 * m * m * n / ms / 1e9})
    _lib.load().gb_set_dgemm_mode(0, 8)


def run_level12x(out):
    """dscal / dcopy (16 B per element) and idamax (8 B) at n = 2^28, dger on
    32768^2 (16 B per matrix element), dtrsv L/N/N m = 16384 (latency: 256
    diagonal blocks and gemv updates); HBM figures against the measured copy
    bandwidth."""
    import torch
    pk, kind = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    n = 1 << (25 if SMALL else 28)
    x = _mat(n, 1, seed=61).view(-1)
    y = torch.empty_like(x)
    idx = torch.zeros(1, dtype=torch.int64, device="cuda")
    for name, fn, byts in (("dscal", lambda: dev.dscalv(1.0000001, x), 16.0 * n),
                           ("dcopy", lambda: dev.dcopyv(x, y), 16.0 * n),
                           ("idamax", lambda: dev.damaxv(x, idx), 8.0 * n)):
        ms = _timer(fn, reps=10)
        gbs = byts / ms / 1e6
        out.append({"workload": "%s_2^%d" % (name, 25 if SMALL else 28), "ms": ms, "gb_s": gbs,
                    "frac_of_hbm": gbs / hbm, "peak": "%s hbm_gbs" % kind})
    del x, y
    m = 8192 if SMALL else 32768
    a = _mat(m, m, seed=62)
    xv = _mat(m, 1, seed=63).view(-1)
    yv = _mat(m, 1, seed=64).view(-1)
    ms = _timer(lambda: dev.dger(1e-9, xv, yv, a), reps=5)
    gbs = 16.0 * m * m / ms / 1e6
    out.append({"workload": "dger_%d" % m, "ms": ms, "gb_s": gbs, "frac_of_hbm": gbs / hbm,
                "peak": "%s hbm_gbs" % kind})
    del a
    mt = 16384
    t = _mat(mt, mt, seed=65)
    t.copy_(torch.tril(t))
    d = torch.arange(mt, device="cuda")
    t[d, d] = mt + t[d, d].abs()
    b = _mat(mt, 1, seed=66).view(-1)
    xs = b.clone()
    ms = _timer(lambda: (xs.copy_(b), dev.dtrsv(0xC0, 0, 0, 1.0, t, xs)), reps=3, warmup=1)
    out.append({"workload": "dtrsv_%d" % mt, "ms": ms, "gflops": float(mt) * mt / ms / 1e6})


def run_complex(out):
    """zgemm 4096^3 (8 m n k real flops) native FP64 and Ozaki s = 7, cgemm
    4096^3 FP32: one real gemm of 2m x n x 2k on the block-real operands."""
    import torch
    n = 2048 if SMALL else 4096
    L = _lib.load()
    for dt, name in ((torch.complex128, "zgemm"), (torch.complex64, "cgemm")):
        a = torch.complex(_mat(n, n, seed=71, dtype=torch.float64), _mat(n, n, seed=72, dtype=torch.float64)).to(dt)
        b = torch.complex(_mat(n, n, seed=73, dtype=torch.float64), _mat(n, n, seed=74, dtype=torch.float64)).to(dt)
        a, b = a.t().contiguous().t(), b.t().contiguous().t()
        c = torch.zeros((n, n), dtype=dt, device="cuda").t()
        forms = _forms(((0, "native_fp64"), (1, "ozaki_s7")) if dt == torch.complex128 else ((0, "fp32_default_dispatch"),))
        for mode, form in forms:
            L.gb_set_dgemm_mode(mode, 7)
            if dt == torch.complex128:
                al, be = _lib.DComplex(1.0, 0.5), _lib.DComplex(0.0, 0.0)
                fn = lambda: _lib.check(L.gb_zgemm_dev(0, 0, n, n, n, al, a.data_ptr(), 1, n, b.data_ptr(), 1, n,
                                                       be, c.data_ptr(), 1, n, _stream()), "zgemm")
            else:
                al, be = _lib.SComplex(1.0, 0.5), _lib.SComplex(0.0, 0.0)
                fn = lambda: _lib.check(L.gb_cgemm_dev(0, 0, n, n, n, al, a.data_ptr(), 1, n, b.data_ptr(), 1, n,
                                                       be, c.data_ptr(), 1, n, _stream()), "cgemm")
            ms = _timer(fn, reps=1 if mode == 0 and dt == torch.complex128 else 3, warmup=1)
            out.append({"workload": "%s_%d" % (name, n), "form": form, "ms": ms,
                        "tflops": 8.0 * n ** 3 / ms / 1e9})
    # ztrsm L/L/N/N m = n, diagonal n + |u|: 4 m^2 n real flops (half of a complex m x n x m gemm)
    a = torch.complex(_mat(n, n, seed=75), _mat(n, n, seed=76)).to(torch.complex128)
    a = torch.tril(a) + n * torch.eye(n, dtype=torch.complex128, device="cuda")
    a = a.t().contiguous().t()
    b0 = torch.complex(_mat(n, n, seed=77), _mat(n, n, seed=78)).t().contiguous().t()
    x = b0.clone()
    one = _lib.DComplex(1.0, 0.0)
    for mode, form in _forms(((0, "native_fp64"), (1, "ozaki_s7"))):
        L.gb_set_dgemm_mode(mode, 7)
        fn = lambda: (x.copy_(b0), _lib.check(L.gb_ztrsm_dev(0, 0xC0, 0, 0, n, n, one, a.data_ptr(), 1, n,
                                                             x.data_ptr(), 1, n, _stream()), "ztrsm"))
        ms = _timer(fn, reps=1 if mode == 0 else 3, warmup=1)
        copy_ms = _timer(lambda: x.copy_(b0), reps=3, warmup=1)
        out.append({"workload": "ztrsm_%dx%d" % (n, n), "form": form, "ms": ms - copy_ms,
                    "tflops": 4.0 * n ** 3 / (ms - copy_ms) / 1e9})
    L.gb_set_dgemm_mode(0, 8)
    # ctrsm, the same solve in single complex: FP32 diagonal solves, cgemm updates
    ac = a.to(torch.complex64).t().contiguous().t()
    bc = b0.to(torch.complex64).t().contiguous().t()
    xc = bc.clone()
    onec = _lib.SComplex(1.0, 0.0)
    fn = lambda: (xc.copy_(bc), _lib.check(L.gb_ctrsm_dev(0, 0xC0, 0, 0, n, n, onec, ac.data_ptr(), 1, n,
                                                          xc.data_ptr(), 1, n, _stream()), "ctrsm"))
    ms = _timer(fn, reps=3, warmup=1)
    copy_ms = _timer(lambda: xc.copy_(bc), reps=3, warmup=1)
    out.append({"workload": "ctrsm_%dx%d" % (n, n), "form": "fp32_default_dispatch", "ms": ms - copy_ms,
                "tflops": 4.0 * n ** 3 / (ms - copy_ms) / 1e9})
    # zgemv / cgemv N and T on a 16384 x 16384 column-major A (8192 when small): HBM-bound, the
    # algorithmic bytes are A's once
    g = 8192 if SMALL else 16384
    for dt, name, fn_name, S in ((torch.complex128, "zgemv", "gb_zgemv_dev", _lib.DComplex),
                                 (torch.complex64, "cgemv", "gb_cgemv_dev", _lib.SComplex)):
        ag = torch.complex(_mat(g, g, seed=79), _mat(g, g, seed=80)).to(dt)
        xg = torch.complex(_mat(g, 1, seed=81), _mat(g, 1, seed=82)).to(dt).view(-1)
        yg = torch.zeros(g, dtype=dt, device="cuda")
        fn_dev = getattr(L, fn_name)
        for tr, tname in ((0, "N"), (8, "T")):
            fn = lambda: _lib.check(fn_dev(tr, 0, g, g, S(1.0, 0.5), ag.data_ptr(), 1, g, xg.data_ptr(), 1,
                                           S(0.0, 0.0), yg.data_ptr(), 1, _stream()), name)
            ms = _timer(fn, reps=5, warmup=2)
            out.append({"workload": "%s_%s_%d" % (name, tname, g), "ms": ms,
                        "gbs": ag.element_size() * g * g / ms / 1e6})
        del ag


def run_hermitian(out):
    """zherk L/N n = k = 4096 (4 n^2 k real flops: half of the complex product),
    zher2k (8 n^2 k), zhemm L/L 4096 x 4096 (8 m^2 n) and dsyr2k L/N n = k =
    8192 (2 n^2 k), native FP64 and Ozaki s = 7; U[-1,1] parts."""
    import torch
    n = 2048 if SMALL else 4096
    L = _lib.load()

    def cm(seed):
        z = torch.complex(_mat(n, n, seed=seed), _mat(n, n, seed=seed + 1))
        return z.t().contiguous().t()

    a, b, c = cm(81), cm(83), cm(85)
    one, half = _lib.DComplex(1.0, 0.0), _lib.DComplex(0.5, 0.0)
    m2 = 2 * n
    ra, rb, rc = _mat(m2, m2, seed=87), _mat(m2, m2, seed=88), _mat(m2, m2, seed=89)
    for mode, form in _forms(((0, "native_fp64"), (1, "ozaki_s7"))):
        L.gb_set_dgemm_mode(mode, 7)
        reps = 1 if mode == 0 else 3
        p = lambda t: t.data_ptr()
        ms = _timer(lambda: _lib.check(L.gb_zherk_dev(0xC0, 0, n, n, 1.0, p(a), 1, n, 0.5, p(c), 1, n, _stream()),
                                       "zherk"), reps=reps, warmup=1)
        out.append({"workload": "zherk_%d_k%d" % (n, n), "form": form, "ms": ms, "tflops": 4.0 * n ** 3 / ms / 1e9})
        ms = _timer(lambda: _lib.check(L.gb_zher2k_dev(0xC0, 0, 0, n, n, one, p(a), 1, n, p(b), 1, n, 0.5, p(c), 1, n,
                                                       _stream()), "zher2k"), reps=reps, warmup=1)
        out.append({"workload": "zher2k_%d_k%d" % (n, n), "form": form, "ms": ms, "tflops": 8.0 * n ** 3 / ms / 1e9})
        ms = _timer(lambda: _lib.check(L.gb_zhemm_dev(0, 0xC0, 0, 0, n, n, one, p(a), 1, n, p(b), 1, n, half, p(c), 1,
                                                      n, _stream()), "zhemm"), reps=reps, warmup=1)
        out.append({"workload": "zhemm_%dx%d" % (n, n), "form": form, "ms": ms, "tflops": 8.0 * n ** 3 / ms / 1e9})
        ms = _timer(lambda: dev.dsyr2k(0xC0, 0, 0, 1.0, ra, rb, 0.5, rc), reps=reps, warmup=1)
        out.append({"workload": "dsyr2k_%d_k%d" % (m2, m2), "form": form, "ms": ms,
                    "tflops": 2.0 * float(m2) ** 3 / ms / 1e9})
    L.gb_set_dgemm_mode(0, 8)


def run_crt(out):
    """The CRT form of the Ozaki product alone, 16 moduli, exponent-spread operands (the
    benchmark's inputs) at 16384^3, or 4096^3 with --small (the profiling case: each of the
    split, slice GEMM and recombination kernels launches once per product, three products)."""
    n = CRT_N or (4096 if SMALL else 16384)
    a = _mat(n, n, kind=dev.RAND_EXPSPREAD, seed=61, p0=-20, p1=20)
    b = _mat(n, n, kind=dev.RAND_EXPSPREAD, seed=62, p0=-20, p1=20)
    c = _mat(n, n, seed=63)
    ms = _timer(lambda: dev.dgemm_ozaki_crt(0, 0, 1.0, a, b, 0.0, c, 16), reps=3, warmup=1)
    dev.set_kernel_timing(True)
    dev.kernel_time_ms("")
    for _ in range(3):
        dev.dgemm_ozaki_crt(0, 0, 1.0, a, b, 0.0, c, 16)
    stages = {pre: dev.kernel_time_ms(pre)[0] / 3 for pre in ("oz_rowmax", "oz_split_crt", "ozaki_slice_gemm",
                                                              "oz_recombine")}
    dev.set_kernel_timing(False)
    out.append({"workload": "dgemm_%d_crt16_expspread" % n, "ms": ms, "tflops": 2.0 * n ** 3 / ms / 1e9,
                "stage_ms": stages})


def run_e2e(out, calls=8):
    """dgemm_ on pinned host buffers through the C ABI (the pipelined host path): the host
    time of each call, and the launch/copy timeline of the fastest and the slowest call."""
    import time
    import torch
    n = 4096 if SMALL else 16384
    hs = [torch.empty((n, n), dtype=torch.float64, pin_memory=True) for _ in range(3)]
    for i, h in enumerate(hs[:2]):
        d = _mat(n, n, kind=dev.RAND_EXPSPREAD, seed=71 + i, p0=-20, p1=20)
        h.copy_(d.t())  # row-major storage of the transpose: column-major d
        del d
    torch.cuda.synchronize()
    an, bn, cn = (h.numpy() for h in hs)
    blas.set_dgemm_mode(blas.DGEMM_OZAKI_CRT, 16)
    try:
        blas.dgemm("N", "N", n, n, n, 1.0, an, n, bn, n, 0.0, cn, n)
        dev.set_kernel_timing(True)
        dev.kernel_trace()
        runs = []
        for _ in range(calls):
            t0 = time.perf_counter()
            blas.dgemm("N", "N", n, n, n, 1.0, an, n, bn, n, 0.0, cn, n)
            runs.append(((time.perf_counter() - t0) * 1e3, dev.kernel_trace()))
    finally:
        dev.set_kernel_timing(False)
        blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    ms = sorted(r[0] for r in runs)
    rec = {"workload": "dgemm_%d_e2e_crt16" % n, "calls": calls, "ms": [r[0] for r in runs],
           "tflops_median": 2.0 * n ** 3 / ms[len(ms) // 2] / 1e9, "tflops_best": 2.0 * n ** 3 / ms[0] / 1e9}
    for label, (t, tr) in (("fastest", min(runs, key=lambda r: r[0])), ("slowest", max(runs, key=lambda r: r[0]))):
        rec[label] = {"ms": t, "timeline": [(nm, round(a, 3), round(b, 3)) for nm, a, b in sorted(tr, key=lambda x: x[1])]}
    out.append(rec)


SUITES = {"crt": run_crt, "e2e": run_e2e, "gemm": run_gemm, "trsm": run_trsm, "strsm": run_strsm, "trsm_ozaki": run_trsm_ozaki, "level12": run_level12,
          "batch": run_batch, "batch_fp32_large": run_batch_large_fp32, "batch_ozaki": run_batch_ozaki,
          "sgemm": run_sgemm, "bgemm": run_bgemm,
          "level3x": run_level3x, "level12x": run_level12x, "complex": run_complex, "hermitian": run_hermitian}


def main():
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="")
    ap.add_argument("--json")
    ap.add_argument("--batch-count", type=int, default=4096, help="problems of the batch_ozaki suite")
    ap.add_argument("--small", action="store_true", help="profiling sizes (workload names keep the full size)")
    ap.add_argument("--crt-n", type=int, default=0, help="size of the crt suite's product (0: 16384, 4096 with --small)")
    ap.add_argument("--trsm-forms", default="native,ozaki", help="DTRSM forms of the trsm suites")
    ap.add_argument("--forms", default="native,ozaki", help="forms of the level3x, hermitian and complex suites")
    a = ap.parse_args()
    global BATCH_COUNT, SMALL, TRSM_FORMS, FORMS, CRT_N
    BATCH_COUNT = a.batch_count
    CRT_N = a.crt_n
    SMALL = a.small
    TRSM_FORMS = tuple(f for f in a.trsm_forms.split(",") if f)
    FORMS = tuple(f for f in a.forms.split(",") if f)
    torch.cuda.set_device(0)
    _lib.check(_lib.load().gb_init(0), "gb_init")
    names = [s for s in a.only.split(",") if s] or list(SUITES)
    out = []
    for nm in names:
        SUITES[nm](out)
    for r in out:
        print(json.dumps(r), flush=True)
    if a.json:
        with open(a.json, "w") as f:
            for r in out:
                f.write(json.dumps(r) + "\n")


if __name__ == "__main__":
    main()
