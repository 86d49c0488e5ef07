#!/usr/bin/env python
"""bench.py -- emulated (Ozaki split-product) vs native DGEMM on one GB300.

Workload (the configuration the headline metric is quoted on): DGEMM
C := A*B with m = n = k = 16384, column-major FP64, entries (1+u)*2^e with
e uniform in [-20, 20] and random sign, generated on the device by the
library's seeded generator.  A "step" is one full DGEMM.

  value      emulated DGEMM on the bf16 tensor cores (tcgen05) in
             FP64-equivalent TFLOP/s (2mnk per step), operands resident in
             HBM, CUDA events on the launching stream, K steps after W
             warm-up steps.  Two forms are swept: digit slices (s = 3..8,
             s(s+1)/2 products) and CRT residues (N = 10..16 moduli, N
             products); the value is the fastest whose max componentwise
             error is at most native FP64 DGEMM's on the same inputs
             (--slices or --moduli fixes the form instead).
  e2e        the same DGEMM through the BLAS entry point dgemm_ (C ABI) on
             pinned host buffers: H2D of A and B and D2H of C inside the
             timed region of every step.
  forms      native FP64 DGEMM (DMMA) on the same inputs, both results'
             max componentwise error against a double-double evaluation of
             4096 sampled entries, and the speed-up of the emulated form.
  roofline   the dominant kernel (ozaki_slice_gemm): slice-product flops
             (s(s+1)/2 * 2mnk) per launch over its event-timed duration,
             against the measured bf16 tensor peak.
  cpu_baseline  BLIS's own DGEMM (the reference compiled from its sources
             by oracle/ref_blis.py, the sub-configuration BLIS picks on this
             host, all host cores) on a column sample of the workload;
             cpu_baseline_port is the oracle's C restatement of the five-loop
             DGEMM on the same kind of sample, for comparison.

`--impl reference` times BLIS's own DGEMM alone on the same workload (a
column sample per step) and prints the reference line (the restatement when
the reference build is missing, which the line's cpu_baseline.kind says).
Multi-GPU: the path is replicated (one independent DGEMM per rank, no
collective); `value` sums the ranks' flops over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZE = 16384
SLICES = 8
EMIN, EMAX = -20, 20
SEED_A, SEED_B = 20261204, 20261205
# DRAM bytes read and written by one ozaki_slice_gemm_pair_kernel launch at 4096^3 from ncu --set
# full captures (dram__bytes_read.sum, dram__bytes_write.sum), with the products and int32 planes
# of that launch: the digit form at 7 slices (28 products, 7 level planes) and the CRT form at 16
# moduli (16 products, 16 planes)
TRAFFIC_4096 = {"digits": (7136346112, 473230848, 28, 7), "crt": (1368333000, 532505600, 16, 16)}
# One block product of the CRT form's blocked layout (2048 x 4096 x 8192, 16 moduli) moved 2.78 GB
# from DRAM (ncu, SpeedOfLight + MemoryWorkloadAnalysis: dram__bytes.sum.per_second x duration);
# a block launch of another size is scaled by its units m_b n_b k
TRAFFIC_CRT_BLOCK = (2.782e9, 2048 * 4096 * 8192, 16)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, default=SIZE)
    p.add_argument("--slices", type=int, default=0,
                   help="slice count of the timed form; 0 = the smallest count of the 3..8 sweep whose "
                        "max componentwise error is at most native FP64's")
    p.add_argument("--moduli", type=int, default=0,
                   help="run the CRT form with this many moduli instead of the sweep's choice")
    p.add_argument("--e2e-steps", type=int, default=0, help="end-to-end steps (0: --steps)")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    return p.parse_args()


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _blis_ref():
    """ctypes handle of the reference BLIS build, or None when it is not built here."""
    try:
        from oracle import blis_ctypes as bc
        if bc.available():
            bc.lib()
            return bc
    except OSError:
        pass
    return None


def cpu_dgemm_sample(n, seconds, threads, seed=SEED_A, use_blis=True):
    """Times a CPU DGEMM on an n x cols x n column sample sized for about `seconds` of
    work: BLIS's own bli_dgemm when the reference build is present (kind "reference"),
    else the oracle's restatement (kind "port").  Returns (TFLOP/s, kind, description, s)."""
    import numpy as np
    from oracle import pyoracle as po
    bc = _blis_ref() if use_blis else None
    if bc is not None:
        bc.set_threads(threads)

        def gemm(a, b, c):
            bc.dgemm(0, 0, 1.0, a, b, 0.0, c)
        kind, what = "reference", "BLIS bli_dgemm (%s sub-configuration, pthreads)" % bc.arch_name()
    else:
        def gemm(a, b, c):
            po.dgemm(0, 0, 1.0, a, b, 0.0, c, nthreads=threads)
        kind, what = "port", "five-loop C restatement of bli_gemm"
    a = po.expspread((n, n), seed, EMIN, EMAX)
    cols = 64
    b = po.expspread((n, cols), seed + 1, EMIN, EMAX)
    c = np.zeros((n, cols), order="F")
    gemm(a, b, c)  # warm-up (thread pool, packing buffers)
    t0 = time.perf_counter()
    gemm(a, b, c)
    dt = time.perf_counter() - t0
    rate = 2.0 * n * n * cols / dt
    cols2 = int(max(64, min(n, rate * seconds / (2.0 * n * n)))) // 64 * 64
    b = po.expspread((n, cols2), seed + 1, EMIN, EMAX)
    c = np.zeros((n, cols2), order="F")
    t0 = time.perf_counter()
    gemm(a, b, c)
    dt = time.perf_counter() - t0
    tf = 2.0 * n * n * cols2 / dt / 1e12
    return tf, kind, "m=k=%d, n=%d column sample of the %d^3 DGEMM (%.1f s), %s, %d threads" % (
        n, cols2, n, dt, what, threads), dt


def run_reference(args):
    ws, rank, local = dist_setup(args)
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = args.size
    import numpy as np
    from oracle import pyoracle as po
    bc = _blis_ref()
    if bc is not None:
        bc.set_threads(threads)

        def gemm(a, b, c):
            bc.dgemm(0, 0, 1.0, a, b, 0.0, c)
        kind, what = "reference", "BLIS bli_dgemm (%s sub-configuration, pthreads)" % bc.arch_name()
    else:
        def gemm(a, b, c):
            po.dgemm(0, 0, 1.0, a, b, 0.0, c, nthreads=threads)
        kind, what = "port", "five-loop C restatement of bli_gemm (reference build missing)"
    a = po.expspread((n, n), SEED_A, EMIN, EMAX)
    cols = 64
    b = po.expspread((n, cols), SEED_B, EMIN, EMAX)
    c = np.zeros((n, cols), order="F")
    gemm(a, b, c)
    # per-step sample sized so that warm-up + steps stay within a few minutes
    t0 = time.perf_counter()
    gemm(a, b, c)
    rate = 2.0 * n * n * cols / (time.perf_counter() - t0)
    budget = 120.0 / max(1, args.steps + args.warmup)
    cols = int(max(64, min(n, rate * budget / (2.0 * n * n)))) // 64 * 64
    b = po.expspread((n, cols), SEED_B, EMIN, EMAX)
    c = np.zeros((n, cols), order="F")
    for _ in range(args.warmup):
        gemm(a, b, c)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gemm(a, b, c)
    dt = (time.perf_counter() - t0) / max(1, args.steps)
    tf = 2.0 * n * n * cols / dt / 1e12
    sample = "m=k=%d, n=%d column sample per step of the %d^3 DGEMM, %s, %d threads" % (
        n, cols, n, what, threads)
    line = {
        "impl": "reference", "metric": "Emulated vs native DGEMM TFLOP/s on 1 GB300 at FP64-level error; % of roofline",
        "value": tf, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "dgemm_%d_expspread" % n, "m": n, "n": n, "k": n, "e_range": [EMIN, EMAX],
                   "sample_cols": cols},
        "cpu_baseline": {"value": tf, "unit": "TFLOP/s", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": tf, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def host_link_gbs(nbytes=1 << 30, reps=3):
    """Pinned host<->device copy bandwidth of this machine (GB/s), H2D and D2H, one
    cudaMemcpyAsync of `nbytes` at a time on the current stream."""
    import torch
    h = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
    d = torch.empty(nbytes // 8, dtype=torch.float64, device="cuda")
    h.fill_(1.0)
    out = []
    for direction in ("h2d", "d2h"):
        fn = (lambda: d.copy_(h, non_blocking=True)) if direction == "h2d" else \
             (lambda: h.copy_(d, non_blocking=True))
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        out.append(nbytes * reps / (time.perf_counter() - t0) / 1e9)
    del h, d
    return out


def run_gpu(args):
    import numpy as np
    import torch
    from blis_gb300 import _lib, blas, dev

    ws, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    L = _lib.load()
    _lib.check(L.gb_init(local), "gb_init")
    n = args.size
    flops = 2.0 * n * n * n
    peaks, peak_kind = load_peaks()

    A = dev.colmajor(n, n)
    B = dev.colmajor(n, n)
    Cz = dev.colmajor(n, n)
    dev.randm(A, dev.RAND_EXPSPREAD, SEED_A, EMIN, EMAX)
    dev.randm(B, dev.RAND_EXPSPREAD, SEED_B, EMIN, EMAX)
    Cz.zero_()
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.current_stream()

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        fn()
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1)

    # ---------------- double-double reference values of a fixed entry sample
    g = torch.Generator(device="cpu").manual_seed(7)
    ii = torch.randint(0, n, (4096,), generator=g).cuda()
    jj = torch.randint(0, n, (4096,), generator=g).cuda()
    hi, lo = dev.dd_gemm_entries(0, 0, 1.0, A, B, 0.0, None, ii, jj)

    # ---------------- native FP64 form on the same inputs (one timed call)
    Cn = dev.colmajor(n, n)
    w = min(n, 2048)
    dev.dgemm(0, 0, 1.0, A[:w, :w], B[:w, :w], 0.0, Cn[:w, :w])
    native_ms = timed(lambda: dev.dgemm(0, 0, 1.0, A, B, 0.0, Cn))
    native_tf = flops / (native_ms * 1e-3) / 1e12
    err_nat = dev.componentwise_error(Cn[ii, jj], hi, lo)
    del Cn

    # ---------------- sweep of both emulated forms: time and error of each count
    # digit form: s slices, s(s+1)/2 products; CRT form: N moduli, N products
    def run_form(form, cnt):
        if form == "crt":
            dev.dgemm_ozaki_crt(0, 0, 1.0, A, B, 0.0, Cz, cnt)
        else:
            dev.dgemm_ozaki(0, 0, 1.0, A, B, 0.0, Cz, cnt)

    sweep = []
    for form, counts in (("digits", range(3, 9)), ("crt", range(10, 17))):
        for cnt in counts:
            run_form(form, cnt)
            ms_sl = timed(lambda: run_form(form, cnt))
            err_sl = dev.componentwise_error(Cz[ii, jj], hi, lo)
            prods = cnt * (cnt + 1) // 2 if form == "digits" else cnt
            sweep.append({"form": form, "slices" if form == "digits" else "moduli": cnt, "products": prods,
                          "ms": ms_sl, "tflops": flops / (ms_sl * 1e-3) / 1e12, "max_componentwise_err": err_sl})
    ok = [r for r in sweep if r["max_componentwise_err"] <= err_nat]
    if args.slices > 0:
        form, s = "digits", args.slices
    elif args.moduli > 0:
        form, s = "crt", args.moduli
    elif ok:
        best = min(ok, key=lambda r: r["ms"])
        form, s = best["form"], best.get("slices", best.get("moduli"))
    else:
        form, s = "digits", 8
    npairs = s * (s + 1) // 2 if form == "digits" else s

    # ---------------- the chosen emulated form, device resident (value)
    for _ in range(args.warmup):
        run_form(form, s)
    barrier()
    dev.set_kernel_timing(True)
    dev.kernel_time_ms("")  # drop earlier records
    l0 = L.gb_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            run_form(form, s)
        ev1.record(stream)
        barrier()
    launches = int(L.gb_launch_count() - l0)
    dev.set_kernel_timing(False)
    ms = ev0.elapsed_time(ev1) / args.steps
    gemm_ms, gemm_n = dev.kernel_time_ms("ozaki_slice_gemm")
    stage_ms = {nm: dev.kernel_time_ms(nm)[0] / max(1, args.steps)
                for nm in ("oz_rowmax", "oz_split", "oz_recombine", "dgemm_dmma_gated")}  # oz_split: both forms
    split_ms = sum(stage_ms.values()) * max(1, args.steps)
    dev.kernel_time_ms("")
    err_oz = dev.componentwise_error(Cz[ii, jj], hi, lo)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = flops * ws / (ms * 1e-3) / 1e12
    # the product runs as one slice GEMM launch, or as one per block of C (the device entry
    # points' blocked form at large sizes): the algorithmic flops of a launch are the step's
    # divided by the launches per step
    kern_ms = gemm_ms / max(1, gemm_n)
    launches_per_step = max(1.0, gemm_n / max(1, args.steps))
    flops_per_launch = npairs * flops / launches_per_step
    achieved = flops_per_launch / (kern_ms * 1e-3) / 1e12
    peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops"))

    # ---------------- end to end through dgemm_ with pinned host buffers
    h2d_gbs, d2h_gbs = host_link_gbs()
    Ah = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Bh = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ch = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ah.copy_(A.t())  # Ah row-major storage of A^T == column-major A
    Bh.copy_(B.t())
    torch.cuda.synchronize()
    blas.set_dgemm_mode(blas.DGEMM_OZAKI_CRT if form == "crt" else blas.DGEMM_OZAKI, s)
    an, bn, cn = Ah.numpy(), Bh.numpy(), Ch.numpy()
    blas.dgemm("N", "N", n, n, n, 1.0, an, n, bn, n, 0.0, cn, n)  # warm-up
    e2e_steps = args.e2e_steps if args.e2e_steps > 0 else args.steps
    barrier()
    t0 = time.perf_counter()
    call_ms = []
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        blas.dgemm("N", "N", n, n, n, 1.0, an, n, bn, n, 0.0, cn, n)  # returns after C is on the host
        call_ms.append((time.perf_counter() - t1) * 1e3)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    blas.set_dgemm_mode(blas.DGEMM_NATIVE)
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_tf = flops * ws / (e2e_ms * 1e-3) / 1e12
    # cn holds column-major C, i.e. cn[j, i] == C[i, j]: the whole product against the
    # device-resident run's, bit for bit
    Ch2 = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ch2.copy_(Cz.t())
    torch.cuda.synchronize()
    e2e_ok = bool(np.array_equal(cn, Ch2.numpy()))
    del Ch2

    # ---------------- DRAM traffic of the dominant kernel from the ncu captures at 4096^3 above:
    # reads scale with the slice-product units, (n/4096)^3 per product (each tile reads its rows
    # and columns over all of k, in the same tiling), writes with the int32 planes, (n/4096)^2 per
    # plane
    rd, wr, prods, planes = TRAFFIC_4096[form]
    # (per step; a block product moves its share of it: the same tiling over its rows and columns)
    traffic = rd * (n / 4096.0) ** 3 * npairs / prods + wr * (n / 4096.0) ** 2 * (npairs if form == "crt" else s) / planes
    traffic /= launches_per_step
    if form == "crt" and launches_per_step > 1:
        # the blocked form's launch, from the capture of one block product scaled by its units
        tb, units, mod = TRAFFIC_CRT_BLOCK
        traffic = tb * (float(n) ** 3 / launches_per_step) / units * npairs / mod

    if rank != 0:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    threads = os.cpu_count() or 1
    cpu_tf, cpu_kind, cpu_sample, _ = cpu_dgemm_sample(min(n, 16384), args.cpu_seconds, threads)
    port_tf, _, port_sample, _ = cpu_dgemm_sample(min(n, 16384), args.cpu_seconds / 3, threads, use_blis=False)

    line = {
        "metric": "Emulated vs native DGEMM TFLOP/s on 1 GB300 at FP64-level error; % of roofline",
        "value": value,
        "unit": "TFLOP/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: (1+u)*2^e, e in [-20,20], random sign, seeded counter RNG on device",
        "config": {"workload": "ozaki_dgemm_%d" % n, "m": n, "n": n, "k": n, "layout": "column-major",
                   "alpha": 1.0, "beta": 0.0,
                   "form": ("ozaki bf16 slices=%d (triangular, %d products)" % (s, npairs)) if form == "digits"
                   else ("ozaki CRT bf16 residues, %d moduli (%d products)" % (s, npairs)),
                   "l2": "inputs 2 GiB each, larger than the 126 MB L2", "parallelism": "replicas" if ws > 1 else "1 GPU"},
        "forms": {
            "ozaki": {"tflops": value / ws, "max_componentwise_err": err_oz, "form": form,
                      "slices" if form == "digits" else "moduli": s, "products": npairs,
                      "choice": "fastest of the sweep with error <= native"
                      if args.slices == 0 and args.moduli == 0 else "fixed"},
            "slice_sweep": sweep,
            "native_fp64": {"tflops": native_tf, "ms": native_ms, "max_componentwise_err": err_nat,
                            "engine": os.environ.get("GB_DGEMM_ENGINE", "dmma")},
            "speedup_vs_native": (value / ws) / native_tf,
            "error_ratio_ozaki_over_native": err_oz / err_nat if err_nat > 0 else None,
            "err_sample": "4096 random entries, double-double evaluation on the device",
        },
        "e2e": {"value": e2e_tf, "unit": "TFLOP/s", "h2d_bytes_per_step": 2 * 8 * n * n,
                "d2h_bytes_per_step": 8 * n * n, "ms_per_step": e2e_ms, "steps": e2e_steps,
                "api": "dgemm_ (C ABI), pinned host buffers",
                "matches_device_result": e2e_ok, "compared": "all of C, bit for bit",
                "host_link_gbs": {"h2d": h2d_gbs, "d2h": d2h_gbs},
                "copy_ms_if_serial": (2 * 8 * n * n / (h2d_gbs * 1e9) + 8 * n * n / (d2h_gbs * 1e9)) * 1e3,
                "exposed_ms": e2e_ms - ms,
                "per_call_ms": {"min": min(call_ms), "median": float(np.median(call_ms)), "max": max(call_ms)}},
        "roofline": {"bound": "tensor", "kernel": "ozaki_slice_gemm", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "%s bf16_tflops_sustained" % peak_kind,
                     "kernel_ms": kern_ms, "algorithmic_flops_per_launch": flops_per_launch,
                     "launches_per_step": launches_per_step,
                     "split_recombine_ms_per_step": (split_ms / max(1, args.steps)),
                     "stage_ms_per_step": stage_ms,
                     "timing_note": "CUDA-event span of each launch on its own stream; with the product in "
                                    "blocks on two compute streams the spans overlap one another, so kernel_ms "
                                    "and the stage times are upper bounds and achieved a lower bound"
                                    if launches_per_step > 1 else "CUDA-event span of each launch"},
        "cpu_baseline": {"value": cpu_tf, "unit": "TFLOP/s", "cores": threads, "kind": cpu_kind,
                         "sample": cpu_sample},
        "cpu_baseline_port": {"value": port_tf, "unit": "TFLOP/s", "cores": threads, "kind": "port",
                              "sample": port_sample},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
