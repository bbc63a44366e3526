#!/usr/bin/env python
"""Benchmark of the GB300 LU factor-and-solve path.

Workload (one step): plain FP64 LU with partial pivoting of an n=8192 matrix
A ~ iid N(0,1), then the solve of 16 right-hand sides B ~ iid N(0,1) (seed 2),
through the library's C ABI. Throughput is reported in GFLOP/s with the nominal
count 2/3 n^3 + 2 n^2 nrhs (factor + solve).

  value : inputs resident in HBM (la_lu_new_device + la_lu_solve_device),
          timed with CUDA events on the library's stream. The 512 MiB matrix is
          larger than L2 (129 MB), so no flush is needed between steps.
  e2e   : the public host-pointer API (la_lu_new + la_lu_solve) from pinned
          host memory; the copy of A and B to the device and of X back are
          inside the timed region.
  roofline : the trailing-update FP64 GEMM (the dominant kernel), its
          algorithmic flops over its device time (per-phase CUDA events inside
          the library, from two extra untimed factorizations), against this
          GPU's FP64 FMA rate measured live.
  cpu_baseline : the oracle (a single-threaded restatement of the reference's
          left-looking LUDecomposition::new) timed on a bounded prefix of the
          same factorization on this host.

Further sections of the same JSON line (skipped with --no-mixed,
--no-batched, --no-selector):
  mixed_ir : mixed-precision LU (tcgen05 BF16, FP16 or split-FP8 trailing
          updates, or FP32 SIMT ones)
          + FP64 refinement at n=16384, kappa in {1e2, 1e6, 1e10}, 4 RHS,
          against the plain FP64 LU at the same size; the headline speed-up is
          the automatic path (la_lu_solve_auto_device), each fixed precision
          is reported beside it.
  batched_uneven : 20,000 systems, n uniform in [8, 256], 1-4 RHS, half of them
          shifted by 0.5 n I; solves/s of the mixed plan against the plain FP64
          plan, each with its autotuned shape.
  learned_selector : 50,000 held-out Householder-conditioned systems, n in
          [16, 512], log10 kappa uniform in [1, 12]; plain FP64 plan, mixed plan
          with FP32 factors everywhere, and the selector's per-system choice
          (features + inference included).

`--impl reference` times the reference's CPU algorithm (the oracle's
multi-threaded form, bit-identical results) on the same workload instead.
Multi-GPU runs are independent replicas (the single LU does not shard).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "rust-la_gb300"))
sys.path.insert(0, ROOT)

METRIC = "LU-solve GFLOP/s & solves/s at backward err ≤1e-14: mixed-IR vs plain FP64"
WORKLOAD = "plain FP64 LU with partial pivoting + solve, n=8192, 16 RHS, A and B iid N(0,1)"


def lu_solve_flops(n, nrhs):
    return 2.0 / 3.0 * n ** 3 + 2.0 * n ** 2 * nrhs


def trailing_gemm_launches(n, w, lookahead=True):
    """(M, N, K) of every trailing-update GEMM launch of one LU of a square n
    with panel width w, as the library issues them: with lookahead each panel
    updates the next panel's columns first and the rest in a second launch."""
    out = []
    for j0 in range(0, n, w):
        jb = min(w, n - j0)
        j1 = j0 + jb
        if j1 >= n:
            break
        jbn = min(w, n - j1)
        m = n - j1
        if lookahead:
            out.append((m, jbn, jb))
            if n - (j1 + jbn) > 0:
                out.append((m, n - (j1 + jbn), jb))
        else:
            out.append((m, n - j1, jb))
    return out


def gemm_algorithmic(launches):
    """Total flops, and mean flops and mean DRAM bytes per launch (read A and B
    once, read and write C once: 8 (MK + KN + 2 MN) bytes) of the launches."""
    flops = sum(2.0 * m * n * k for m, n, k in launches)
    nbytes = sum(8.0 * (m * k + k * n + 2.0 * m * n) for m, n, k in launches)
    return flops, flops / len(launches), nbytes / len(launches)


# DRAM traffic of the trailing-update GEMM (gemm_f64_tma_kernel) measured by
# ncu (dram__bytes_read.sum + dram__bytes_write.sum) over all 253 launches of
# one n = 8192 factorization of this benchmark's matrix: bytes per launch
# (mean). Summary and command: profiles/gemm_f64_tma_traffic_n8192.md.
GEMM_TRAFFIC_BYTES_PER_LAUNCH = 156961959


def event_ms(torch, fn, reps=5, warmup=1):
    """Median and all device times (ms) of reps calls of fn, each bracketed by
    CUDA events on the current stream (the library's stream) after warmup
    untimed calls, with a synchronize on both sides."""
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        fn()
        e1.record(s)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.median(times), times


def prefix_flops(n, jend):
    """Flops the left-looking reference loop executes for columns [0, jend) of a square n."""
    j = np.arange(jend, dtype=np.float64)
    # sum_i min(i, j) multiply-adds for column j, plus n-j-1 divisions
    madd = j * (j - 1) / 2 + j * (n - j)
    return float(np.sum(2 * madd + np.maximum(n - j - 1, 0)))


class ClockSampler:
    """nvidia-smi samples (200 ms) during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def pick_prefix(oracle, a, n, target_s, threads):
    """Longest column prefix whose left-looking factorization takes about target_s."""
    j_try = 128
    t0 = time.perf_counter()
    oracle.lu_factor(a, j_end=j_try, threads=threads)
    rate = prefix_flops(n, j_try) / max(time.perf_counter() - t0, 1e-4)
    budget = rate * target_s
    lo, hi = j_try, n
    while lo < hi:
        mid = (lo + hi + 1) // 2
        if prefix_flops(n, mid) <= budget:
            lo = mid
        else:
            hi = mid - 1
    return lo


def run_cholesky(la_gpu, torch, ctx, stream, n, nrhs, fp64_peak, cpu_s=5.0):
    """CholeskyDecomposition::new + solve (src/decomp/cholesky.rs:56-145) at
    n = 8192 with 16 RHS, FAST arithmetic, on a seeded symmetric diagonally
    dominant matrix ((G + G')/2 + n I, G iid U(-1, 1)); nominal flops
    n^3/3 + 2 n^2 nrhs. The CPU line is the oracle (the reference's row order,
    one thread) on the first rows of the same factorization."""
    g = torch.Generator(device="cuda").manual_seed(4)
    x0 = torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    a = (x0 + x0.T) / 2 + n * torch.eye(n, device="cuda", dtype=torch.float64)
    del x0
    b = torch.randn((n, nrhs), generator=g, device="cuda", dtype=torch.float64)
    x = torch.empty_like(b)
    torch.cuda.synchronize()

    def step():
        c = la_gpu.CholeskyDecomposition.new_device(a.data_ptr(), n, n, ctx)
        c.solve_device(b.data_ptr(), nrhs, n, nrhs, x.data_ptr(), nrhs)
        return c

    step().free()
    ctx.synchronize()
    reps = 3
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        c = step()
        c.free()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flops = n ** 3 / 3.0 + 2.0 * n * n * nrhs
    eta = la_gpu.backward_error_device(ctx, a.data_ptr(), n, x.data_ptr(), nrhs, b.data_ptr(),
                                       nrhs, n, nrhs)
    out = {"workload": "Cholesky factor + solve, n=8192, 16 RHS, A = (G + G')/2 + n I",
           "ms": ms, "gflops": flops / (ms * 1e-3) / 1e9,
           "frac_of_fp64_peak": flops / (ms * 1e-3) / 1e12 / fp64_peak,
           "flops_basis": "nominal n^3/3 + 2 n^2 nrhs", "eta": eta, "cpu_oracle": None}
    if cpu_s > 0:
        import oracle
        a_np = a.cpu().numpy()
        rows, took = 256, 0.0
        while True:
            t0 = time.perf_counter()
            oracle.chol_new(a_np, j_end=rows)
            took = time.perf_counter() - t0
            if took >= cpu_s or rows >= n:
                break
            rows = min(n, int(rows * max(1.3, (cpu_s / max(took, 1e-3)) ** (1.0 / 3.0))))
        cf = rows ** 3 / 3.0
        out["cpu_oracle"] = {"value": cf / took / 1e9, "unit": "GFLOP/s", "cores": 1,
                             "kind": "port",
                             "sample": "rows [0,%d) of the n=8192 factorization in the reference's "
                                       "row order (cholesky.rs:64-107), %.3g flops in %.1f s"
                                       % (rows, cf, took)}
    del a, b, x
    return out


def guarded(section, *args, **kwargs):
    """Runs one side section of the benchmark; a failure there is reported in
    its own entry and does not take the benchmark line down with it."""
    try:
        return section(*args, **kwargs)
    except Exception as e:
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_qr(la_gpu, torch, ctx, n=2048, nrhs=4, cpu=True, fp64_peak=None):
    """QRDecomposition::new, get_q and solve (src/decomp/qr.rs:26-238), FAST
    arithmetic (blocks of 64 reflections in compact WY form), on an n x n
    N(0,1) matrix (seed 6): nominal flops 4/3 n^3 for the factorization and for
    Q (the reference's Householder form). The CPU line is the oracle (the
    reference's order, one thread) on n = 1024."""
    try:
        rng = np.random.default_rng(6)
        a_np = rng.standard_normal((n, n))
        b_np = rng.standard_normal((n, nrhs))
        a = torch.from_numpy(a_np).cuda()
        torch.cuda.synchronize()
        qr = la_gpu.QRDecomposition.new_device(a.data_ptr(), n, n, n, ctx)
        qr.free()
        reps, t0 = 2, time.perf_counter()
        for _ in range(reps):
            qr = la_gpu.QRDecomposition.new_device(a.data_ptr(), n, n, n, ctx)
            ctx.synchronize()
            qr.free()
        tf = (time.perf_counter() - t0) / reps
        qr = la_gpu.QRDecomposition.new_device(a.data_ptr(), n, n, n, ctx)
        t1 = time.perf_counter()
        qr.solve(la_gpu.Matrix(b_np, ctx))
        ts = time.perf_counter() - t1
        t1 = time.perf_counter()
        qr.get_q()  # includes the m x m copy to the host
        tq = time.perf_counter() - t1
        qr.free()
        flops = 4.0 / 3.0 * n ** 3
        out = {"workload": "QR factor n=%d (Householder reflections, FAST: blocks of 64 in "
                           "compact WY form), then solve %d RHS and get_q" % (n, nrhs),
               "factor_ms": tf * 1e3, "solve_ms": ts * 1e3, "get_q_ms": tq * 1e3,
               "factor_gflops": flops / tf / 1e9, "flops_basis": "nominal 4/3 n^3",
               "factor_frac_of_fp64_peak": (flops / tf / 1e12 / fp64_peak) if fp64_peak else None,
               "cpu_oracle": None}
        if cpu:
            import oracle
            m = 1024
            c = rng.standard_normal((m, m))
            t2 = time.perf_counter()
            oracle.qr_new(c)
            tc = time.perf_counter() - t2
            out["cpu_oracle"] = {"value": 4.0 / 3.0 * m ** 3 / tc / 1e9, "unit": "GFLOP/s",
                                 "cores": 1, "kind": "port",
                                 "sample": "qr_new at n=1024 in the reference's order, %.1f s" % tc}
        del a
        return out
    except Exception as e:  # this section must not take the benchmark line down with it
        return {"error": "%s: %s" % (type(e).__name__, e)}


def run_read_csv(la_gpu, n=2048):
    """util::read_csv (src/util.rs:9-35) with the f64 parser: the native reader
    (all host threads) on an n x n file of %.17g values, against the oracle
    (the reference's rules restated in Python, one thread) on its first 256
    lines. Host-only work; no GPU."""
    import tempfile
    from oracle import csv_ref
    rng = np.random.default_rng(5)
    a = rng.standard_normal((n, n))
    path = os.path.join(tempfile.gettempdir(), "la_bench_%d.csv" % os.getpid())
    head = path + ".head"
    try:
        with open(path, "w") as f:
            for r in range(n):
                f.write(",".join("%.17g" % v for v in a[r]) + "\n")
        size = os.path.getsize(path)
        la_gpu.read_csv(path)
        reps, t0 = 3, time.perf_counter()
        for _ in range(reps):
            m = la_gpu.read_csv(path)
        t = (time.perf_counter() - t0) / reps
        same = bool(np.array_equal(m.data, a))
        with open(path) as f, open(head, "w") as g:
            for i, line in enumerate(f):
                if i >= 256:
                    break
                g.write(line)
        t1 = time.perf_counter()
        csv_ref.read_csv(head)
        to = time.perf_counter() - t1
        return {"workload": "read_csv of a %d x %d file of %%.17g values (%.1f MB)" % (n, n, size / 1e6),
                "ms": t * 1e3, "mb_per_s": size / t / 1e6, "threads": os.cpu_count(),
                "round_trip_exact": same,
                "cpu_oracle": {"value": os.path.getsize(head) / to / 1e6, "unit": "MB/s",
                               "cores": 1, "kind": "port",
                               "sample": "first 256 lines of the same file"}}
    finally:
        for p in (path, head):
            if os.path.exists(p):
                os.remove(p)


def cpu_baseline(a, n, nrhs, target_s=15.0, threads=1):
    """Times the oracle on a bounded prefix of the same factorization."""
    import oracle
    oracle.build()
    jend = pick_prefix(oracle, a, n, target_s, threads)
    t0 = time.perf_counter()
    oracle.lu_factor(a, j_end=jend, threads=threads)
    dt = time.perf_counter() - t0
    fl = prefix_flops(n, jend)
    gf = fl / dt / 1e9
    return {"value": gf, "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": ("columns [0,%d) of the n=%d left-looking factorization (lu.rs:116-161 "
                       "order), %.2e flops in %.1f s; a full LU+solve at this rate would take "
                       "~%.0f s (extrapolated)" % (jend, n, fl, dt,
                                                   lu_solve_flops(n, nrhs) / gf / 1e9)),
            "seconds": dt}


def householder_conditioned(torch, n, kappa, seed):
    """A = H1 diag(s) H2 on the device: H1, H2 products of 4 reflectors
    I - 2 v v^T / v^T v with v iid N(0,1); s geometric from 1 to 1/kappa."""
    rng = np.random.default_rng(seed)
    s = torch.from_numpy(kappa ** (-np.arange(n) / max(n - 1, 1))).cuda()
    a = torch.diag(s)
    for side in ("right", "left"):
        for _ in range(4):
            v = torch.from_numpy(rng.standard_normal(n)).cuda()
            vv = float(v @ v)
            if side == "right":
                a -= (2.0 / vv) * torch.outer(a @ v, v)
            else:
                a -= (2.0 / vv) * torch.outer(v, v @ a)
    return a.contiguous()


def run_mixed(la_gpu, torch, ctx, n, nrhs=4, kappas=(1e2, 1e6, 1e10), precs=(1, 2, 3, 4, 6),
              reps=5):
    """Mixed-precision LU + FP64 refinement against the plain FP64 LU at size n.
    Every time is the median of `reps` runs (CUDA events on the library's
    stream, after one untimed run) of factor + refined solve."""
    names = {1: "bf16", 2: "fp16", 3: "fp32", 4: "fp8", 6: "fp16x3"}
    flops = lu_solve_flops(n, nrhs)
    rng = np.random.default_rng(3)
    b = torch.from_numpy(rng.standard_normal((n, nrhs))).cuda()
    x = torch.zeros((n, nrhs), dtype=torch.float64, device="cuda")
    results = []
    best_by_kappa = {}
    auto_by_kappa = {}
    for kappa in kappas:
        a = householder_conditioned(torch, n, kappa, 30 + int(round(np.log10(kappa))))
        torch.cuda.synchronize()
        for prec in precs:
            last = {}

            def fixed():
                lu = la_gpu.lu_mixed_new_device(ctx, a.data_ptr(), n, n, prec)
                last["r"] = la_gpu.lu_solve_refined_device(lu, b.data_ptr(), nrhs, nrhs,
                                                           x.data_ptr(), nrhs, max_iters=100,
                                                           tol=5e-15)
                lu.free()

            ms, times = event_ms(torch, fixed, reps=reps)
            code, st = last["r"]
            eta = la_gpu.backward_error_device(ctx, a.data_ptr(), n, x.data_ptr(), nrhs,
                                               b.data_ptr(), nrhs, n, nrhs)
            ok = bool(st.converged) and eta <= 1e-14
            r = {"kappa": kappa, "precision": names[prec], "ms": ms,
                 "ms_min_max": [min(times), max(times)],
                 "gflops": flops / (ms * 1e-3) / 1e9, "iterations": st.iterations,
                 "converged": ok, "eta": eta}
            results.append(r)
            if ok and (kappa not in best_by_kappa or r["ms"] < best_by_kappa[kappa]["ms"]):
                best_by_kappa[kappa] = r
        # automatic precision: the library's choice, then the cascade
        last = {}

        def auto():
            last["r"] = la_gpu.lu_solve_auto_device(ctx, a.data_ptr(), n, n, b.data_ptr(), nrhs,
                                                    nrhs, x.data_ptr(), nrhs, tol=5e-15)

        ms, times = event_ms(torch, auto, reps=reps)
        code, st = last["r"]
        eta = la_gpu.backward_error_device(ctx, a.data_ptr(), n, x.data_ptr(), nrhs,
                                           b.data_ptr(), nrhs, n, nrhs)
        auto_by_kappa[kappa] = {"kappa": kappa,
                                "precision_used": {0: "fp64", 1: "bf16", 2: "fp16", 3: "fp32",
                                                   4: "fp8", 6: "fp16x3"}[st.precision],
                                "ms": ms, "ms_min_max": [min(times), max(times)],
                                "gflops": flops / (ms * 1e-3) / 1e9,
                                "iterations": st.iterations, "fell_back": st.fell_back,
                                "converged": eta <= 1e-14, "eta": eta}
        del a
    # plain FP64 LU + solve on the kappa = 1e2 matrix (one warm-up, 3 timed)
    a = householder_conditioned(torch, n, 1e2, 32)
    torch.cuda.synchronize()

    def plain_step():
        lu = la_gpu.LUDecomposition.new_device(a.data_ptr(), n, n, n, ctx)
        lu.solve_device(b.data_ptr(), nrhs, n, nrhs, x.data_ptr(), nrhs)
        lu.free()

    pms, ptimes = event_ms(torch, plain_step, reps=3)
    plain_eta = la_gpu.backward_error_device(ctx, a.data_ptr(), n, x.data_ptr(), nrhs,
                                             b.data_ptr(), nrhs, n, nrhs)
    plain = {"ms": pms, "ms_min_max": [min(ptimes), max(ptimes)],
             "gflops": flops / (pms * 1e-3) / 1e9, "eta": plain_eta}
    del a
    speed = {("%.0e" % k): (auto_by_kappa[k]["gflops"] / plain["gflops"]
                            if auto_by_kappa[k]["converged"] else None) for k in kappas}
    return {"workload": "mixed-precision LU + FP64 iterative refinement, n=%d, %d RHS, "
                        "A = H1 diag(s) H2 (4 Householder reflectors each), s geometric 1 -> "
                        "1/kappa; nominal flops 2/3 n^3 + 2 n^2 nrhs" % (n, nrhs),
            "timing": "median of %d runs, CUDA events on the library stream, after one "
                      "untimed run (plain FP64: median of 3)" % reps,
            "auto_by_kappa": {("%.0e" % k): v for k, v in auto_by_kappa.items()},
            "speedup_vs_plain_fp64": speed,
            "speedup_basis": "la_lu_solve_auto_device (split-FP16 factors with refinement and "
                             "GMRES-IR, the plain FP64 LU where they do not reach tol; nothing "
                             "chosen after the fact) against the plain FP64 LU + solve, device "
                             "time of factor + solve",
            "max_eta": max([r["eta"] for r in results if r["converged"]] +
                           [v["eta"] for v in auto_by_kappa.values()] + [plain_eta]),
            "plain_fp64": plain, "runs": results,
            "fastest_fixed_precision_by_kappa": {("%.0e" % k): v
                                                 for k, v in best_by_kappa.items()}}


# Refinement target of the batch plans. A plan checks convergence with its own
# uncompensated FP64 residual, which near 1e-14 can understate the backward
# error by about 1e-15; 5e-15 keeps every answer at or below 1e-14 by the
# compensated check below (the single-system runs use the same target).
BATCH_TOL = 5e-15


def all_eta(la_gpu, ctx, torch, systems, da, db, dx):
    """Largest normwise backward error over every system of the batch, each
    by the library's compensated FP64 residual (one device kernel)."""
    eta = torch.empty(len(systems), dtype=torch.float64, device="cuda")
    worst = la_gpu.batch_backward_error_device(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(),
                                               systems, eta.data_ptr())
    del eta
    return worst


def shard(la_gpu, systems, world, rank, da, db, dx):
    """This rank's cost-balanced slice of a batch (la_batch_partition): its
    systems rebased to the slice and views of the device buffers."""
    bounds = la_gpu.batch_partition(systems, world)
    sl, a0, alen, b0, blen = la_gpu.batch_slice(systems, bounds[rank], bounds[rank + 1])
    return sl, da[a0:a0 + alen], db[b0:b0 + blen], dx[b0:b0 + blen], bounds


def sum_over_ranks(dist, value, device="cuda"):
    """The sum of one number per rank, on every rank (the value itself alone)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.item()


def run_batched(la_gpu, torch, ctx, count=20000, seed=4, reps=5, dist=None, world=1, rank=0):
    """Uneven batch: count systems, n uniform in [8, 256], 1-4 RHS, A iid N(0,1)
    plus 0.5 n I on even-indexed systems, B iid N(0,1) (generated on the device,
    seeded). Each arm runs its autotuned plan shape (CTAs per SM x warps per
    system) from a captured CUDA graph; solves/s = count / batch time (median of
    `reps` graph launches, CUDA events). With several GPUs every rank takes a
    cost-balanced contiguous slice of the same batch (no collective in the
    plans) and the batch time is the slowest rank's."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(8, 257, size=count)
    rs = rng.integers(1, 5, size=count)
    systems, na, nb = la_gpu.batch_systems(ns, rs)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    da = torch.randn(na, dtype=torch.float64, device="cuda", generator=gen)
    db = torch.randn(nb, dtype=torch.float64, device="cuda", generator=gen)
    dx = torch.zeros(nb, dtype=torch.float64, device="cuda")
    idx = np.concatenate([s.a_offset + np.arange(s.n) * (s.n + 1)
                          for i, s in enumerate(systems) if i % 2 == 0])
    shift = np.concatenate([np.full(s.n, 0.5 * s.n) for i, s in enumerate(systems) if i % 2 == 0])
    da[torch.from_numpy(idx).cuda()] += torch.from_numpy(shift).cuda()
    torch.cuda.synchronize()
    mine, va, vb, vx, bounds = shard(la_gpu, systems, world, rank, da, db, dx)
    out = {"workload": "uneven batch: %d systems, n uniform in [8, 256], 1-4 RHS, A iid N(0,1) "
                       "+ 0.5 n I on even systems" % count, "count": count,
           "timing": "median of %d graph launches, CUDA events" % reps,
           "ranks": world, "scaling": "strong" if world > 1 else None,
           "systems_per_rank": [bounds[r + 1] - bounds[r] for r in range(world)]}
    for mode, name in ((la_gpu.BATCH_FP64, "plain_fp64"), (la_gpu.BATCH_MIXED, "mixed_ir")):
        ms, c, w, fell, worst = 0.0, 0, 0, 0, 0.0
        if len(mine) > 0:
            c, w, _ = la_gpu.batch_autotune(ctx, va.data_ptr(), vb.data_ptr(), vx.data_ptr(), mine,
                                            mode, tol=BATCH_TOL)
            plan = la_gpu.BatchPlan(ctx, va.data_ptr(), vb.data_ptr(), vx.data_ptr(), mine, mode,
                                    ctas_per_sm=c, warps_per_system=w, tol=BATCH_TOL)
            if dist:
                dist.barrier()
            ms, times = event_ms(torch, plan.run, reps=reps)
            its, eta, fb = plan.stats()
            fell = int(fb.sum())
            worst = all_eta(la_gpu, ctx, torch, mine, va, vb, vx)
            plan.free()
        elif dist:
            dist.barrier()
        ms = max_over_ranks(dist, ms)
        out[name] = {"ms": ms, "solves_per_s": count / (ms * 1e-3), "ctas_per_sm": c,
                     "warps_per_system": w, "fell_back": int(sum_over_ranks(dist, fell)),
                     "max_eta_all": max_over_ranks(dist, worst)}
    out["speedup_solves_per_s"] = (out["mixed_ir"]["solves_per_s"] /
                                   out["plain_fp64"]["solves_per_s"])
    del da, db, dx, va, vb, vx
    torch.cuda.empty_cache()
    return out


def run_selector(la_gpu, torch, ctx, count=50000, seed=7, reps=5, dist=None, world=1, rank=0):
    """Learned precision selector on a held-out Householder-conditioned batch:
    count systems, n uniform in [16, 512], 1-4 RHS, log10 kappa_2 uniform in
    [1, 12] (seed 7; the committed weights were trained on 200,000 systems with
    seeds 1000+). Times, per batch (median of `reps`, CUDA events): the plain
    FP64 plan; the mixed plan with FP32 factors for every system (the method
    without the selector); and the selector path (features + MLP inference +
    per-system class choice + the same mixed plan), everything on the device.
    With several GPUs every rank takes a cost-balanced slice, as for the
    uneven batch."""
    import selector as S
    weights = os.path.join(ROOT, "rust-la_gb300", "selector_weights.npy")
    systems, da, db, dx, kappa = S.conditioned_batch(ctx, count, seed)
    mine, va, vb, vx, bounds = shard(la_gpu, systems, world, rank, da, db, dx)
    cnt = len(mine)
    sel = S.PrecisionSelector.from_file(ctx, weights)
    out = {"workload": "learned selector: %d systems, n uniform in [16, 512], 1-4 RHS, "
                       "A = H1 diag(s) H2, log10 kappa uniform in [1, 12]" % count,
           "count": count, "timing": "median of %d runs, CUDA events" % reps,
           "ranks": world, "scaling": "strong" if world > 1 else None}

    def timed(fn):
        if dist:
            dist.barrier()
        ms = event_ms(torch, fn, reps=reps)[0] if cnt > 0 else 0.0
        return max_over_ranks(dist, ms)

    def worst():
        return max_over_ranks(dist, all_eta(la_gpu, ctx, torch, mine, va, vb, vx) if cnt else 0.0)

    c64 = w64 = 0
    if cnt:
        c64, w64, _ = la_gpu.batch_autotune(ctx, va.data_ptr(), vb.data_ptr(), vx.data_ptr(), mine,
                                            la_gpu.BATCH_FP64, tol=BATCH_TOL)
        p64 = la_gpu.BatchPlan(ctx, va.data_ptr(), vb.data_ptr(), vx.data_ptr(), mine,
                               la_gpu.BATCH_FP64, ctas_per_sm=c64, warps_per_system=w64,
                               tol=BATCH_TOL)
    t64 = timed(p64.run if cnt else None)
    out["plain_fp64"] = {"ms": t64, "solves_per_s": count / (t64 * 1e-3), "ctas_per_sm": c64,
                         "warps_per_system": w64, "max_eta_all": worst()}
    if cnt:
        p64.free()
        plan = la_gpu.BatchPlan(ctx, va.data_ptr(), vb.data_ptr(), vx.data_ptr(), mine,
                                la_gpu.BATCH_MIXED, ctas_per_sm=2, warps_per_system=8,
                                tol=BATCH_TOL)
    fp32 = torch.full((max(cnt, 1),), 2, dtype=torch.int32, device="cuda")
    cls = torch.empty(max(cnt, 1), dtype=torch.int32, device="cuda")
    fbuf = torch.empty((max(cnt, 1), 16), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def fixed():
        plan.select_device(fp32.data_ptr())
        plan.run()

    def choose():
        la_gpu.batch_features_device(ctx, va.data_ptr(), mine, fbuf.data_ptr())
        sel.predict(fbuf, out=cls, sync=False)

    def selected():
        choose()
        plan.select_device(cls.data_ptr())
        plan.run()

    def fell():
        return int(sum_over_ranks(dist, int(plan.stats()[2].sum()) if cnt else 0))

    t32 = timed(fixed)
    out["mixed_fp32_factors"] = {"ms": t32, "solves_per_s": count / (t32 * 1e-3),
                                 "fell_back": fell(), "max_eta_all": worst()}
    tf = timed(choose)
    ts = timed(selected)
    counts = np.bincount(cls[:cnt].cpu().numpy(), minlength=4).astype(np.float64)
    counts = [int(sum_over_ranks(dist, float(c))) for c in counts]
    out["mixed_selector"] = {"ms": ts, "solves_per_s": count / (ts * 1e-3),
                             "features_inference_ms": tf, "fell_back": fell(),
                             "class_counts_fp8_bf16_fp32_fp64": counts,
                             "max_eta_all": worst()}
    if cnt:
        plan.free()
    out["speedup_selector_vs_plain_fp64"] = t64 / ts
    out["speedup_selector_vs_fp32_factors"] = t32 / ts
    del da, db, dx, va, vb, vx
    torch.cuda.empty_cache()
    return out


def summarize(line):
    """The headline figures of every section in one small object."""
    def get(d, *keys):
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    def r3(v):
        return round(v, 3) if isinstance(v, float) else v

    out = {"plain_fp64_gflops": r3(line.get("value")), "e2e_gflops": r3(get(line, "e2e", "value")),
           "gemm_roofline_frac": r3(get(line, "roofline", "frac")),
           "backward_error": line.get("backward_error")}
    mixed = line.get("mixed_ir")
    if isinstance(mixed, dict) and "auto_by_kappa" in mixed:
        out["mixed_auto"] = {k: {"ms": r3(v["ms"]), "precision": v["precision_used"],
                                 "speedup_vs_plain_fp64": r3(get(mixed, "speedup_vs_plain_fp64", k)),
                                 "eta": v["eta"]}
                             for k, v in mixed["auto_by_kappa"].items()}
        out["mixed_plain_fp64_ms"] = r3(get(mixed, "plain_fp64", "ms"))
    bat = line.get("batched_uneven")
    if isinstance(bat, dict) and "speedup_solves_per_s" in bat:
        out["batched"] = {"speedup_solves_per_s": r3(bat["speedup_solves_per_s"]),
                          "mixed_solves_per_s": r3(get(bat, "mixed_ir", "solves_per_s")),
                          "max_eta_all": max(get(bat, "mixed_ir", "max_eta_all"),
                                             get(bat, "plain_fp64", "max_eta_all"))}
    sel = line.get("learned_selector")
    if isinstance(sel, dict) and "speedup_selector_vs_fp32_factors" in sel:
        out["selector"] = {"vs_fp32_factors": r3(sel["speedup_selector_vs_fp32_factors"]),
                           "vs_plain_fp64": r3(sel["speedup_selector_vs_plain_fp64"]),
                           "max_eta_all": max(get(sel, "mixed_selector", "max_eta_all"),
                                              get(sel, "plain_fp64", "max_eta_all"))}
    for key in ("gemm_8192", "cholesky_8192", "qr_2048"):
        sec = line.get(key)
        if isinstance(sec, dict):
            out[key + "_gflops"] = r3(sec.get("gflops", sec.get("factor_gflops")))
    return out


DEFAULT_PANEL_WIDTH = 64  # the library's default LA_OPT_PANEL_WIDTH


def bench_config(args, panel_w, world):
    """The workload's description, identical for this library's line and the
    reference arm's line."""
    return {"workload": WORKLOAD, "n": args.n, "nrhs": args.nrhs, "arith": args.arith,
            "panel_width": panel_w, "parallelism": "replicas" if world > 1 else "1 GPU",
            "l2": "inputs larger than L2 (512 MiB matrix), no flush"}


def dist_setup(args, backend="nccl"):
    """One process per GPU (replicas): (world, rank, local rank, the process
    group module or None when the job has one rank)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group(backend=backend)
        dist = dist_mod
    return world, rank, local, dist


def max_over_ranks(dist, value, device="cuda"):
    """The largest of one float per rank, returned on every rank (the job's
    step time is its slowest replica's); the value itself with no group."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, seconds):
    """Whole-job throughput of independent replicas (weak scaling): every rank
    processed units_per_rank in the job's (slowest) time."""
    return units_per_rank * world / seconds


def run_reference(args):
    # Rank 0 alone times the CPU reference; other ranks exit without work.
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import oracle
    oracle.build()
    n, nrhs = args.n, args.nrhs
    a = np.random.default_rng(2).standard_normal((n, n))
    threads = os.cpu_count() or 1
    # one step = a prefix of the factorization sized to about ref_step_seconds
    jend = pick_prefix(oracle, a, n, args.ref_step_seconds, threads)
    fl = prefix_flops(n, jend)
    for _ in range(args.warmup):
        oracle.lu_factor(a, j_end=jend, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.lu_factor(a, j_end=jend, threads=threads)
    el = time.perf_counter() - t0
    gf = fl * args.steps / el / 1e9
    sample = ("each step: columns [0,%d) of the n=%d left-looking factorization "
              "(lu.rs:116-161 order) on %d threads, %.2e flops" % (jend, n, threads, fl))
    line = {
        "impl": "reference", "metric": METRIC, "value": gf, "unit": "GFLOP/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: A iid N(0,1), seed 2",
        "config": bench_config(args, DEFAULT_PANEL_WIDTH, world),
        "cpu_baseline": {"value": gf, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": gf, "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    world, rank, local, dist = dist_setup(args)
    torch.cuda.set_device(local)
    import la_gpu
    la_gpu.lib()
    n, nrhs, K, W = args.n, args.nrhs, args.steps, args.warmup
    rng = np.random.default_rng(2)
    a_np = rng.standard_normal((n, n))
    b_np = rng.standard_normal((n, nrhs))
    # pinned host copies for the end-to-end leg
    ha = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    hb = torch.empty((n, nrhs), dtype=torch.float64, pin_memory=True)
    hx = torch.empty((n, nrhs), dtype=torch.float64, pin_memory=True)
    ha.numpy()[:] = a_np
    hb.numpy()[:] = b_np
    da = ha.to("cuda")
    db = hb.to("cuda")
    dx = torch.empty((n, nrhs), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    ctx = la_gpu.Context(local, la_gpu.ARITH_EXACT if args.arith == "exact" else la_gpu.ARITH_FAST)
    # A created (non-NULL) stream shared by the library and the timing events.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    fp64_peak = ctx.fp64_peak_tflops()
    panel_w = ctx.get_option(la_gpu.OPT_PANEL_WIDTH)

    def step():
        lu = la_gpu.LUDecomposition.new_device(da.data_ptr(), n, n, n, ctx)
        lu.solve_device(db.data_ptr(), nrhs, n, nrhs, dx.data_ptr(), nrhs)
        lu.free()

    for _ in range(W):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.kernel_launches() - launches0
    clk = clocks.stop()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1) / K
    # Per-phase device times (the roofline's trailing-update time) from
    # separate, untimed steps: the phase events would perturb the timed loop.
    PK = 2
    ctx.set_option(la_gpu.OPT_PROFILE, 1)
    phases = np.zeros(5)
    for _ in range(PK):
        lu = la_gpu.LUDecomposition.new_device(da.data_ptr(), n, n, n, ctx)
        phases += np.array(ctx.phase_ms())
        lu.free()
    ctx.set_option(la_gpu.OPT_PROFILE, 0)
    torch.cuda.synchronize()
    ms = max_over_ranks(dist, ms)
    flops = lu_solve_flops(n, nrhs)
    value = replica_throughput(flops, world, ms * 1e-3) / 1e9

    eta = la_gpu.backward_error_device(ctx, da.data_ptr(), n, dx.data_ptr(), nrhs, db.data_ptr(),
                                       nrhs, n, nrhs)

    # roofline of the trailing-update GEMM: all its launches of one factorization
    gl = trailing_gemm_launches(n, panel_w, lookahead=bool(ctx.get_option(la_gpu.OPT_LOOKAHEAD)))
    flops_gemm, flops_per_launch, bytes_per_launch = gemm_algorithmic(gl)
    gemm_ms = phases[3] / PK
    achieved = flops_gemm / (gemm_ms * 1e-3) / 1e12 if gemm_ms > 0 else None
    roof = {
        "bound": "fp64", "compute_pipe": "FP64 FMA (DFMA): GB300 has no faster FP64 path "
                                         "(no FP64 tensor-core rate above it)",
        "kernel": "gemm_f64_tma_kernel (trailing update A22 -= L21*U12)",
        "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
        "frac": (achieved / fp64_peak) if achieved else None,
        "peak_source": "FP64 FMA issue rate measured live in this process "
                       "(la_probe_fp64_peak); the measured-peaks file has no FP64 figure",
        "traffic": GEMM_TRAFFIC_BYTES_PER_LAUNCH,
        "traffic_unit": "DRAM bytes per launch (mean over the factorization's launches), one "
                        "ncu capture of the same n=8192 factorization",
        "launches_per_factorization": len(gl),
        "algorithmic_flops_per_launch": flops_per_launch,
        "algorithmic_bytes_per_launch": bytes_per_launch,
        "gemm_ms_per_factorization": gemm_ms,
        "phase_ms_per_factorization": {"panel": phases[0] / PK, "row_swaps": phases[1] / PK,
                                       "row_panel_trsm": phases[2] / PK,
                                       "trailing_gemm": phases[3] / PK, "finish": phases[4] / PK,
                                       "note": "device time per phase from 2 untimed, profiled "
                                               "factorizations; the panel overlaps the "
                                               "trailing update"},
    }

    # end-to-end through the host-pointer API, copies included
    def e2e_step():
        lu = la_gpu.LUDecomposition.new(la_gpu.Matrix(ha.numpy(), ctx), ctx)
        x = lu.solve(la_gpu.Matrix(hb.numpy(), ctx))
        hx.numpy()[:] = x.data
        lu.free()

    for _ in range(max(1, W // 2)):
        e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / K
    e2e_s = max_over_ranks(dist, e2e_s)
    e2e = {"value": replica_throughput(flops, world, e2e_s) / 1e9, "unit": "GFLOP/s",
           "h2d_bytes_per_step": 8 * n * n + 8 * n * nrhs, "d2h_bytes_per_step": 8 * n * nrhs,
           "ms_per_step": e2e_s * 1e3}

    gemm = None
    if not args.no_gemm:
        db2 = torch.from_numpy(np.random.default_rng(3).standard_normal((n, n))).cuda()
        dc = torch.empty((n, n), dtype=torch.float64, device="cuda")
        la_gpu.matrix_mul_device(ctx, da.data_ptr(), n, db2.data_ptr(), n, dc.data_ptr(), n, n, n, n)
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        reps = 2
        g0.record(stream)
        for _ in range(reps):
            la_gpu.matrix_mul_device(ctx, da.data_ptr(), n, db2.data_ptr(), n, dc.data_ptr(), n,
                                     n, n, n)
        g1.record(stream)
        torch.cuda.synchronize()
        gms = g0.elapsed_time(g1) / reps
        gemm = {"workload": "C = A*B, 8192^3 f64 (Matrix * Matrix)", "ms": gms,
                "gflops": 2.0 * n ** 3 / (gms * 1e-3) / 1e9,
                "frac_of_fp64_peak": 2.0 * n ** 3 / (gms * 1e-3) / 1e12 / fp64_peak}
        del db2, dc

    chol = None
    if not args.no_cholesky and rank == 0:
        chol = guarded(run_cholesky, la_gpu, torch, ctx, stream, n, nrhs, fp64_peak,
                       cpu_s=0.0 if args.no_cpu else 4.0)

    qrs = None
    if not args.no_qr and rank == 0:
        qrs = run_qr(la_gpu, torch, ctx, cpu=not args.no_cpu, fp64_peak=fp64_peak)

    csv = None
    if not args.no_csv and rank == 0:
        csv = guarded(run_read_csv, la_gpu)

    mixed = None
    if not args.no_mixed:
        mixed = run_mixed(la_gpu, torch, ctx, args.mixed_n)
    batched = None
    if not args.no_batched:
        batched = run_batched(la_gpu, torch, ctx, args.batched_count, dist=dist, world=world,
                              rank=rank)
    selected = None
    if not args.no_selector:
        selected = run_selector(la_gpu, torch, ctx, args.selector_count, dist=dist, world=world,
                                rank=rank)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(a_np, n, nrhs, target_s=args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: A iid N(0,1) f64 n=8192 (seed 2), 16 RHS iid N(0,1)",
            "config": bench_config(args, panel_w, world),
            "solves_per_s": world / (ms * 1e-3),
            "backward_error": eta,
            "gpu_launches": int(launches),
            "roofline": roof,
            "e2e": e2e,
            "clocks": clk,
            "cpu_baseline": cpu,
            "gemm_8192": gemm,
            "cholesky_8192": chol,
            "qr_2048": qrs,
            "read_csv": csv,
            "mixed_ir": mixed,
            "batched_uneven": batched,
            "learned_selector": selected,
            "fp64_peak_tflops": fp64_peak,
        }
        line["summary"] = summarize(line)  # last, so that a tail of the line shows it
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"])
    ap.add_argument("--no-gemm", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-cholesky", action="store_true")
    ap.add_argument("--no-csv", action="store_true")
    ap.add_argument("--no-qr", action="store_true")
    ap.add_argument("--mixed-n", type=int, default=16384)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-count", type=int, default=20000)
    ap.add_argument("--no-selector", action="store_true")
    ap.add_argument("--selector-count", type=int, default=50000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
