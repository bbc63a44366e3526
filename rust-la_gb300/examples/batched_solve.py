"""Example: batched uneven solves through a captured plan.

    python rust-la_gb300/examples/batched_solve.py [count] [mode] [ctas_per_sm warps_per_system]

count systems (default 20000) with n uniform in [8, 256] and 1-4 right-hand
sides; A iid N(0,1), plus 0.5 n I on even-indexed systems (seed 4). mode 0 =
plain FP64, 1 = FP32 + FP64 refinement (default both). The plan shape is
autotuned unless ctas_per_sm and warps_per_system are given (then the plan
runs once while it is built and five times from its graph, which keeps the
launch sequence short for a profiler). Prints solves/s.
"""
import os
import sys
import time

import numpy as np
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import la_gpu  # noqa: E402


def make(count, seed=4):
    rng = np.random.default_rng(seed)
    ns = rng.integers(8, 257, size=count)
    rs = rng.integers(1, 5, size=count)
    systems, na, nb = la_gpu.batch_systems(ns, rs)
    a = np.empty(na)
    b = rng.standard_normal(nb)
    for i, s in enumerate(systems):
        n = s.n
        m = rng.standard_normal((n, n))
        if i % 2 == 0:
            m += 0.5 * n * np.eye(n)
        a[s.a_offset:s.a_offset + n * n] = m.ravel()
    return systems, a, b


def main():
    count = int(sys.argv[1]) if len(sys.argv) > 1 else 20000
    modes = [int(sys.argv[2])] if len(sys.argv) > 2 else [0, 1]
    systems, a, b = make(count)
    ctx = la_gpu.Context(0)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    dx = torch.zeros_like(db)
    fixed = (int(sys.argv[3]), int(sys.argv[4])) if len(sys.argv) > 4 else None
    for mode in modes:
        if fixed:
            best, warps = fixed
        else:
            best, warps, _ = la_gpu.batch_autotune(ctx, da.data_ptr(), db.data_ptr(),
                                                   dx.data_ptr(), systems, mode)
        plan = la_gpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems, mode,
                                ctas_per_sm=best, warps_per_system=warps)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            plan.run()
        ctx.synchronize()
        dt = (time.perf_counter() - t0) / 5
        its, eta, fb = plan.stats()
        print("mode=%d ctas/SM=%d warps/system=%d %.2f ms/batch %.0f solves/s fell_back=%d "
              "max_iters=%d" % (mode, best, warps, dt * 1e3, count / dt, int(fb.sum()),
                                int(its.max())))
        plan.free()


if __name__ == "__main__":
    main()
