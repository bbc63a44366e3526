"""Example: mixed-precision LU + FP64 iterative refinement through the C ABI.

    python rust-la_gb300/examples/mixed_solve.py [n] [precision] [panel]

precision: 1 = BF16, 2 = FP16 (default), 3 = FP32, 4 = split FP8 (e4m3 high and
low parts), 6 = split FP16 trailing updates. panel: the FP32 panel kernel
(LA_OPT_CLUSTER_PANEL: 1 = one thread-block cluster, the default;
0 = cooperative). A is N(0,1) + 2 sqrt(n) I
(seed 3), four right-hand sides; prints the factor and refinement times of the
second of two runs (the first pays the one-time kernel set-up) and the final
backward error.
"""
import os
import sys
import time

import numpy as np
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import la_gpu  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 8192
    prec = int(sys.argv[2]) if len(sys.argv) > 2 else 2
    ctx = la_gpu.Context(0)
    if len(sys.argv) > 3:
        ctx.set_option(la_gpu.OPT_CLUSTER_PANEL, int(sys.argv[3]))
    rng = np.random.default_rng(3)
    a = torch.from_numpy(rng.standard_normal((n, n))).cuda()
    a += 2 * np.sqrt(n) * torch.eye(n, dtype=torch.float64, device="cuda")
    b = torch.from_numpy(rng.standard_normal((n, 4))).cuda()
    x = torch.zeros((n, 4), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        l0 = ctx.kernel_launches()
        t0 = time.perf_counter()
        lu = la_gpu.lu_mixed_new_device(ctx, a.data_ptr(), n, n, prec)
        t1 = time.perf_counter()
        _, st = la_gpu.lu_solve_refined_device(lu, b.data_ptr(), 4, 4, x.data_ptr(), 4,
                                               max_iters=30, tol=5e-15)
        t2 = time.perf_counter()
        lu.free()
    print("n=%d prec=%d panel=%d factor %.1f ms refine %.1f ms iterations=%d eta=%.2e launches=%d"
          % (n, prec, ctx.get_option(la_gpu.OPT_CLUSTER_PANEL), 1e3 * (t1 - t0), 1e3 * (t2 - t1),
             st.iterations, st.eta, ctx.kernel_launches() - l0))


if __name__ == "__main__":
    main()
