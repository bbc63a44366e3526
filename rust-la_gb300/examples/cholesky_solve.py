"""Example: Cholesky factor and solve (CholeskyDecomposition::new / solve,
src/decomp/cholesky.rs:56-145) through the C ABI.

    python rust-la_gb300/examples/cholesky_solve.py [n] [nrhs] [fast|exact] [lookahead 1|0]

A = (G + G')/2 + n I with G iid U(-1, 1) (seed 4), symmetric and positive
definite; prints the factor and solve times of the second of two runs (the
first pays the one-time kernel set-up), the launch count and the backward
error. lookahead 0 runs each panel after the trailing update instead of beside
it (LA_OPT_LOOKAHEAD).
"""
import os
import sys
import time

import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import la_gpu  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 8192
    nrhs = int(sys.argv[2]) if len(sys.argv) > 2 else 16
    arith = la_gpu.ARITH_EXACT if len(sys.argv) > 3 and sys.argv[3] == "exact" else la_gpu.ARITH_FAST
    ctx = la_gpu.Context(0, arith=arith)
    if len(sys.argv) > 4:
        ctx.set_option(la_gpu.OPT_LOOKAHEAD, int(sys.argv[4]))
    g = torch.Generator(device="cuda").manual_seed(4)
    x0 = torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    a = (x0 + x0.T) / 2 + n * torch.eye(n, device="cuda", dtype=torch.float64)
    del x0
    b = torch.randn((n, nrhs), generator=g, device="cuda", dtype=torch.float64)
    x = torch.empty_like(b)
    torch.cuda.synchronize()
    for rep in range(2):
        if rep:
            c.free()
        l0 = ctx.kernel_launches()
        t0 = time.perf_counter()
        c = la_gpu.CholeskyDecomposition.new_device(a.data_ptr(), n, n, ctx)
        ctx.synchronize()
        t1 = time.perf_counter()
        if c is None:
            print("None (not symmetric positive definite)")
            return
        c.solve_device(b.data_ptr(), nrhs, n, nrhs, x.data_ptr(), nrhs)
        ctx.synchronize()
        t2 = time.perf_counter()
    eta = la_gpu.backward_error_device(ctx, a.data_ptr(), n, x.data_ptr(), nrhs, b.data_ptr(),
                                       nrhs, n, nrhs)
    print("n=%d nrhs=%d %s factor %.1f ms solve %.1f ms launches=%d eta=%.2e"
          % (n, nrhs, "exact" if arith == la_gpu.ARITH_EXACT else "fast", (t1 - t0) * 1e3,
             (t2 - t1) * 1e3, ctx.kernel_launches() - l0, eta))
    c.free()
    ctx.close()


if __name__ == "__main__":
    main()
