"""Example: QR decomposition, Q, solve and pinverse (src/decomp/qr.rs:26-238,
src/matrix/mod.rs:1049-1057) through the C ABI.

    python rust-la_gb300/examples/qr_solve.py [n] [fast|exact]

A is n x n N(0,1) (seed 6); prints the factor, Q and solve times. The
reference's solve is not a least-squares solve for a general A (its Q'B step
divides by -u_k where its reflection uses a * u_k); the library returns the
reference's numbers.
"""
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import la_gpu  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 1024
    arith = la_gpu.ARITH_EXACT if len(sys.argv) > 2 and sys.argv[2] == "exact" else la_gpu.ARITH_FAST
    ctx = la_gpu.Context(0, arith=arith)
    rng = np.random.default_rng(6)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 4))
    t0 = time.perf_counter()
    qr = la_gpu.QRDecomposition.new(a, ctx)
    t1 = time.perf_counter()
    q = qr.get_q().data
    t2 = time.perf_counter()
    x = qr.solve(la_gpu.Matrix(b, ctx))
    t3 = time.perf_counter()
    r = qr.get_r().data
    print("n=%d %s factor %.1f ms, get_q %.1f ms, solve %.1f ms, |QR - A| = %.2e, full rank %s"
          % (n, "exact" if arith == la_gpu.ARITH_EXACT else "fast", (t1 - t0) * 1e3,
             (t2 - t1) * 1e3, (t3 - t2) * 1e3, np.abs(q @ r - a).max(), x is not None))
    qr.free()
    ctx.close()


if __name__ == "__main__":
    main()
