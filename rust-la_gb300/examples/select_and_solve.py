"""Example: learned precision selection for a batch of systems.

    python rust-la_gb300/examples/select_and_solve.py [count] [seed]

count (default 5000) Householder-conditioned systems (n uniform in [16, 512],
1-4 right-hand sides, log10 kappa_2 uniform in [1, 12], seeded). The 16
features per system are computed on the GPU, the committed MLP weights pick
each system's factor storage (FP8, BF16 or FP32), and a mixed batch plan
solves everything with FP64 refinement (the FP64 pass redoes what does not
converge). Prints the class counts, the times of each stage and the number of
systems the FP64 pass redid.
"""
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, ".."))
import la_gpu  # noqa: E402
import selector as S  # noqa: E402


def main():
    count = int(sys.argv[1]) if len(sys.argv) > 1 else 5000
    seed = int(sys.argv[2]) if len(sys.argv) > 2 else 7
    ctx = la_gpu.Context(0)
    systems, da, db, dx, kappa = S.conditioned_batch(ctx, count, seed)
    sel = S.PrecisionSelector.from_file(ctx, os.path.join(HERE, "..", "selector_weights.npy"))
    plan = la_gpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems,
                            la_gpu.BATCH_MIXED, ctas_per_sm=2, warps_per_system=8)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    feats = S.features(ctx, systems, da)
    t1 = time.perf_counter()
    cls = sel.predict(feats)
    t2 = time.perf_counter()
    plan.select_device(cls.data_ptr())
    plan.run()
    ctx.synchronize()
    t3 = time.perf_counter()
    its, eta, fb = plan.stats()
    plan.free()
    counts = np.bincount(cls.cpu().numpy(), minlength=3)
    print("systems=%d classes fp8/bf16/fp32=%s features %.1f ms inference %.1f ms solve %.1f ms "
          "fp64_redone=%d" % (count, counts.tolist(), 1e3 * (t1 - t0), 1e3 * (t2 - t1),
                              1e3 * (t3 - t2), int(fb.sum())))


if __name__ == "__main__":
    main()
