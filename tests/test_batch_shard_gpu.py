"""Sharded batches on one GPU: the slices that la_batch_partition gives to
several GPUs, each run by its own plan over views of its part of the buffers,
reproduce the one-plan answer bit for bit (a system's arithmetic does not
depend on the other systems of its plan). The plans run one after the other;
none waits on another."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("mode,parts", [(0, 2), (1, 3)], ids=["fp64-2", "mixed-3"])
def test_slices_reproduce_the_single_plan(lagpu, ctx_fast, torch, mode, parts):
    rng = np.random.default_rng(31 + parts)
    ns = rng.integers(8, 257, size=400)
    rs = rng.integers(1, 5, size=400)
    systems, na, nb = lagpu.batch_systems(ns, rs)
    g = torch.Generator(device="cuda").manual_seed(9)
    da = torch.randn(na, dtype=torch.float64, device="cuda", generator=g)
    db = torch.randn(nb, dtype=torch.float64, device="cuda", generator=g)
    for i, s in enumerate(systems):
        if i % 2 == 0:
            d = torch.arange(s.n, device="cuda") * (s.n + 1) + s.a_offset
            da[d] += 0.5 * s.n
    x1 = torch.zeros(nb, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    warps = 4 if mode == 0 else 8  # two FP64 CTAs of 8 warps do not fit an SM at n = 256
    plan = lagpu.BatchPlan(ctx_fast, da.data_ptr(), db.data_ptr(), x1.data_ptr(), systems, mode,
                           ctas_per_sm=2, warps_per_system=warps, tol=5e-15)
    plan.run()
    plan.free()
    xs = torch.zeros(nb, dtype=torch.float64, device="cuda")
    bounds = lagpu.batch_partition(systems, parts)
    for p in range(parts):
        sl, a0, alen, b0, blen = lagpu.batch_slice(systems, bounds[p], bounds[p + 1])
        va, vb, vx = da[a0:a0 + alen], db[b0:b0 + blen], xs[b0:b0 + blen]
        pp = lagpu.BatchPlan(ctx_fast, va.data_ptr(), vb.data_ptr(), vx.data_ptr(), sl, mode,
                             ctas_per_sm=2, warps_per_system=warps, tol=5e-15)
        pp.run()
        pp.free()
    torch.cuda.synchronize()
    assert torch.equal(x1, xs)
