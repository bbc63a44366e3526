"""Failure detection without a GPU fault: failures injected on the host
(LA_OPT_INJECT_ALLOC_FAIL, LA_OPT_INJECT_IR_STALL), a bounded device wait made
to run out (LA_OPT_INJECT_PANEL_STALL with a short LA_OPT_WAIT_LIMIT_US: the
panel's grid barrier waits for one arrival more than it has CTAs), and the
statuses the C ABI returns for them. Every call that fails must leave the
context usable: the next call on it gives the same answer as before the
failure.

The injected calls run in a child process, so that an unexpected crash in an
error path fails this test alone and not the rest of the GPU suite."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import la_gpu
import torch

out = {}
ctx = la_gpu.Context()
rng = np.random.default_rng(1)
n = 300
a = rng.uniform(-1.0, 1.0, (n, n))
b = rng.uniform(-1.0, 1.0, (n, 2))
x0 = la_gpu.LUDecomposition.new(a, ctx).solve(la_gpu.Matrix(b, ctx)).data

def status(fn):
    try:
        fn()
        return 0
    except la_gpu.LaError as e:
        return e.status

# la_lu_new: its three allocations, one at a time
for k in (1, 2, 3):
    ctx.set_option(la_gpu.OPT_INJECT_ALLOC_FAIL, k)
    out["lu_new_%d" % k] = status(lambda: la_gpu.LUDecomposition.new(a, ctx))
    out["lu_new_%d_msg" % k] = "injected" in ctx.last_error()
    out["lu_new_%d_left" % k] = ctx.get_option(la_gpu.OPT_INJECT_ALLOC_FAIL)
lu = la_gpu.LUDecomposition.new(a, ctx)
out["lu_after"] = bool(np.array_equal(lu.solve(la_gpu.Matrix(b, ctx)).data, x0))
# la_lu_solve: its two buffers
for k in (1, 2):
    ctx.set_option(la_gpu.OPT_INJECT_ALLOC_FAIL, k)
    out["lu_solve_%d" % k] = status(lambda: lu.solve(la_gpu.Matrix(b, ctx)))
out["lu_solve_after"] = bool(np.array_equal(lu.solve(la_gpu.Matrix(b, ctx)).data, x0))
lu.free()
spd = (a + a.T) / 2 + n * np.eye(n)
ctx.set_option(la_gpu.OPT_INJECT_ALLOC_FAIL, 1)
out["chol_new_1"] = status(lambda: la_gpu.CholeskyDecomposition.new(spd, ctx))
c = la_gpu.CholeskyDecomposition.new(spd, ctx)
out["chol_after"] = c is not None
c.free()
for k in (1, 2):
    ctx.set_option(la_gpu.OPT_INJECT_ALLOC_FAIL, k)
    out["qr_new_%d" % k] = status(lambda: la_gpu.QRDecomposition.new(a, ctx))
q = la_gpu.QRDecomposition.new(a, ctx)
out["qr_after"] = q.is_full_rank()
q.free()

# refinement stalls
m = 512
am = rng.standard_normal((m, m)) + 2.0 * np.sqrt(m) * np.eye(m)
bm = rng.standard_normal((m, 2))
ta = torch.from_numpy(am).cuda()
tb = torch.from_numpy(bm).cuda()
tx = torch.zeros((m, 2), dtype=torch.float64, device="cuda")
torch.cuda.synchronize()
lm = la_gpu.lu_mixed_new_device(ctx, ta.data_ptr(), m, m, 3)
ctx.set_option(la_gpu.OPT_INJECT_IR_STALL, 1)
st, stats = la_gpu.lu_solve_refined_device(lm, tb.data_ptr(), 2, 2, tx.data_ptr(), 2,
                                           max_iters=40, tol=5e-15)
out["stall_status"] = st
out["stall_iterations"] = stats.iterations
out["stall_left"] = ctx.get_option(la_gpu.OPT_INJECT_IR_STALL)
st, stats = la_gpu.lu_solve_refined_device(lm, tb.data_ptr(), 2, 2, tx.data_ptr(), 2,
                                           max_iters=40, tol=5e-15)
out["after_stall_status"] = st
out["after_stall_eta"] = stats.eta
lm.free()
ctx.set_option(la_gpu.OPT_INJECT_IR_STALL, 1)  # the split-FP16 stage stalls
st, stats = la_gpu.lu_solve_auto_device(ctx, ta.data_ptr(), m, m, tb.data_ptr(), 2, 2,
                                        tx.data_ptr(), 2, tol=5e-15)
out["auto_status"] = st
out["auto_fell_back"] = stats.fell_back
out["auto_eta"] = la_gpu.backward_error_device(ctx, ta.data_ptr(), m, tx.data_ptr(), 2,
                                               tb.data_ptr(), 2, m, 2)

# A bounded device wait that runs out: the k-th cooperative panel launch of
# the FP64 LU waits for a CTA too many; after 50 ms every CTA gives up and
# returns, the kernels that would apply its interchanges return at entry, and
# the call reports LA_TIMEOUT. The next factorization on the context is normal.
big = np.random.default_rng(77).standard_normal((1024, 1024))
bb = np.random.default_rng(78).standard_normal((1024, 2))
lu0 = la_gpu.LUDecomposition.new(big, ctx)
out["panel_piv0"] = [int(v) for v in lu0.get_piv()]
xb0 = lu0.solve(la_gpu.Matrix(bb, ctx)).data
lu0.free()
ctx.set_option(la_gpu.OPT_WAIT_LIMIT_US, 50000)
out["wait_limit"] = ctx.get_option(la_gpu.OPT_WAIT_LIMIT_US)
for k in (1, 3):
    ctx.set_option(la_gpu.OPT_INJECT_PANEL_STALL, k)
    out["panel_stall_%d" % k] = status(lambda: la_gpu.LUDecomposition.new(big, ctx))
    out["panel_stall_%d_msg" % k] = "gave up" in ctx.last_error()
    out["panel_stall_%d_left" % k] = ctx.get_option(la_gpu.OPT_INJECT_PANEL_STALL)
    lu1 = la_gpu.LUDecomposition.new(big, ctx)
    out["panel_after_%d_piv" % k] = [int(v) for v in lu1.get_piv()]
    out["panel_after_%d_x" % k] = bool(np.array_equal(lu1.solve(la_gpu.Matrix(bb, ctx)).data, xb0))
    lu1.free()
ctx.set_option(la_gpu.OPT_WAIT_LIMIT_US, 0)
ctx.close()
print(json.dumps(out))
"""


def test_injected_failures_return_statuses_and_leave_the_context_usable(lagpu):
    r = subprocess.run([sys.executable, "-c", CHILD, os.path.join(ROOT, "rust-la_gb300")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    la_gpu = lagpu
    nomem, nc = la_gpu.NOMEM, la_gpu.NOT_CONVERGED
    for k in (1, 2, 3):
        assert out["lu_new_%d" % k] == nomem
        assert out["lu_new_%d_msg" % k]
        assert out["lu_new_%d_left" % k] == 0
    assert out["lu_after"]
    assert out["lu_solve_1"] == nomem and out["lu_solve_2"] == nomem
    assert out["lu_solve_after"]
    assert out["chol_new_1"] == nomem and out["chol_after"]
    assert out["qr_new_1"] == nomem and out["qr_new_2"] == nomem and out["qr_after"]
    assert out["stall_status"] == nc
    assert out["stall_iterations"] == 0
    assert out["stall_left"] == 0
    assert out["after_stall_status"] == la_gpu.OK
    assert out["after_stall_eta"] <= 5e-15
    assert out["auto_status"] == la_gpu.OK
    assert out["auto_fell_back"] == 1
    assert out["auto_eta"] <= 1e-14
    # the wait that ran out, and the same answer afterwards
    import numpy as np
    import oracle
    big = np.random.default_rng(77).standard_normal((1024, 1024))
    ref = [int(v) for v in oracle.lu_factor(big, threads=4).piv]
    assert out["panel_piv0"] == ref
    assert out["wait_limit"] == 50000
    for k in (1, 3):
        assert out["panel_stall_%d" % k] == la_gpu.TIMEOUT
        assert out["panel_stall_%d_msg" % k]
        assert out["panel_stall_%d_left" % k] == 0
        assert out["panel_after_%d_piv" % k] == ref
        assert out["panel_after_%d_x" % k]


def test_injection_options_range(lagpu):
    ctx = lagpu.Context()
    try:
        for opt in (lagpu.OPT_INJECT_ALLOC_FAIL, lagpu.OPT_INJECT_IR_STALL,
                    lagpu.OPT_INJECT_PANEL_STALL, lagpu.OPT_WAIT_LIMIT_US):
            assert ctx.get_option(opt) == 0
            with pytest.raises(lagpu.LaError):
                ctx.set_option(opt, -1)
            ctx.set_option(opt, 3)
            assert ctx.get_option(opt) == 3
            ctx.set_option(opt, 0)
    finally:
        ctx.close()
