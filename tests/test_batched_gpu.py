"""Batched uneven solves (one persistent fused factor + solve kernel in a CUDA
graph): every system's solution reaches a normwise backward error <= 1e-14
(oracle's compensated residual), in plain FP64 and in FP32 + FP64 refinement,
and the FP64 pass takes over where refinement stalls."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
ETA_MAX = 1e-14


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def make_batch(count, seed, nmax=256, shift_even=True):
    rng = np.random.default_rng(seed)
    ns = rng.integers(1, nmax + 1, size=count)
    rs = rng.integers(1, 5, size=count)
    mats, rhss = [], []
    for i, (n, r) in enumerate(zip(ns, rs)):
        a = rng.standard_normal((n, n))
        if shift_even and i % 2 == 0:
            a += 0.5 * n * np.eye(n)
        mats.append(a)
        rhss.append(rng.standard_normal((n, r)))
    return ns, rs, mats, rhss


def run_batch(lagpu, torch, ctx, ns, rs, mats, rhss, mode, ctas=1, precisions=None, warps=8):
    systems, na, nb = lagpu.batch_systems(ns, rs, precisions)
    a = torch.from_numpy(np.concatenate([m.ravel() for m in mats])).cuda()
    b = torch.from_numpy(np.concatenate([r.ravel() for r in rhss])).cuda()
    x = torch.zeros(nb, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    plan = lagpu.BatchPlan(ctx, a.data_ptr(), b.data_ptr(), x.data_ptr(), systems, mode,
                           ctas_per_sm=ctas, warps_per_system=warps, tol=5e-15, max_iters=10)
    x.zero_()
    plan.run()
    its, eta, fb = plan.stats()
    plan.free()
    xs = x.cpu().numpy()
    out = []
    for s, n, r in zip(systems, ns, rs):
        out.append(xs[s.b_offset:s.b_offset + n * r].reshape(n, r))
    return out, its, eta, fb


@pytest.mark.parametrize("mode,ctas,warps,nmax", [
    (0, 1, 8, 256), (0, 2, 4, 256), (0, 4, 2, 128), (1, 1, 8, 256), (1, 2, 8, 256),
    (1, 4, 4, 256), (1, 8, 2, 100)],
    ids=["fp64-1x8", "fp64-2x4", "fp64-4x2", "mixed-1x8", "mixed-2x8", "mixed-4x4", "mixed-8x2"])
def test_batched_backward_error(lagpu, ctx_fast, torch, mode, ctas, warps, nmax):
    # every supported (CTAs per SM, warps per system) shape gives eta <= 1e-14
    ns, rs, mats, rhss = make_batch(160, 11 + ctas + warps, nmax=nmax)
    xs, its, eta, fb = run_batch(lagpu, torch, ctx_fast, ns, rs, mats, rhss, mode, ctas,
                                 warps=warps)
    worst = max(oracle.backward_error(m, x, r) for m, x, r in zip(mats, xs, rhss))
    assert worst <= ETA_MAX
    if mode == 1:
        assert (its >= 0).all()


def test_batched_plan_rejects_shapes_that_do_not_fit(lagpu, ctx_fast, torch):
    # n = 512 in FP64 needs a whole SM's shared memory per CTA
    rng = np.random.default_rng(2)
    ns, rs = [512, 8], [1, 1]
    mats = [rng.standard_normal((n, n)) + n * np.eye(n) for n in ns]
    rhss = [rng.standard_normal((n, r)) for n, r in zip(ns, rs)]
    with pytest.raises(lagpu.LaError) as e:
        run_batch(lagpu, torch, ctx_fast, ns, rs, mats, rhss, 0, ctas=2, warps=4)
    assert e.value.status == lagpu.UNSUPPORTED
    xs, _, _, _ = run_batch(lagpu, torch, ctx_fast, ns, rs, mats, rhss, 0, ctas=1)
    for m, x, r in zip(mats, xs, rhss):
        assert oracle.backward_error(m, x, r) <= ETA_MAX


@pytest.mark.parametrize("prec", ["fp8", "bf16", "fp32", "mixed"])
def test_batched_storage_classes_up_to_512(lagpu, ctx_fast, torch, prec):
    # n up to 512 (global-scratch systems included); every storage class ends at
    # eta <= 1e-14, by refinement or by the FP64 pass.
    rng = np.random.default_rng(21)
    ns = np.concatenate([rng.integers(1, 513, size=40), [512, 511, 300, 1]])
    rs = rng.integers(1, 5, size=len(ns))
    mats, rhss = [], []
    for i, (n, r) in enumerate(zip(ns, rs)):
        a = rng.standard_normal((n, n))
        if i % 3 != 2:
            a += (1.0 + n) * np.eye(n)   # well conditioned: refinement converges
        mats.append(a)
        rhss.append(rng.standard_normal((n, r)))
    code = {"fp8": lagpu.PREC_FP8, "bf16": lagpu.PREC_BF16, "fp32": lagpu.PREC_FP32}
    if prec == "mixed":
        precs = [(lagpu.PREC_FP8, lagpu.PREC_BF16, lagpu.PREC_FP32)[i % 3] for i in range(len(ns))]
    else:
        precs = [code[prec]] * len(ns)
    xs, its, eta, fb = run_batch(lagpu, torch, ctx_fast, ns, rs, mats, rhss, 1, 1, precs)
    for i, (m, x, r) in enumerate(zip(mats, xs, rhss)):
        assert oracle.backward_error(m, x, r) <= ETA_MAX, (i, ns[i], precs[i], fb[i])
    shifted = [i for i in range(len(ns)) if i % 3 != 2]
    if prec == "fp32":
        assert (fb[shifted] == 0).all()   # FP32 factors of shifted systems refine to tol
    if prec == "bf16":
        assert (fb[shifted] == 0).mean() >= 0.8


def test_batched_select_device_and_cycles(lagpu, ctx_fast, torch):
    ns, rs, mats, rhss = make_batch(50, 8, nmax=512)
    systems, na, nb = lagpu.batch_systems(ns, rs)
    a = torch.from_numpy(np.concatenate([m.ravel() for m in mats])).cuda()
    b = torch.from_numpy(np.concatenate([r.ravel() for r in rhss])).cuda()
    x = torch.zeros(nb, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    plan = lagpu.BatchPlan(ctx_fast, a.data_ptr(), b.data_ptr(), x.data_ptr(), systems, 1,
                           tol=5e-15)
    for c in range(3):
        sel = torch.full((len(ns),), c, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        plan.select_device(sel.data_ptr())
        x.zero_()
        torch.cuda.synchronize()
        plan.run()
        cyc = plan.cycles()
        its, eta, fb = plan.stats()
        assert (cyc > 0).all()
        xs = x.cpu().numpy()
        for s, m, r in zip(systems, mats, rhss):
            xi = xs[s.b_offset:s.b_offset + s.n * s.nrhs].reshape(s.n, s.nrhs)
            assert oracle.backward_error(m, xi, r) <= ETA_MAX
    plan.free()


def test_batched_fp64_pivots_match_reference_solution(lagpu, ctx_fast, torch):
    # small systems: the batched FP64 solve equals the oracle's solve to rounding
    ns, rs, mats, rhss = make_batch(40, 3, nmax=40, shift_even=False)
    xs, _, _, _ = run_batch(lagpu, torch, ctx_fast, ns, rs, mats, rhss, 0)
    for m, x, r in zip(mats, xs, rhss):
        ref = oracle.solve(oracle.lu_factor(m), r)
        assert np.allclose(x, ref, rtol=1e-9, atol=1e-9)


def test_batched_mixed_falls_back_on_ill_conditioned(lagpu, ctx_fast, torch):
    # Hilbert-like systems: FP32 factors cannot be refined to 1e-14; the FP64
    # pass must produce the answer.
    ns = [12, 200, 30]
    rs = [1, 2, 4]
    mats, rhss = [], []
    rng = np.random.default_rng(9)
    for n, r in zip(ns, rs):
        i = np.arange(n)
        h = 1.0 / (i[:, None] + i[None, :] + 1.0)
        mats.append(h if n != 200 else rng.standard_normal((n, n)))
        rhss.append(rng.standard_normal((n, r)))
    xs, its, eta, fb = run_batch(lagpu, torch, ctx_fast, ns, rs, mats, rhss, 1)
    assert fb[2] == 1 and fb[1] == 0
    for m, x, r in zip(mats, xs, rhss):
        assert oracle.backward_error(m, x, r) <= ETA_MAX


def test_batch_autotune_writes_table(lagpu, ctx_fast, torch, tmp_path):
    ns, rs, mats, rhss = make_batch(60, 5)
    systems, na, nb = lagpu.batch_systems(ns, rs)
    a = torch.from_numpy(np.concatenate([m.ravel() for m in mats])).cuda()
    b = torch.from_numpy(np.concatenate([r.ravel() for r in rhss])).cuda()
    x = torch.zeros(nb, dtype=torch.float64, device="cuda")
    path = str(tmp_path / "tune.txt")
    best, warps, ms = lagpu.batch_autotune(ctx_fast, a.data_ptr(), b.data_ptr(), x.data_ptr(),
                                           systems, 1, table_path=path)
    assert best in (1, 2, 4, 8) and warps in (2, 4, 8) and ms > 0
    lines = open(path).read().strip().splitlines()
    assert 1 <= len(lines) <= 12 and all(l.startswith("mixed") for l in lines)
    assert (str(best), str(warps)) in [(l.split()[3], l.split()[4]) for l in lines]


def _conditioned(lagpu, ctx, torch, count, seed, n_range, lk):
    import selector
    return selector.conditioned_batch(ctx, count, seed, n_range=n_range, nrhs_range=(1, 2),
                                      log10_kappa=lk)


def _check_all(lagpu, systems, da, db, dx, tol):
    a, b, x = da.cpu().numpy(), db.cpu().numpy(), dx.cpu().numpy()
    for s in systems:
        A = a[s.a_offset:s.a_offset + s.n * s.n].reshape(s.n, s.n)
        B = b[s.b_offset:s.b_offset + s.n * s.nrhs].reshape(s.n, s.nrhs)
        X = x[s.b_offset:s.b_offset + s.n * s.nrhs].reshape(s.n, s.nrhs)
        assert oracle.backward_error(A, X, B) <= tol


def test_batched_gmres_ir_rescues_stalled_refinement(lagpu, torch):
    # BF16 factors on kappa_2 in [1e1, 1e2] with at most 4 LU-IR steps: LU-IR
    # gets below 1e-6 but not to 1e-14; GMRES-IR preconditioned by the same
    # factors finishes and saves FP64 redos. With the stage off the FP64 pass redoes every stalled system.
    # Every answer ends at eta <= 1e-14 either way.
    fbs = {}
    for gmres in (20, 0):
        ctx = lagpu.Context()
        ctx.set_option(lagpu.OPT_BATCH_GMRES, gmres)
        systems, da, db, dx, kappa = _conditioned(lagpu, ctx, torch, 24, 31, (120, 300),
                                                  (1.0, 2.0))
        lagpu.set_precisions(systems, [lagpu.PREC_BF16] * len(systems))
        plan = lagpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems, 1,
                               ctas_per_sm=2, tol=1e-14, max_iters=4)
        its, eta, fbs[gmres] = plan.stats()
        plan.free()
        _check_all(lagpu, systems, da, db, dx, 1e-14)
        ctx.close()
    assert fbs[0].sum() > 0
    assert fbs[20].sum() < fbs[0].sum()


def test_batched_gmres_option_bounds(lagpu):
    ctx = lagpu.Context()
    with pytest.raises(lagpu.LaError):
        ctx.set_option(lagpu.OPT_BATCH_GMRES, 21)
    ctx.set_option(lagpu.OPT_BATCH_GMRES, 5)
    assert ctx.get_option(lagpu.OPT_BATCH_GMRES) == 5
    ctx.close()
