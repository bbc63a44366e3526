"""Learned precision selector on the GPU: the generator's singular values, the
feature kernel and the hand-written MLP kernels (forward, gradients, Adam)
against the CPU oracle, and the gain of selector-chosen factor precisions over
always-FP32 factors on a seeded Householder-conditioned batch."""
import os

import numpy as np
import pytest

import oracle
from oracle import selector_ref as sr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.fixture(scope="module")
def sel_mod(lagpu, torch):
    import selector
    return selector


def _system(lagpu, systems, da, i):
    s = systems[i]
    return da[s.a_offset:s.a_offset + s.n * s.n].reshape(s.n, s.n)


def test_generator_singular_values(lagpu, ctx_fast, torch, sel_mod):
    systems, da, db, dx, kappa = sel_mod.conditioned_batch(ctx_fast, 12, seed=3, n_range=(2, 96),
                                                           log10_kappa=(1.0, 6.0))
    a = da.cpu().numpy()
    for i, s in enumerate(systems):
        sv = np.linalg.svd(_system(lagpu, systems, a, i), compute_uv=False)
        want = kappa[i] ** (-np.arange(s.n) / (s.n - 1))
        assert 10.0 <= kappa[i] <= 1e6
        assert np.allclose(sv, want, rtol=1e-9, atol=1e-12), i


def test_generator_is_reproducible(lagpu, ctx_fast, torch, sel_mod):
    r1 = sel_mod.conditioned_batch(ctx_fast, 5, seed=8, n_range=(16, 64))
    r2 = sel_mod.conditioned_batch(ctx_fast, 5, seed=8, n_range=(16, 64))
    assert torch.equal(r1[1], r2[1]) and torch.equal(r1[2], r2[2])


def test_features_match_oracle(lagpu, ctx_fast, torch, sel_mod):
    systems, da, db, dx, kappa = sel_mod.conditioned_batch(ctx_fast, 24, seed=4, n_range=(1, 512))
    f = sel_mod.features(ctx_fast, systems, da).cpu().numpy()
    a = da.cpu().numpy()
    # FP32 arithmetic on the device against float64 arithmetic on the same FP32
    # matrix: 1e-3 on the log-scale features; the Lanczos condition estimate
    # (feature 15) within 0.1 in log10.
    for i, s in enumerate(systems):
        want = sr.features(_system(lagpu, systems, a, i), s.nrhs)
        assert np.allclose(f[i][:15], want[:15], rtol=1e-3, atol=1e-3), (i, s.n, f[i] - want)
        assert abs(f[i][15] - want[15]) <= 0.1, (i, s.n, f[i][15], want[15])


def _random_mlp_data(torch, m, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((m, 16)).astype(np.float32) * 2 + 1
    y = rng.integers(0, 3, size=m).astype(np.int32)
    return X, y, torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda()


def _set_random_params(lagpu, mlp, seed):
    rng = np.random.default_rng(seed)
    p = (rng.standard_normal(mlp.nparam + 32) * 0.2).astype(np.float32)
    p[mlp.nparam:mlp.nparam + 16] = 1.0
    p[mlp.nparam + 16:] = 2.0
    mlp.set_params(p)
    return p


def test_mlp_gradients_match_oracle(lagpu, ctx_fast, torch):
    mlp = lagpu.Mlp(ctx_fast, seed=1)
    p = _set_random_params(lagpu, mlp, 2)
    X, y, dX, dy = _random_mlp_data(torch, 777, 3)
    torch.cuda.synchronize()
    g, loss = mlp.gradients(dX.data_ptr(), dy.data_ptr(), len(y))
    want_loss, want = sr.mlp_loss_grad(p.astype(np.float64), X, y)
    assert abs(loss - want_loss) <= 1e-5 * max(1.0, abs(want_loss))
    assert np.allclose(g, want, rtol=2e-4, atol=2e-6)
    # and both agree with central differences of the oracle's loss
    idx = np.arange(0, sr.NPARAM, 97)
    assert np.allclose(g[idx], sr.numeric_grad(p.astype(np.float64), X, y, idx), rtol=2e-3,
                       atol=1e-5)
    mlp.free()


def test_mlp_expected_cost_gradients_match_oracle(lagpu, ctx_fast, torch):
    mlp = lagpu.Mlp(ctx_fast, seed=3)
    p = _set_random_params(lagpu, mlp, 4)
    X, y, dX, dy = _random_mlp_data(torch, 777, 5)
    cost = np.random.default_rng(6).random((777, 3)).astype(np.float32) * 2.0
    dc = torch.from_numpy(cost).cuda()
    torch.cuda.synchronize()
    g, loss = mlp.gradients_cost(dX.data_ptr(), dc.data_ptr(), len(y))
    want_loss, want = sr.mlp_cost_grad(p.astype(np.float64), X, cost.astype(np.float64))
    assert abs(loss - want_loss) <= 1e-5 * max(1.0, abs(want_loss))
    assert np.allclose(g, want, rtol=2e-4, atol=2e-6)
    mlp.free()


def test_mlp_predict_matches_oracle(lagpu, ctx_fast, torch):
    mlp = lagpu.Mlp(ctx_fast, seed=5)
    p = _set_random_params(lagpu, mlp, 6)
    X, y, dX, dy = _random_mlp_data(torch, 1000, 7)
    probs = torch.empty((1000, 3), dtype=torch.float32, device="cuda")
    cls = torch.empty(1000, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    mlp.predict(dX.data_ptr(), 1000, probs.data_ptr(), cls.data_ptr())
    ctx_fast.synchronize()
    want = sr.mlp_forward(p.astype(np.float64), X)
    assert np.allclose(probs.cpu().numpy(), want, atol=1e-5)
    c = cls.cpu().numpy()
    sure = np.sort(want, 1)[:, -1] - np.sort(want, 1)[:, -2] > 1e-4
    assert (c[sure] == want.argmax(1)[sure]).all()
    mlp.free()


def test_adam_step_matches_oracle(lagpu, ctx_fast, torch):
    mlp = lagpu.Mlp(ctx_fast, seed=9)
    p = _set_random_params(lagpu, mlp, 10).astype(np.float64)
    X, y, dX, dy = _random_mlp_data(torch, 300, 11)
    torch.cuda.synchronize()
    lr = 1e-2
    m = np.zeros(sr.NPARAM)
    v = np.zeros(sr.NPARAM)
    w = p[:sr.NPARAM].copy()
    for t in range(1, 4):
        _, g = sr.mlp_loss_grad(np.concatenate([w, p[sr.NPARAM:]]), X, y)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        w = w - lr * (m / (1 - 0.9 ** t)) / (np.sqrt(v / (1 - 0.999 ** t)) + 1e-8)
        mlp.train_step(dX.data_ptr(), dy.data_ptr(), 300, lr)
    got = mlp.get_params()[:sr.NPARAM]
    assert np.abs(got - w).max() <= 2e-4
    mlp.free()


def test_training_learns_a_separable_rule(lagpu, ctx_fast, torch, sel_mod):
    rng = np.random.default_rng(12)
    X = rng.standard_normal((6000, 16)).astype(np.float32)
    y = np.where(X[:, 15] < -0.4, 0, np.where(X[:, 15] < 0.6, 1, 2)).astype(np.int32)
    dX = torch.from_numpy(X).cuda()
    s = sel_mod.PrecisionSelector(ctx_fast, seed=13)
    log = s.fit(dX, y, steps=400, lr=3e-3, batch=1024, log_every=100)
    assert log[-1][1] < 0.5 * log[0][1]
    acc = (s.predict(dX).cpu().numpy() == y).mean()
    assert acc >= 0.95


WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "rust-la_gb300",
                       "selector_weights.npy")


def test_gate_sends_scored_systems_to_fp64_pass(lagpu, ctx_fast, torch, sel_mod):
    # la_mlp_set_gate: class 3 exactly where coef . [x, p] + bias >= 0, on the
    # raw features x and the class probabilities p; None turns it off.
    systems, da, db, dx, kappa = sel_mod.conditioned_batch(ctx_fast, 300, seed=31)
    f = sel_mod.features(ctx_fast, systems, da)
    s = sel_mod.PrecisionSelector.from_file(ctx_fast, WEIGHTS, gate=False)
    probs = s.probs(f).cpu().numpy().astype(np.float64)
    plain = s.predict(f).cpu().numpy()
    coef = np.zeros(19, dtype=np.float32)
    coef[15] = 1.0   # log10 of the Lanczos condition estimate
    coef[18] = 0.5   # and the FP32-class probability
    bias = -2.0
    s.set_gate(coef, bias)
    gated = s.predict(f).cpu().numpy()
    x = f.cpu().numpy().astype(np.float64)
    score = x @ coef[:16] + probs @ coef[16:] + bias
    clear = np.abs(score) > 1e-4  # away from the threshold's rounding
    assert np.array_equal(gated[clear & (score >= 0)], np.full((clear & (score >= 0)).sum(), 3))
    assert np.array_equal(gated[clear & (score < 0)], plain[clear & (score < 0)])
    assert 0 < (gated == 3).sum() < len(gated)
    s.set_gate(None)
    assert np.array_equal(s.predict(f).cpu().numpy(), plain)
    with pytest.raises(lagpu.LaError):
        s.set_gate(np.full(19, np.nan, dtype=np.float32), 0.0)


def test_selector_wall_clock_gain_over_fp32_factors(lagpu, ctx_fast, torch, sel_mod):
    """The committed network and gate on a freshly seeded batch of 20,000
    systems: features + inference + the plan with the chosen classes takes
    less device time than the same plan with FP32 factors for every system
    (the method without the selector), medians of 5 runs, and every answer
    ends at eta <= 1e-14."""
    tol = 5e-15
    s = sel_mod.PrecisionSelector.from_file(ctx_fast, WEIGHTS)
    systems, da, db, dx, kappa = sel_mod.conditioned_batch(ctx_fast, 20000, seed=202)
    count = len(systems)
    plan = lagpu.BatchPlan(ctx_fast, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems, 1,
                           ctas_per_sm=2, warps_per_system=8, tol=tol)
    fp32 = torch.full((count,), 2, dtype=torch.int32, device="cuda")
    cls = torch.empty(count, dtype=torch.int32, device="cuda")
    fbuf = torch.empty((count, 16), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    ctx_fast.set_stream(stream.cuda_stream)

    def timed(fn, reps=5):
        fn()
        out = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1))
        return float(np.median(out))

    def fixed():
        plan.select_device(fp32.data_ptr())
        plan.run()

    def selected():
        lagpu.batch_features_device(ctx_fast, da.data_ptr(), systems, fbuf.data_ptr())
        s.predict(fbuf, out=cls, sync=False)
        plan.select_device(cls.data_ptr())
        plan.run()

    try:
        t32 = timed(fixed)
        ts = timed(selected)
        eta = torch.empty(count, dtype=torch.float64, device="cuda")
        worst = lagpu.batch_backward_error_device(ctx_fast, da.data_ptr(), db.data_ptr(),
                                                  dx.data_ptr(), systems, eta.data_ptr())
    finally:
        plan.free()
        ctx_fast.set_stream(None)
    print("selector path %.1f ms, FP32 factors everywhere %.1f ms (x%.3f)" % (ts, t32, t32 / ts))
    assert worst <= 1e-14
    assert ts < t32


def test_selector_gain_over_fp32_factors(lagpu, ctx_fast, torch, sel_mod):
    """The trained network (selector_weights.npy: 200,000 labelled systems,
    rust-la_gb300/examples/train_selector.py), without its gate, chooses factor
    precisions for a freshly seeded batch: its choices spend fewer SM cycles
    than FP32 factors for every system (the method without the selector),
    measured system by system, and every answer ends at eta <= 1e-14
    (refinement or the FP64 pass)."""
    tol = 1e-14
    s = sel_mod.PrecisionSelector.from_file(ctx_fast, WEIGHTS, gate=False)
    systems, da, db, dx, kappa = sel_mod.conditioned_batch(ctx_fast, 6000, seed=202)
    cyc, conv = sel_mod.measure_costs(ctx_fast, systems, da, db, dx, tol=tol)
    f = sel_mod.features(ctx_fast, systems, da)
    pred = s.predict(f)
    p = pred.cpu().numpy()
    idx = np.arange(len(p))
    ratio = cyc[idx, p].sum() / cyc[:, 2].sum()
    best = cyc[idx, sel_mod.labels_from_costs(cyc)].sum() / cyc[:, 2].sum()
    # solve with the selector's choices and check the answers
    plan = lagpu.BatchPlan(ctx_fast, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems, 1,
                           ctas_per_sm=2, tol=tol)
    plan.select_device(pred.data_ptr())
    dx.zero_()
    torch.cuda.synchronize()
    plan.run()
    ctx_fast.synchronize()
    plan.free()
    x, a, b = dx.cpu().numpy(), da.cpu().numpy(), db.cpu().numpy()
    rng = np.random.default_rng(0)
    for i in rng.choice(len(systems), 60, replace=False):
        si = systems[int(i)]
        xi = x[si.b_offset:si.b_offset + si.n * si.nrhs].reshape(si.n, si.nrhs)
        bi = b[si.b_offset:si.b_offset + si.n * si.nrhs].reshape(si.n, si.nrhs)
        assert oracle.backward_error(_system(lagpu, systems, a, int(i)), xi, bi) <= tol
    print("selector cycles / fp32 cycles = %.3f (best class per system %.3f)" % (ratio, best))
    assert ratio < 0.99
