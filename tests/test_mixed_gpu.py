"""Mixed-precision path: the tcgen05 trailing-update kernel against an FP64
reference of the same op, and the FP32-factor LU with FP64 iterative refinement
reaching a normwise backward error <= 1e-14 (checked with the oracle's
compensated residual)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
ETA_MAX = 1e-14


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("fmt", [1, 2], ids=["bf16", "fp16"])
@pytest.mark.parametrize("mnk", [(128, 128, 64), (1, 1, 16), (200, 300, 100), (256, 384, 256),
                                 (1000, 130, 512), (129, 257, 8)])
def test_tc_update_matches_fp64_reference(lagpu, ctx_fast, torch, fmt, mnk):
    m, n, k = mnk
    dt = torch.bfloat16 if fmt == 1 else torch.float16
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    ldk = (k + 7) // 8 * 8
    ldc = (n + 3) // 4 * 4
    a = torch.zeros((m, ldk), dtype=dt, device="cuda")
    b = torch.zeros((n, ldk), dtype=dt, device="cuda")
    a[:, :k] = torch.randn((m, k), generator=g, device="cuda").to(dt)
    b[:, :k] = torch.randn((n, k), generator=g, device="cuda").to(dt)
    c = torch.randn((m, ldc), generator=g, device="cuda", dtype=torch.float32)
    alpha = 0.75
    ref = c[:, :n].double() - alpha * (a[:, :k].double() @ b[:, :k].double().T)
    torch.cuda.synchronize()
    lagpu.lowp_update_device(ctx_fast, fmt, m, n, k, a.data_ptr(), ldk, b.data_ptr(), ldk,
                             c.data_ptr(), ldc, alpha)
    got = c[:, :n].double()
    scale = 1.0 + alpha * (a[:, :k].double().abs() @ b[:, :k].double().abs().T)
    err = ((got - ref).abs() / scale).max().item()
    assert err < 4 * k * 2.0 ** -24 + 1e-6, err
    # columns beyond n in the padded pitch are untouched
    if ldc > n:
        assert torch.isfinite(c[:, n:]).all()


@pytest.mark.parametrize("fmt", [3, 4], ids=["e4m3x3", "fp16x3"])
@pytest.mark.parametrize("mnk", [(128, 128, 128), (1, 1, 16), (200, 300, 100), (256, 384, 256),
                                 (1000, 130, 512), (129, 257, 8)])
def test_tc_update_split_matches_fp64_reference(lagpu, ctx_fast, torch, fmt, mnk):
    # Split operands (high parts in columns [0, k), low parts from column lo,
    # k padded to a 128-byte chunk): C -= alpha (Ah Bh^T + Ah Bl^T + Al Bh^T);
    # FP8 e4m3 by kind::f8f6f4, FP16 by kind::f16.
    m, n, k = mnk
    dt = torch.float8_e4m3fn if fmt == 3 else torch.float16
    st = torch.uint8 if fmt == 3 else torch.int16
    per = 128 if fmt == 3 else 64  # elements per 128-byte chunk
    g = torch.Generator(device="cuda").manual_seed(m * 5 + n * 11 + k + fmt)
    lo = (k + per - 1) // per * per
    ldc = (n + 3) // 4 * 4

    def split(x):
        hi = x.to(dt)
        return hi, (x - hi.float()).to(dt)

    ah, al = split(torch.randn((m, k), generator=g, device="cuda") * 8)
    bh, bl = split(torch.randn((n, k), generator=g, device="cuda") * 8)
    a = torch.zeros((m, 2 * lo), dtype=st, device="cuda")
    b = torch.zeros((n, 2 * lo), dtype=st, device="cuda")
    a[:, :k] = ah.view(st)
    a[:, lo:lo + k] = al.view(st)
    b[:, :k] = bh.view(st)
    b[:, lo:lo + k] = bl.view(st)
    c = torch.randn((m, ldc), generator=g, device="cuda", dtype=torch.float32)
    alpha = 1.0 / 64
    d = lambda t: t.double()
    prod = d(ah) @ d(bh).T + d(ah) @ d(bl).T + d(al) @ d(bh).T
    ref = c[:, :n].double() - alpha * prod
    torch.cuda.synchronize()
    lagpu.lowp_update_device(ctx_fast, fmt, m, n, k, a.data_ptr(), 2 * lo, b.data_ptr(), 2 * lo,
                             c.data_ptr(), ldc, alpha)
    got = c[:, :n].double()
    scale = 1.0 + alpha * (d(ah).abs() @ d(bh).abs().T + d(ah).abs() @ d(bl).abs().T +
                           d(al).abs() @ d(bh).abs().T)
    err = ((got - ref).abs() / scale).max().item()
    assert err < 4 * 3 * k * 2.0 ** -24 + 1e-6, err


def test_tc_update_split_fp8_rejects_overlapping_low_parts(lagpu, ctx_fast, torch):
    # The low parts must start at or beyond k rounded up to a 128-byte chunk.
    a = torch.zeros((128, 128), dtype=torch.uint8, device="cuda")
    c = torch.zeros((128, 128), dtype=torch.float32, device="cuda")
    with pytest.raises(lagpu.LaError) as e:
        lagpu.lowp_update_device(ctx_fast, 3, 128, 128, 96, a.data_ptr(), 128, a.data_ptr(), 128,
                                 c.data_ptr(), 128, 1.0)
    assert e.value.status == lagpu.INVALID


def _problem(n, nrhs, seed, shift=0.0):
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n)) + shift * np.eye(n)
    b = rng.standard_normal((n, nrhs))
    return a, b


@pytest.mark.parametrize("prec", [1, 2, 3, 4, 6], ids=["bf16", "fp16", "fp32", "fp8", "fp16x3"])
@pytest.mark.parametrize("n", [64, 300, 1000, 1536])
def test_mixed_lu_ir_reaches_fp64_backward_error(lagpu, ctx_fast, torch, prec, n):
    a, b = _problem(n, 4, 100 + n, shift=0.0 if prec == 3 else 2.0 * np.sqrt(n))
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    tx = torch.zeros((n, 4), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    lu = lagpu.lu_mixed_new_device(ctx_fast, ta.data_ptr(), n, n, prec)
    st, stats = lagpu.lu_solve_refined_device(lu, tb.data_ptr(), 4, 4, tx.data_ptr(), 4,
                                              max_iters=60, tol=5e-15)
    lu.free()
    x = tx.cpu().numpy()
    assert st == lagpu.OK, (stats.iterations, stats.eta)
    assert oracle.backward_error(a, x, b) <= ETA_MAX
    assert stats.iterations >= 1


def test_mixed_fp32_factor_pivots_match_fp32_partial_pivoting(lagpu, ctx_fast, torch):
    # The FP32 factorization follows partial pivoting on its own FP32 values;
    # on a diagonally dominant matrix no row is swapped at all.
    n = 700
    a, _ = _problem(n, 1, 5, shift=4.0 * n)
    ta = torch.from_numpy(a).cuda()
    lu = lagpu.lu_mixed_new_device(ctx_fast, ta.data_ptr(), n, n, 1)
    assert np.array_equal(lu.get_piv(), np.arange(n, dtype=np.uint64))
    lu.free()


def _hh(torch, n, kappa, seed):
    rng = np.random.default_rng(seed)
    s = torch.from_numpy(kappa ** (-np.arange(n) / (n - 1))).cuda()
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


@pytest.mark.parametrize("prec,kappa", [(1, 1e6), (2, 1e8), (3, 1e10), (4, 1e3), (6, 1e10)],
                         ids=["bf16-1e6", "fp16-1e8", "fp32-1e10", "fp8-1e3", "fp16x3-1e10"])
def test_ill_conditioned_refinement_converges(lagpu, ctx_fast, torch, prec, kappa):
    n = 1024
    a = _hh(torch, n, kappa, 7)
    rng = np.random.default_rng(8)
    b = torch.from_numpy(rng.standard_normal((n, 2))).cuda()
    x = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    lu = lagpu.lu_mixed_new_device(ctx_fast, a.data_ptr(), n, n, prec)
    st, stats = lagpu.lu_solve_refined_device(lu, b.data_ptr(), 2, 2, x.data_ptr(), 2,
                                              max_iters=40, tol=5e-15)
    lu.free()
    assert st == lagpu.OK, (stats.iterations, stats.gmres_steps, stats.eta)
    eta = oracle.backward_error(a.cpu().numpy(), x.cpu().numpy(), b.cpu().numpy())
    assert eta <= ETA_MAX


@pytest.mark.parametrize("n", [1500, 6000, 12000], ids=["rows1", "rows2", "rows4"])
def test_cluster_and_cooperative_fp32_panels_agree(lagpu, torch, n):
    # The FP32 panel kernels implement the same pivoting: identical pivots from
    # the cluster panel (1, 2 and 4 rows per thread held in registers at these
    # sizes) and the cooperative multi-CTA panel.
    rng = np.random.default_rng(44)
    a = torch.from_numpy(rng.standard_normal((n, n))).cuda()
    outs = []
    for cl in (1, 0):
        ctx = lagpu.Context(0)
        ctx.set_option(lagpu.OPT_CLUSTER_PANEL, cl)
        lu = lagpu.lu_mixed_new_device(ctx, a.data_ptr(), n, n, 3)
        outs.append(lu.get_piv())
        lu.free()
        ctx.close()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("kappa,scale,want", [(1e2, 1.0, (6,)), (1e10, 1.0, (6,)),
                                               (1e2, 1e40, (0,))],
                         ids=["kappa1e2", "kappa1e10", "fp32-overflow"])
def test_auto_precision_cascade(lagpu, ctx_fast, torch, kappa, scale, want):
    # Split-FP16 factors (refinement, then GMRES-IR at kappa 1e10); the plain
    # FP64 LU where no FP32 copy of A exists (entries 1e40 overflow FP32);
    # every answer at eta <= 1e-14.
    n = 1024
    a = _hh(torch, n, kappa, 17) * scale
    rng = np.random.default_rng(18)
    b = torch.from_numpy(rng.standard_normal((n, 3))).cuda()
    x = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st, stats = lagpu.lu_solve_auto_device(ctx_fast, a.data_ptr(), n, n, b.data_ptr(), 3, 3,
                                           x.data_ptr(), 3, tol=5e-15)
    assert st == lagpu.OK
    assert stats.precision in want, (stats.precision, stats.iterations, stats.eta)
    assert stats.fell_back == (1 if stats.precision == 0 else 0)
    eta = oracle.backward_error(a.cpu().numpy(), x.cpu().numpy(), b.cpu().numpy())
    assert eta <= ETA_MAX


def test_auto_precision_singular_and_limits(lagpu, ctx_fast, torch):
    n = 64
    a = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    a[:, :n - 1] = torch.randn((n, n - 1), dtype=torch.float64, device="cuda")
    b = torch.ones((n, 1), dtype=torch.float64, device="cuda")
    x = torch.zeros((n, 17), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st, _ = lagpu.lu_solve_auto_device(ctx_fast, a.data_ptr(), n, n, b.data_ptr(), 1, 1,
                                       x.data_ptr(), 1)
    assert st == lagpu.SINGULAR  # a zero column: the reference's None
    with pytest.raises(lagpu.LaError) as e:
        lagpu.lu_solve_auto_device(ctx_fast, a.data_ptr(), n, n, x.data_ptr(), 17, 17,
                                   x.data_ptr(), 17)
    assert e.value.status == lagpu.UNSUPPORTED


@pytest.mark.parametrize("n,prec", [(1500, 3), (4099, 2), (6000, 6), (9000, 1)],
                         ids=["fp32-1500", "fp16-4099", "fp16x3-6000", "bf16-9000"])
def test_dependent_launches_change_no_bit(lagpu, torch, n, prec):
    # LA_OPT_PDL lets each kernel of the panel chain and of the serial part
    # between outer panels start while the one before it finishes, each
    # waiting on the device for its predecessor's results; the pivots and the
    # refined solution must be the same bits as in plain stream order (1, 2
    # and 4 rows per thread in the cluster panels, odd panel widths at 4099).
    a_np, b_np = _problem(n, 2, 60 + prec, shift=0.0 if prec == 3 else 2.0 * np.sqrt(n))
    a = torch.from_numpy(a_np).cuda()
    b = torch.from_numpy(b_np).cuda()
    outs = []
    for pdl in (0, 1):
        ctx = lagpu.Context(0)
        ctx.set_option(lagpu.OPT_PDL, pdl)
        assert ctx.get_option(lagpu.OPT_PDL) == pdl
        x = torch.zeros((n, 2), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        lu = lagpu.lu_mixed_new_device(ctx, a.data_ptr(), n, n, prec)
        piv = lu.get_piv()
        lagpu.lu_solve_refined_device(lu, b.data_ptr(), 2, 2, x.data_ptr(), 2, max_iters=60,
                                      tol=1e-14)
        lu.free()
        ctx.close()
        outs.append((piv, x.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    assert oracle.backward_error(a_np, outs[1][1], b_np) <= ETA_MAX
