"""GPU parity of the QR path (liblagpu.so through its C ABI) against the oracle
(a restatement of src/decomp/qr.rs:26-238 and src/matrix/mod.rs:1049-1057) and
the reference's own tests (qr.rs:241-260).

Bars: EXACT arithmetic is bit-identical to the reference (R, H, Q, solve,
pinverse). FAST arithmetic (the default) is within 1e-12 relative of it for R,
H and Q, and 1e-9 for solve and pinverse (which go through R and R'R).
"""
import json
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "qr_kats.json")))["kats"]
SMALL = np.load(os.path.join(HERE, "golden", "qr_small.npz"))
NAMES = sorted({k.rsplit("_", 1)[0] for k in SMALL.files if k.endswith("_a")})


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _same_bits(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return x.shape == y.shape and np.array_equal(x.view(np.uint64), y.view(np.uint64))


def _close(x, y, rel=1e-12):
    return x.shape == y.shape and np.abs(x - y).max() <= rel * max(1.0, np.abs(y).max())


@pytest.mark.parametrize("k", KATS, ids=[k["ref"] for k in KATS])
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_reference_kats(lagpu, ctx_exact, ctx_fast, k, mode):
    ctx = ctx_exact if mode == "exact" else ctx_fast
    a = np.array(k["a"])
    qr = lagpu.QRDecomposition.new(a, ctx)
    assert (qr.get_q() * qr.get_r()).approx_eq(lagpu.Matrix(a))
    qr.free()


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_golden_fixtures(lagpu, ctx_exact, ctx_fast, name, mode):
    ctx = ctx_exact if mode == "exact" else ctx_fast
    same = _same_bits if mode == "exact" else _close
    a = SMALL[name + "_a"]
    qr = lagpu.QRDecomposition.new(a, ctx)
    assert same(qr.get_r().data, SMALL[name + "_r"])
    f = oracle.QR(SMALL[name + "_qr"], SMALL[name + "_rdiag"])
    assert same(qr.get_h().data, oracle.qr_get_h(f))
    assert same(qr.get_q().data, SMALL[name + "_q"])
    # solve and pinverse (through R'R) amplify FAST's rounding differences
    loose = _same_bits if mode == "exact" else (lambda x, y: _close(x, y, 1e-9))
    if name + "_x" in SMALL.files:
        assert loose(qr.solve(lagpu.Matrix(SMALL[name + "_b"], ctx)).data, SMALL[name + "_x"])
    if name + "_pinv" in SMALL.files:
        assert loose(lagpu.Matrix(a, ctx).pinverse().data, SMALL[name + "_pinv"])
    qr.free()


@pytest.mark.parametrize("m,n", [(300, 200), (257, 257), (100, 300)])
def test_exact_bitwise_against_oracle(lagpu, ctx_exact, m, n):
    rng = np.random.default_rng(m + 7 * n)
    a = rng.standard_normal((m, n))
    f = oracle.qr_new(a)
    qr = lagpu.QRDecomposition.new(a, ctx_exact)
    assert _same_bits(qr.get_r().data, oracle.qr_get_r(f))
    assert _same_bits(qr.get_q().data, oracle.qr_get_q(f))
    if m == n:
        b = rng.standard_normal((m, 3))
        assert _same_bits(qr.solve(lagpu.Matrix(b, ctx_exact)).data, oracle.qr_solve(f, b))
    qr.free()


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_rank_and_shape_rules(lagpu, ctx_exact, ctx_fast, mode):
    ctx = ctx_exact if mode == "exact" else ctx_fast
    rng = np.random.default_rng(3)
    sq = lagpu.QRDecomposition.new(rng.standard_normal((6, 6)), ctx)
    assert sq.is_full_rank()
    with pytest.raises(lagpu.Panic):
        sq.solve(lagpu.Matrix(np.ones((5, 1)), ctx))  # qr.rs:200
    tall = lagpu.QRDecomposition.new(rng.standard_normal((8, 5)), ctx)
    assert tall.is_full_rank()
    with pytest.raises(lagpu.Panic):
        tall.solve(lagpu.Matrix(np.ones((8, 1)), ctx))  # Matrix::new length assert (:237)
    wide = lagpu.QRDecomposition.new(rng.standard_normal((4, 7)), ctx)
    with pytest.raises(lagpu.Panic):
        wide.is_full_rank()  # rdiag indexed past min(m, n)
    z = rng.standard_normal((5, 5))
    z[:, 2] = 0.0
    zq = lagpu.QRDecomposition.new(z, ctx)
    assert not zq.is_full_rank()
    assert zq.solve(lagpu.Matrix(np.ones((5, 1)), ctx)) is None
    p = rng.standard_normal((12, 4))
    p[:, 1] = 0.0  # R'R singular: inverse() is None, unwrap panics
    with pytest.raises(lagpu.Panic):
        lagpu.Matrix(p, ctx).pinverse()
    for q in (sq, tall, wide, zq):
        q.free()


def test_device_entry_point(lagpu, ctx_exact):
    torch = pytest.importorskip("torch")
    m, n = 200, 120
    a_np = np.random.default_rng(5).standard_normal((m, n))
    a = torch.from_numpy(a_np).cuda()
    torch.cuda.synchronize()
    qr = lagpu.QRDecomposition.new_device(a.data_ptr(), n, m, n, ctx_exact)
    assert _same_bits(qr.get_r().data, oracle.qr_get_r(oracle.qr_new(a_np)))
    qr.free()


# FAST arithmetic from 128 columns on factors in blocks of 64 (compact WY:
# cluster panel, split-K GEMMs, substitutions with V'V), which applies the same
# reflections as the reference with differently ordered sums. Shapes: square
# with zero columns (skipped reflections, qr.rs:62), tall, wide, a ragged last
# block, and the largest rows one cluster holds.
@pytest.mark.parametrize("m,n", [(520, 520), (700, 300), (300, 700), (2100, 130), (6000, 192)])
def test_fast_blocked_against_oracle(lagpu, ctx_fast, m, n):
    rng = np.random.default_rng(m * 3 + n)
    a = rng.standard_normal((m, n))
    if m == n:
        a[:, 70] = 0.0
        a[:, 200] = 0.0
    f = oracle.qr_new(a)
    before = ctx_fast.kernel_launches()
    qr = lagpu.QRDecomposition.new(a, ctx_fast)
    launches = ctx_fast.kernel_launches() - before
    assert launches < 10 * ((min(m, n) + 63) // 64) + 4, "blocked form expected"
    assert _close(qr.get_r().data, oracle.qr_get_r(f), 1e-11)
    assert _close(qr.get_h().data, oracle.qr_get_h(f), 1e-11)
    if m <= 2100:  # Q is m x m
        assert _close(qr.get_q().data, oracle.qr_get_q(f), 1e-11)
    if m >= n:
        assert qr.is_full_rank() == (m != n)
    if m == n:
        assert qr.solve(lagpu.Matrix(np.ones((m, 1)), ctx_fast)) is None
    qr.free()


@pytest.mark.parametrize("n", [256, 1000])
def test_fast_blocked_solve_against_oracle(lagpu, ctx_fast, n):
    # The reference's Q'B step is not orthogonal for a general A (it divides
    # by -u_k where the reflection uses a u_k), so the solution's size grows
    # quickly with n; the bar is relative to it.
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 3))
    f = oracle.qr_new(a)
    qr = lagpu.QRDecomposition.new(a, ctx_fast)
    x = qr.solve(lagpu.Matrix(b, ctx_fast)).data
    qr.free()
    want = oracle.qr_solve(f, b)
    assert np.all(np.isfinite(want))
    assert _close(x, want, 1e-9)
