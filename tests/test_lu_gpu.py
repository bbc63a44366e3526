"""GPU parity of the LU path (liblagpu.so through its C ABI) against the oracle
(a restatement of src/decomp/lu.rs and src/matrix/mod.rs) and the reference's
own known-answer tests.

Bars: EXACT arithmetic is bit-identical to the reference (LU, pivots, sign,
det, solve, inverse, Mul). FAST arithmetic (the default) has the reference's
pivot vector bit for bit on these matrices and a normwise backward error
eta = ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= 1e-14.
"""
import json
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "kats.json")))["kats"]
EPS32 = float(np.finfo(np.float32).eps)
ETA_MAX = 1e-14


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _a(k, key="a"):
    return np.array(k[key], dtype=np.float64)


def run_kat(la, ctx, k, bitwise):
    kind = k["kind"]
    a = la.Matrix(_a(k), ctx)
    if kind == "lu_reconstruct_exact":
        lu = la.LUDecomposition.new(a, ctx)
        lhs = lu.get_l() * lu.get_u()
        rhs = lu.get_p() * a
        if bitwise:
            assert lhs == rhs
        else:
            assert np.allclose(lhs.data, rhs.data, rtol=0, atol=1e-14)
    elif kind in ("solve_approx", "solve_exact"):
        x = la.LUDecomposition.new(a, ctx).solve(la.Matrix(_a(k, "b"), ctx))
        if kind == "solve_exact" and bitwise:
            assert x == la.Matrix(_a(k, "x"))
        else:
            assert x.approx_eq(la.Matrix(_a(k, "x")))
    elif kind == "solve_panic":
        with pytest.raises(la.Panic):
            la.LUDecomposition.new(a, ctx).solve(la.Matrix(_a(k, "b"), ctx))
    elif kind == "solve_none":
        assert la.LUDecomposition.new(a, ctx).solve(la.Matrix(_a(k, "b"), ctx)) is None
    elif kind == "is_singular":
        assert la.LUDecomposition.new(a, ctx).is_singular() == k["expect"]
    elif kind == "is_non_singular":
        assert la.LUDecomposition.new(a, ctx).is_non_singular() == k["expect"]
    elif kind == "matrix_is_non_singular":
        assert a.is_non_singular() == k["expect"]
    elif kind == "matrix_is_singular":
        assert a.is_singular() == k["expect"]
    elif kind == "matrix_is_singular_panic":
        with pytest.raises(la.Panic):
            a.is_singular()
    elif kind == "lu_det_exact":
        assert la.LUDecomposition.new(a, ctx).det() == k["expect"]
    elif kind == "lu_det_panic":
        with pytest.raises(la.Panic):
            la.LUDecomposition.new(a, ctx).det()
    elif kind == "matrix_det_le":
        assert a.det() - k["expect"] <= EPS32
    elif kind == "matrix_det_panic":
        with pytest.raises(la.Panic):
            a.det()
    elif kind == "inverse_approx":
        assert a.inverse().approx_eq(la.Matrix(_a(k, "expect")))
    elif kind == "inverse_panic":
        with pytest.raises(la.Panic):
            a.inverse()
    elif kind == "inverse_none":
        assert a.inverse() is None
    elif kind == "mul_exact":
        assert (a * la.Matrix(_a(k, "b"), ctx)) == la.Matrix(_a(k, "expect"))
    elif kind == "mul_panic":
        with pytest.raises(la.Panic):
            a * la.Matrix(_a(k, "b"), ctx)
    elif kind == "mmul_exact":
        dst = la.Matrix(np.full(k["dst_shape"], np.nan), ctx)
        a.mmul(la.Matrix(_a(k, "b"), ctx), dst)
        assert dst == la.Matrix(_a(k, "expect"))
    elif kind == "mmul_panic":
        dst = la.Matrix(np.zeros(k["dst_shape"]), ctx)
        with pytest.raises(la.Panic):
            a.mmul(la.Matrix(_a(k, "b"), ctx), dst)
    else:
        raise AssertionError(kind)


@pytest.mark.parametrize("k", KATS, ids=lambda k: k["ref"] + ":" + k["kind"])
def test_reference_kats_exact(lagpu, ctx_exact, k):
    run_kat(lagpu, ctx_exact, k, bitwise=True)


@pytest.mark.parametrize("k", KATS, ids=lambda k: k["ref"] + ":" + k["kind"])
def test_reference_kats_fast(lagpu, ctx_fast, k):
    run_kat(lagpu, ctx_fast, k, bitwise=False)


def _golden():
    g = np.load(os.path.join(HERE, "golden", "random_small.npz"))
    return g, sorted({k.rsplit("_", 1)[0] for k in g.files})


def test_golden_fixtures_exact(lagpu, ctx_exact):
    g, names = _golden()
    for name in names:
        lu = lagpu.LUDecomposition.new(g[name + "_a"], ctx_exact)
        assert np.array_equal(lu.get_packed().data, g[name + "_lu"]), name
        assert np.array_equal(lu.get_piv(), g[name + "_piv"]), name
        assert int(lu.pospivsign()) == int(g[name + "_sign"][0]), name
        if name + "_det" in g.files:
            assert lu.det() == g[name + "_det"][0], name
            x = lu.solve(lagpu.Matrix(g[name + "_b"], ctx_exact))
            assert np.array_equal(x.data, g[name + "_x"]), name


def test_golden_fixtures_fast(lagpu, ctx_fast):
    g, names = _golden()
    for name in names:
        a = g[name + "_a"]
        lu = lagpu.LUDecomposition.new(a, ctx_fast)
        assert np.array_equal(lu.get_piv(), g[name + "_piv"]), name
        assert np.allclose(lu.get_packed().data, g[name + "_lu"], rtol=1e-12, atol=1e-12), name
        if name + "_det" in g.files:
            b = g[name + "_b"]
            x = lu.solve(lagpu.Matrix(b, ctx_fast)).data
            assert oracle.backward_error(a, x, b) <= ETA_MAX, name


SIZES = [1, 2, 3, 8, 31, 63, 64, 65, 100, 127, 128, 129, 200, 256, 300]


@pytest.mark.parametrize("n", SIZES)
def test_square_exact_bitwise(lagpu, ctx_exact, n):
    rng = np.random.default_rng(1000 + n)
    a = rng.uniform(-1, 1, size=(n, n))
    b = rng.uniform(-1, 1, size=(n, 2))
    ref = oracle.lu_factor(a)
    lu = lagpu.LUDecomposition.new(a, ctx_exact)
    assert np.array_equal(lu.get_piv(), ref.piv)
    assert np.array_equal(lu.get_packed().data, ref.lu)
    assert lu.pospivsign() == ref.pospivsign
    assert lu.det() == oracle.det(ref)
    assert np.array_equal(lu.solve(lagpu.Matrix(b, ctx_exact)).data, oracle.solve(ref, b))


@pytest.mark.parametrize("n", SIZES)
def test_square_fast(lagpu, ctx_fast, n):
    rng = np.random.default_rng(2000 + n)
    a = rng.uniform(-1, 1, size=(n, n))
    b = rng.uniform(-1, 1, size=(n, 3))
    ref = oracle.lu_factor(a)
    lu = lagpu.LUDecomposition.new(a, ctx_fast)
    assert np.array_equal(lu.get_piv(), ref.piv)
    assert lu.pospivsign() == ref.pospivsign
    x = lu.solve(lagpu.Matrix(b, ctx_fast)).data
    assert oracle.backward_error(a, x, b) <= ETA_MAX
    d, dr = lu.det(), oracle.det(ref)
    assert abs(d - dr) <= 1e-10 * abs(dr) + 1e-300


@pytest.mark.parametrize("seed", list(range(1, 22)))
def test_n512_uniform_pivots_and_eta(lagpu, ctx_fast, seed):
    """The n=512 Uniform[-1,1] case, seed 1 plus twenty more seeds."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, size=(512, 512))
    b = rng.uniform(-1, 1, size=(512, 1))
    ref = oracle.lu_factor(a, threads=8)
    lu = lagpu.LUDecomposition.new(a, ctx_fast)
    assert np.array_equal(lu.get_piv(), ref.piv)
    x = lu.solve(lagpu.Matrix(b, ctx_fast)).data
    assert oracle.backward_error(a, x, b) <= ETA_MAX


def test_n512_exact_bitwise(lagpu, ctx_exact):
    rng = np.random.default_rng(1)
    a = rng.uniform(-1, 1, size=(512, 512))
    b = rng.uniform(-1, 1, size=(512, 1))
    ref = oracle.lu_factor(a, threads=8)
    lu = lagpu.LUDecomposition.new(a, ctx_exact)
    assert np.array_equal(lu.get_packed().data, ref.lu)
    assert np.array_equal(lu.get_piv(), ref.piv)
    assert np.array_equal(lu.solve(lagpu.Matrix(b, ctx_exact)).data, oracle.solve(ref, b))


@pytest.mark.parametrize("shape", [(40, 25), (25, 40), (130, 70), (70, 130), (200, 1), (1, 200),
                                   (129, 128), (128, 129)])
def test_non_square(lagpu, ctx_exact, ctx_fast, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    a = rng.uniform(-1, 1, size=shape)
    ref = oracle.lu_factor(a)
    lu = lagpu.LUDecomposition.new(a, ctx_exact)
    assert np.array_equal(lu.get_packed().data, ref.lu)
    assert np.array_equal(lu.get_piv(), ref.piv)
    assert np.array_equal(lu.get_l().data, oracle.get_l(ref))
    assert np.array_equal(lu.get_u().data, oracle.get_u(ref))
    assert np.array_equal(lu.get_p().data, oracle.get_p(ref))
    with pytest.raises(lagpu.Panic):
        lu.det()
    lf = lagpu.LUDecomposition.new(a, ctx_fast)
    assert np.array_equal(lf.get_piv(), ref.piv)
    m, n = shape
    b = rng.uniform(-1, 1, size=(m, 2))
    if m < n:
        # is_non_singular indexes past the data (lu.rs:177) unless a zero comes first
        with pytest.raises(lagpu.Panic):
            lu.solve(lagpu.Matrix(b, ctx_exact))
    else:
        assert np.array_equal(lu.solve(lagpu.Matrix(b, ctx_exact)).data, oracle.solve(ref, b))


def test_singular_and_zero_pivots(lagpu, ctx_exact, ctx_fast):
    rng = np.random.default_rng(9)
    a = rng.uniform(-1, 1, size=(70, 70))
    a[:, 5] = 0.0          # zero column: pivot 0, scaling skipped (lu.rs:156)
    a[40] = a[3]           # duplicate row
    ref = oracle.lu_factor(a)
    for ctx in (ctx_exact, ctx_fast):
        lu = lagpu.LUDecomposition.new(a, ctx)
        assert np.array_equal(lu.get_piv(), ref.piv)
        assert lu.is_singular()
        assert lu.solve(lagpu.Matrix(np.ones((70, 1)), ctx)) is None
        assert lu.det() == 0.0 or lu.det() == -0.0
    lu = lagpu.LUDecomposition.new(a, ctx_exact)
    assert np.array_equal(lu.get_packed().data, ref.lu)
    assert lagpu.Matrix(a, ctx_exact).inverse() is None


def test_nan_inf_inputs_follow_pivot_rule(lagpu, ctx_exact):
    rng = np.random.default_rng(10)
    for trial in range(4):
        a = rng.uniform(-1, 1, size=(33, 33))
        idx = rng.integers(0, 33, size=(6, 2))
        vals = [np.nan, np.inf, -np.inf, np.nan, 1e308, -0.0]
        for (i, j), v in zip(idx, vals):
            a[i, j] = v
        ref = oracle.lu_factor(a)
        lu = lagpu.LUDecomposition.new(a, ctx_exact)
        assert np.array_equal(lu.get_piv(), ref.piv)
        got = lu.get_packed().data
        assert np.array_equal(np.isnan(got), np.isnan(ref.lu))
        assert np.array_equal(got[~np.isnan(got)], ref.lu[~np.isnan(ref.lu)])


def test_ties_pick_first_row(lagpu, ctx_fast, ctx_exact):
    # many equal magnitudes: the lowest row index must win every time
    a = np.array([[1.0, 2.0, 3.0, 4.0],
                  [-1.0, 2.0, 0.0, 1.0],
                  [1.0, -2.0, 5.0, 0.5],
                  [-1.0, 0.0, 1.0, 9.0]])
    ref = oracle.lu_factor(a)
    for ctx in (ctx_fast, ctx_exact):
        assert np.array_equal(lagpu.LUDecomposition.new(a, ctx).get_piv(), ref.piv)
    big = np.tile(np.arange(1.0, 97.0), (96, 1)) * np.where(np.arange(96) % 2, 1.0, -1.0)[:, None]
    big += np.eye(96) * 0.5
    ref = oracle.lu_factor(big)
    assert np.array_equal(lagpu.LUDecomposition.new(big, ctx_exact).get_piv(), ref.piv)


@pytest.mark.parametrize("n", [1, 3, 64, 65, 150])
def test_inverse(lagpu, ctx_exact, ctx_fast, n):
    rng = np.random.default_rng(300 + n)
    a = rng.uniform(-1, 1, size=(n, n)) + np.eye(n) * 2
    ref = oracle.inverse(a)
    assert np.array_equal(lagpu.Matrix(a, ctx_exact).inverse().data, ref)
    got = lagpu.Matrix(a, ctx_fast).inverse().data
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("mkn", [(1, 1, 1), (2, 2, 2), (3, 5, 7), (64, 64, 64), (65, 33, 17),
                                 (100, 200, 50), (129, 257, 130)])
def test_matrix_mul(lagpu, ctx_exact, ctx_fast, mkn):
    m, k, n = mkn
    rng = np.random.default_rng(m * 31 + k * 7 + n)
    a = rng.standard_normal((m, k))
    b = rng.standard_normal((k, n))
    ref = oracle.matmul(a, b)
    assert np.array_equal((lagpu.Matrix(a, ctx_exact) * lagpu.Matrix(b, ctx_exact)).data, ref)
    got = (lagpu.Matrix(a, ctx_fast) * lagpu.Matrix(b, ctx_fast)).data
    bound = 2 * k * np.finfo(float).eps * (np.abs(a) @ np.abs(b))
    assert np.all(np.abs(got - ref) <= bound)


def test_panel_widths_and_cta_caps_agree(lagpu, ctx_fast):
    rng = np.random.default_rng(77)
    a = rng.uniform(-1, 1, size=(300, 300))
    ref = oracle.lu_factor(a)
    for w in (16, 32, 64):
        for ctas in (0, 3):
            ctx_fast.set_option(lagpu.OPT_PANEL_WIDTH, w)
            ctx_fast.set_option(lagpu.OPT_PANEL_CTAS, ctas)
            assert np.array_equal(lagpu.LUDecomposition.new(a, ctx_fast).get_piv(), ref.piv)
    ctx_fast.set_option(lagpu.OPT_PANEL_WIDTH, 64)
    ctx_fast.set_option(lagpu.OPT_PANEL_CTAS, 0)


def test_exact_mode_panel_widths_bitwise(lagpu, ctx_exact):
    rng = np.random.default_rng(78)
    a = rng.uniform(-1, 1, size=(150, 150))
    ref = oracle.lu_factor(a)
    for w in (16, 32, 64):
        ctx_exact.set_option(lagpu.OPT_PANEL_WIDTH, w)
        assert np.array_equal(lagpu.LUDecomposition.new(a, ctx_exact).get_packed().data, ref.lu)
    ctx_exact.set_option(lagpu.OPT_PANEL_WIDTH, 64)


def test_device_entry_points(lagpu, ctx_fast):
    torch = pytest.importorskip("torch")
    n, nrhs = 257, 5
    rng = np.random.default_rng(5)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, nrhs))
    ta = torch.from_numpy(a).cuda()
    tb = torch.from_numpy(b).cuda()
    tx = torch.empty((n, nrhs), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    lu = lagpu.LUDecomposition.new_device(ta.data_ptr(), n, n, n, ctx_fast)
    assert np.array_equal(lu.get_piv(), oracle.lu_factor(a).piv)
    st = lu.solve_device(tb.data_ptr(), nrhs, n, nrhs, tx.data_ptr(), nrhs)
    assert st == lagpu.OK
    ctx_fast.synchronize()
    x = tx.cpu().numpy()
    assert oracle.backward_error(a, x, b) <= ETA_MAX
    tc = torch.empty((n, nrhs), dtype=torch.float64, device="cuda")
    lagpu.matrix_mul_device(ctx_fast, ta.data_ptr(), n, tb.data_ptr(), nrhs, tc.data_ptr(), nrhs,
                            n, n, nrhs)
    ctx_fast.synchronize()
    assert np.allclose(tc.cpu().numpy(), a @ b, rtol=1e-12, atol=1e-12)


def test_n2048_fast_pivots_and_eta(lagpu, ctx_fast):
    rng = np.random.default_rng(2)
    n = 2048
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 16))
    ref = oracle.lu_factor(a, threads=os.cpu_count() or 4)
    lu = lagpu.LUDecomposition.new(a, ctx_fast)
    assert np.array_equal(lu.get_piv(), ref.piv)
    x = lu.solve(lagpu.Matrix(b, ctx_fast)).data
    assert oracle.backward_error(a, x, b) <= ETA_MAX


def test_lookahead_on_off_agree(lagpu, ctx_fast, ctx_exact):
    rng = np.random.default_rng(91)
    a = rng.uniform(-1, 1, size=(700, 700))
    ref = oracle.lu_factor(a, threads=4)
    for la in (1, 0):
        ctx_fast.set_option(lagpu.OPT_LOOKAHEAD, la)
        assert np.array_equal(lagpu.LUDecomposition.new(a, ctx_fast).get_piv(), ref.piv)
        ctx_exact.set_option(lagpu.OPT_LOOKAHEAD, la)
        assert np.array_equal(lagpu.LUDecomposition.new(a, ctx_exact).get_packed().data, ref.lu)
    ctx_fast.set_option(lagpu.OPT_LOOKAHEAD, 1)
    ctx_exact.set_option(lagpu.OPT_LOOKAHEAD, 1)


@pytest.mark.parametrize("nrhs", [1, 2, 31, 33, 100])
def test_solve_many_rhs(lagpu, ctx_fast, ctx_exact, nrhs):
    rng = np.random.default_rng(400 + nrhs)
    n = 150
    a = rng.uniform(-1, 1, size=(n, n))
    b = rng.uniform(-1, 1, size=(n, nrhs))
    ref = oracle.lu_factor(a)
    xe = lagpu.LUDecomposition.new(a, ctx_exact).solve(lagpu.Matrix(b, ctx_exact)).data
    assert np.array_equal(xe, oracle.solve(ref, b))
    xf = lagpu.LUDecomposition.new(a, ctx_fast).solve(lagpu.Matrix(b, ctx_fast)).data
    assert oracle.backward_error(a, xf, b) <= ETA_MAX


def test_device_backward_error_matches_oracle(lagpu, ctx_fast):
    rng = np.random.default_rng(17)
    n = 300
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 3))
    x = np.linalg.solve(a, b) + rng.standard_normal((n, 3)) * 1e-9
    got = lagpu.backward_error(ctx_fast, a, x, b)
    want = oracle.backward_error(a, x, b)
    assert abs(got - want) <= 1e-3 * want
