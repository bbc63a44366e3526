"""GPU parity of the Cholesky path (liblagpu.so through its C ABI) against the
oracle (a restatement of src/decomp/cholesky.rs:56-145) and the reference's own
tests (cholesky.rs:147-182).

Bars: EXACT arithmetic is bit-identical to the reference (L, solve, None).
FAST arithmetic (the default) returns the same Some/None on these matrices, L
within 1e-13 relative of the reference's, and a solve with normwise backward
error eta <= 1e-14.
"""
import json
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "chol_kats.json")))["kats"]
SMALL = np.load(os.path.join(HERE, "golden", "chol_small.npz"))
NAMES = sorted({k.rsplit("_", 1)[0] for k in SMALL.files})
ETA_MAX = 1e-14


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _spd(n, seed, shift=None):
    rng = np.random.default_rng(seed)
    g = rng.uniform(-1.0, 1.0, size=(n, n))
    a = (g + g.T) / 2.0
    a += (n if shift is None else shift) * np.eye(n)
    return a


def _same_bits(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return x.shape == y.shape and np.array_equal(x.view(np.uint64), y.view(np.uint64))


@pytest.mark.parametrize("k", KATS, ids=[k["ref"] for k in KATS])
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_reference_kats(lagpu, ctx_exact, ctx_fast, k, mode):
    ctx = ctx_exact if mode == "exact" else ctx_fast
    a = np.array(k["a"])
    c = lagpu.CholeskyDecomposition.new(a, ctx)
    if k["kind"] == "chol_l_exact":
        lo = c.get_l()
        assert lo * lo.t() == lagpu.Matrix(a)
        assert lo.data.ravel().tolist() == k["expect"]
    elif k["kind"] == "chol_none":
        assert c is None
    elif k["kind"] == "chol_solve_approx":
        assert c.solve(lagpu.Matrix(np.array(k["b"]), ctx)).approx_eq(lagpu.Matrix(np.array(k["x"])))
    elif k["kind"] == "chol_solve_panic":
        with pytest.raises(lagpu.Panic):
            c.solve(lagpu.Matrix(np.array(k["b"]), ctx))
    else:
        raise AssertionError(k["kind"])
    if c is not None:
        c.free()


@pytest.mark.parametrize("name", NAMES)
def test_golden_fixtures_exact(lagpu, ctx_exact, name):
    a = SMALL[name + "_a"]
    c = lagpu.CholeskyDecomposition.new(a, ctx_exact)
    assert (c is not None) == bool(SMALL[name + "_some"][0])
    if c is None:
        return
    assert _same_bits(c.get_l().data, SMALL[name + "_l"])
    assert _same_bits(c.solve(lagpu.Matrix(SMALL[name + "_b"], ctx_exact)).data, SMALL[name + "_x"])
    c.free()


@pytest.mark.parametrize("name", NAMES)
def test_golden_fixtures_fast(lagpu, ctx_fast, name):
    a = SMALL[name + "_a"]
    c = lagpu.CholeskyDecomposition.new(a, ctx_fast)
    assert (c is not None) == bool(SMALL[name + "_some"][0])
    if c is None:
        return
    lo = c.get_l().data
    ref = SMALL[name + "_l"]
    assert np.all(np.triu(lo, 1) == 0.0)
    assert np.abs(lo - ref).max() <= 1e-13 * np.abs(ref).max()
    b = SMALL[name + "_b"]
    x = c.solve(lagpu.Matrix(b, ctx_fast)).data
    assert oracle.backward_error(a, x, b) <= ETA_MAX
    c.free()


@pytest.mark.parametrize("n,nrhs", [(1, 1), (63, 2), (64, 1), (65, 3), (129, 5), (300, 4),
                                    (1000, 9), (2049, 2)])
def test_exact_bitwise_against_oracle(lagpu, ctx_exact, n, nrhs):
    a = _spd(n, 300 + n)
    b = np.random.default_rng(n).standard_normal((n, nrhs))
    ref = oracle.chol_new(a)
    c = lagpu.CholeskyDecomposition.new(a, ctx_exact)
    assert ref is not None and c is not None
    assert _same_bits(c.get_l().data, ref)
    assert _same_bits(c.solve(lagpu.Matrix(b, ctx_exact)).data, oracle.chol_solve(ref, b))
    c.free()


@pytest.mark.parametrize("n,nrhs", [(100, 1), (640, 16), (3000, 4), (4097, 1)])
def test_fast_accuracy(lagpu, ctx_fast, n, nrhs):
    a = _spd(n, 700 + n, shift=2.0 * np.sqrt(n))
    b = np.random.default_rng(n + 1).standard_normal((n, nrhs))
    c = lagpu.CholeskyDecomposition.new(a, ctx_fast)
    assert c is not None
    lo = c.get_l().data
    assert np.all(np.triu(lo, 1) == 0.0)
    # L L' = A to working accuracy (the FP64 GEMM reference is only a check here)
    assert np.abs(lo @ lo.T - a).max() <= 1e-13 * np.abs(a).max()
    x = c.solve(lagpu.Matrix(b, ctx_fast)).data
    assert oracle.backward_error(a, x, b) <= ETA_MAX
    c.free()


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_none_cases(lagpu, ctx_exact, ctx_fast, mode):
    ctx = ctx_exact if mode == "exact" else ctx_fast
    n = 1000
    a = _spd(n, 5)
    assert lagpu.CholeskyDecomposition.new(np.ascontiguousarray(a[:, :999]), ctx) is None
    b = a.copy()
    b[999, 1] = np.nextafter(b[999, 1], 2.0)  # one ulp off its twin, far from the diagonal
    assert lagpu.CholeskyDecomposition.new(b, ctx) is None
    c = a.copy()
    c[700, 700] = -1.0  # not positive definite at row 700
    assert lagpu.CholeskyDecomposition.new(c, ctx) is None
    d = a.copy()
    d[300, 10] = d[10, 300] = np.nan  # NaN != NaN
    assert lagpu.CholeskyDecomposition.new(d, ctx) is None
    e = a.copy()
    e[5, 3], e[3, 5] = 0.0, -0.0  # -0 == +0: still symmetric
    ce = lagpu.CholeskyDecomposition.new(e, ctx)
    assert ce is not None
    ce.free()


def test_nan_on_the_diagonal_is_some_like_the_reference(lagpu, ctx_exact):
    a = _spd(80, 6)
    a[40, 40] = np.nan
    ref = oracle.chol_new(a)
    c = lagpu.CholeskyDecomposition.new(a, ctx_exact)
    assert ref is not None and c is not None
    lo = c.get_l().data
    assert np.array_equal(np.isnan(lo), np.isnan(ref))
    assert _same_bits(np.nan_to_num(lo), np.nan_to_num(ref))
    c.free()


def test_many_rhs_in_chunks(lagpu, ctx_exact, ctx_fast):
    n, nrhs = 40, 4100
    a = _spd(n, 7)
    b = np.random.default_rng(8).standard_normal((n, nrhs))
    ref = oracle.chol_new(a)
    for ctx in (ctx_exact, ctx_fast):
        c = lagpu.CholeskyDecomposition.new(a, ctx)
        x = c.solve(lagpu.Matrix(b, ctx)).data
        if ctx is ctx_exact:
            assert _same_bits(x, oracle.chol_solve(ref, b))
        else:
            assert oracle.backward_error(a, x, b) <= ETA_MAX
        c.free()


def test_device_entry_points(lagpu, ctx_fast):
    torch = pytest.importorskip("torch")
    n, nrhs = 4096, 8
    g = torch.Generator(device="cuda").manual_seed(9)
    x0 = torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
    a = (x0 + x0.T) / 2 + n * torch.eye(n, device="cuda", dtype=torch.float64)
    b = torch.randn((n, nrhs), generator=g, device="cuda", dtype=torch.float64)
    x = torch.empty_like(b)
    torch.cuda.synchronize()
    c = lagpu.CholeskyDecomposition.new_device(a.data_ptr(), n, n, ctx_fast)
    assert c is not None
    c.solve_device(b.data_ptr(), nrhs, n, nrhs, x.data_ptr(), nrhs)
    ctx_fast.synchronize()
    eta = lagpu.backward_error_device(ctx_fast, a.data_ptr(), n, x.data_ptr(), nrhs,
                                      b.data_ptr(), nrhs, n, nrhs)
    assert eta <= ETA_MAX
    with pytest.raises(lagpu.Panic):
        c.solve_device(b.data_ptr(), nrhs, n - 1, nrhs, x.data_ptr(), nrhs)
    c.free()
