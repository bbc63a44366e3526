"""The Cholesky oracle (a CPU restatement of src/decomp/cholesky.rs:56-145) pinned
against the reference crate's own tests (cholesky.rs:147-182, restated in
tests/golden/chol_kats.json), an independent pure-Python restatement, and the
committed fixtures. CPU only."""
import json
import os

import numpy as np
import pytest

import oracle
from oracle import pyref

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "chol_kats.json")))["kats"]
SMALL = np.load(os.path.join(HERE, "golden", "chol_small.npz"))
NAMES = sorted({k.rsplit("_", 1)[0] for k in SMALL.files})


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_lib):
    return oracle_lib


def _approx_eq(x, y):
    # ApproxEq for f64 (src/approxeq.rs:34-47): |x - y| < 1e-6 elementwise
    return np.all(np.abs(np.asarray(x) - np.asarray(y)) < 1e-6)


@pytest.mark.parametrize("k", KATS, ids=[k["ref"] for k in KATS])
def test_reference_kat(k):
    a = np.array(k["a"])
    if k["kind"] == "chol_l_exact":
        lo = oracle.chol_new(a)
        assert lo is not None
        assert np.array_equal(oracle.matmul(lo, lo.T.copy()), a)
        assert lo.ravel().tolist() == k["expect"]
    elif k["kind"] == "chol_none":
        assert oracle.chol_new(a) is None
    elif k["kind"] == "chol_solve_approx":
        lo = oracle.chol_new(a)
        assert _approx_eq(oracle.chol_solve(lo, np.array(k["b"])), k["x"])
    elif k["kind"] == "chol_solve_panic":
        lo = oracle.chol_new(a)
        with pytest.raises(oracle.ReferencePanic):
            oracle.chol_solve(lo, np.array(k["b"]))
    else:
        raise AssertionError(k["kind"])


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 2), (5, 3), (17, 4), (40, 5)])
def test_c_oracle_matches_python_restatement(n, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n))
    a = (g + g.T) / 2 + (n + 8) * np.eye(n)
    b = rng.standard_normal((n, 3))
    lo = oracle.chol_new(a)
    lp = pyref.chol_new(a.tolist())
    assert lo is not None and lp is not None
    assert np.array_equal(lo.ravel(), np.array(lp))
    x = oracle.chol_solve(lo, b)
    xp = pyref.chol_solve(lp, n, b.ravel().tolist(), 3)
    assert np.array_equal(x.ravel(), np.array(xp))


def test_none_rules():
    n = 6
    a = np.eye(n) * 4.0
    a[1, 0] = a[0, 1] = 1.0
    assert oracle.chol_new(a) is not None
    b = a.copy()
    b[4, 2] = 0.5  # the upper twin stays 0: not symmetric
    assert oracle.chol_new(b) is None
    c = a.copy()
    c[3, 3] = 0.0  # d = 0 is not positive
    assert oracle.chol_new(c) is None
    d = a.copy()
    d[5, 1] = d[1, 5] = np.nan  # NaN != NaN: the symmetry test fails
    assert oracle.chol_new(d) is None
    e = a.copy()
    e[2, 2] = np.nan  # NaN on the diagonal is not '<= 0': Some, with NaN in L
    le = oracle.chol_new(e)
    assert le is not None and np.isnan(le[2, 2])
    f = a.copy()
    f[2, 1] = f[1, 2] = -0.0
    f[3, 0], f[0, 3] = 0.0, -0.0  # -0 == +0: symmetric
    assert oracle.chol_new(f) is not None
    assert pyref.chol_new(b.tolist()) is None and pyref.chol_new(c.tolist()) is None


def test_partial_rows_match_full():
    rng = np.random.default_rng(9)
    n = 50
    g = rng.standard_normal((n, n))
    a = (g + g.T) / 2 + n * np.eye(n)
    full = oracle.chol_new(a)
    part = oracle.chol_new(a, j_end=20)
    assert np.array_equal(part[:20], full[:20])


@pytest.mark.parametrize("name", NAMES)
def test_golden_fixtures_reproduce(name):
    a = SMALL[name + "_a"]
    lo = oracle.chol_new(a)
    assert (lo is not None) == bool(SMALL[name + "_some"][0])
    if lo is not None:
        assert np.array_equal(lo, SMALL[name + "_l"])
        assert np.array_equal(oracle.chol_solve(lo, SMALL[name + "_b"]), SMALL[name + "_x"])
