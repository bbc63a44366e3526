"""The SVD::direct oracle (a CPU restatement of src/decomp/svd.rs:454-497 with
the symmetric EigenDecomposition, eigen.rs:33-247 and 755-790) pinned against
the reference crate's own tests (eigen.rs:841-848, svd.rs:532-557, restated in
tests/golden/svd_kats.json), the committed fixtures, and the properties an
eigendecomposition must have. CPU only."""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "svd_kats.json")))["kats"]
SMALL = np.load(os.path.join(HERE, "golden", "svd_small.npz"))
NAMES = sorted({k.rsplit("_", 1)[0] for k in SMALL.files if k.endswith("_a")})


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_lib):
    return oracle_lib


def _approx_eq(x, y):
    return x.shape == y.shape and bool(np.all(np.abs(x - y) < 1e-6))  # approxeq.rs:34-47


@pytest.mark.parametrize("k", KATS, ids=[k["ref"] for k in KATS])
def test_reference_kat(k):
    a = np.array(k["a"])
    if k["kind"] == "eig_sym_of_ata_approx":
        d, e, v = oracle.eig_sym(oracle.matmul(np.ascontiguousarray(a.T), a))
        assert _approx_eq(d, np.array(k["eigenvalues"]))
    else:
        u, s, v = oracle.svd_direct(a)
        usv = oracle.matmul(oracle.matmul(u, s), np.ascontiguousarray(v.T))
        assert _approx_eq(usv, a)


@pytest.mark.parametrize("name", NAMES)
def test_fixtures_reproduce(name):
    a = SMALL[name + "_a"]
    d, e, v = oracle.eig_sym(oracle.matmul(np.ascontiguousarray(a.T), a))
    assert np.array_equal(d, SMALL[name + "_d"])
    assert np.array_equal(v, SMALL[name + "_v"])
    u, s, vs = oracle.svd_direct(a)
    assert np.array_equal(u, SMALL[name + "_u"])
    assert np.array_equal(s, SMALL[name + "_s"])
    assert np.array_equal(vs, SMALL[name + "_vs"])


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 2), (6, 3), (33, 4), (120, 5)])
def test_eigendecomposition_properties(n, seed):
    g = np.random.default_rng(seed).standard_normal((n, n))
    a = g + g.T
    d, e, v = oracle.eig_sym(a)
    assert np.all(np.diff(d) <= 0)  # sorted descending (eigen.rs:226-246)
    assert np.array_equal(e, np.zeros(n))
    assert np.allclose(v.T @ v, np.eye(n), atol=1e-12)
    assert np.allclose(a @ v, v * d, atol=1e-10 * max(1.0, np.abs(d).max()))
    assert np.allclose(d, np.sort(np.linalg.eigvalsh(a))[::-1], atol=1e-10 * np.abs(d).max())


def test_shapes_and_panics():
    rng = np.random.default_rng(9)
    for m, n in ((7, 4), (4, 7), (5, 5)):
        a = rng.standard_normal((m, n))
        u, s, v = oracle.svd_direct(a)
        assert u.shape == (m, m) and s.shape == (m, n) and v.shape == (n, n)
        assert np.allclose(u @ s @ v.T, a, atol=1e-10)
        if m > n:  # U's last m - n columns are zero (S^-1 padded with zero columns, :484-489)
            assert np.array_equal(u[:, n:], np.zeros((m, m - n)))
    with pytest.raises(oracle.ReferencePanic):  # a zero singular value: inverse().unwrap()
        oracle.svd_direct(np.zeros((3, 3)))
    with pytest.raises(ValueError):  # A'A with a NaN: the nonsymmetric branch
        oracle.svd_direct(np.array([[1.0, np.nan], [2.0, 3.0]]))
