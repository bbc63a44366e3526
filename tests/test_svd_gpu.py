"""SVD::direct (src/decomp/svd.rs:454-497) through the C ABI against the oracle:
EXACT arithmetic gives the reference's bits (U, S, V) on the reference's test
matrices, the committed fixtures and larger seeded shapes; FAST arithmetic
reconstructs A and agrees with the oracle's singular values."""
import json
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KATS = json.load(open(os.path.join(HERE, "golden", "svd_kats.json")))["kats"]
SMALL = np.load(os.path.join(HERE, "golden", "svd_small.npz"))
NAMES = sorted({k.rsplit("_", 1)[0] for k in SMALL.files if k.endswith("_a")})


def _svd(lagpu, ctx, a):
    r = lagpu.SVD.direct(a, ctx)
    return r.get_u().data, r.get_s().data, r.get_v().data


@pytest.mark.parametrize("k", [k for k in KATS if k["kind"] != "eig_sym_of_ata_approx"],
                         ids=lambda k: k["ref"])
def test_reference_kats_exact(lagpu, ctx_exact, k):
    a = np.array(k["a"])
    u, s, v = _svd(lagpu, ctx_exact, a)
    ru, rs, rv = oracle.svd_direct(a)
    assert np.array_equal(u, ru) and np.array_equal(s, rs) and np.array_equal(v, rv)
    usv = oracle.matmul(oracle.matmul(u, s), np.ascontiguousarray(v.T))
    assert np.all(np.abs(usv - a) < 1e-6)  # the reference's own check (ApproxEq)


@pytest.mark.parametrize("name", NAMES)
def test_fixtures_exact(lagpu, ctx_exact, name):
    u, s, v = _svd(lagpu, ctx_exact, SMALL[name + "_a"])
    assert np.array_equal(u, SMALL[name + "_u"])
    assert np.array_equal(s, SMALL[name + "_s"])
    assert np.array_equal(v, SMALL[name + "_vs"])


@pytest.mark.parametrize("m,n", [(160, 160), (300, 130), (130, 300), (257, 256)])
def test_larger_shapes_exact(lagpu, ctx_exact, m, n):
    a = np.random.default_rng(m * 3 + n).standard_normal((m, n))
    u, s, v = _svd(lagpu, ctx_exact, a)
    ru, rs, rv = oracle.svd_direct(a)
    assert np.array_equal(u, ru) and np.array_equal(s, rs) and np.array_equal(v, rv)


@pytest.mark.parametrize("m,n", [(200, 200), (300, 120), (120, 300)])
def test_fast_reconstructs_and_matches_singular_values(lagpu, ctx_fast, m, n):
    a = np.random.default_rng(m + 7 * n).standard_normal((m, n))
    u, s, v = _svd(lagpu, ctx_fast, a)
    _, rs, _ = oracle.svd_direct(a)
    k = min(m, n)
    sv, rsv = np.diag(s)[:k], np.diag(rs)[:k]
    assert np.all(np.abs(sv - rsv) <= 1e-12 * rsv[0])
    assert np.max(np.abs(u @ s @ v.T - a)) <= 1e-8 * np.abs(a).max()


def test_panics_and_unsupported(lagpu, ctx_exact):
    with pytest.raises(lagpu.Panic):  # zero singular values: inverse().unwrap() on None
        lagpu.SVD.direct(np.zeros((4, 3)), ctx_exact)
    with pytest.raises(lagpu.LaError) as e:  # A'A with a NaN: the nonsymmetric branch
        lagpu.SVD.direct(np.array([[1.0, np.nan], [2.0, 3.0]]), ctx_exact)
    assert e.value.status == lagpu.UNSUPPORTED
