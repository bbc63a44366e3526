"""The two schedules of the triangular solves of LUDecomposition::solve
(src/decomp/lu.rs:256-275): the persistent wavefront kernel (default) and the
one-launch-per-block-step kernels. Both apply every term of every row in the
reference's order, so their results must be bit-identical in FAST and EXACT
arithmetic; EXACT must also equal the oracle's solve bit for bit.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle(oracle_lib):
    return oracle_lib


def _solve(lagpu, a, b, arith, wave):
    ctx = lagpu.Context(arith=arith)
    lu = None
    try:
        ctx.set_option(lagpu.OPT_SOLVE_WAVE, wave)
        assert ctx.get_option(lagpu.OPT_SOLVE_WAVE) == wave
        lu = lagpu.LUDecomposition.new(a, ctx)
        return lu.solve(lagpu.Matrix(b, ctx)).data
    finally:
        # The factorization belongs to the context: free it first.
        if lu is not None:
            lu.free()
        ctx.close()


CASES = [(1, 1), (5, 3), (31, 4), (32, 5), (33, 16), (97, 17), (300, 1), (1000, 8), (2049, 16)]


@pytest.mark.parametrize("n,nrhs", CASES, ids=["n%d-r%d" % c for c in CASES])
@pytest.mark.parametrize("arith", ["fast", "exact"])
def test_wave_matches_block_steps(lagpu, n, nrhs, arith):
    rng = np.random.default_rng(70 * n + nrhs)
    a = rng.uniform(-1, 1, size=(n, n))
    b = rng.standard_normal((n, nrhs))
    mode = lagpu.ARITH_FAST if arith == "fast" else lagpu.ARITH_EXACT
    x_wave = _solve(lagpu, a, b, mode, 2)
    x_step = _solve(lagpu, a, b, mode, 0)
    assert np.array_equal(x_wave.view(np.uint64), x_step.view(np.uint64))
    if arith == "exact" and n <= 300:
        ref = oracle.lu_factor(a)
        assert np.array_equal(x_wave, oracle.solve(ref, b))
    else:
        assert oracle.backward_error(a, x_wave, b) <= 1e-14


@pytest.mark.parametrize("wave", [1, 4, 8])
def test_wave_occupancy_settings_agree(lagpu, wave):
    """The number of resident CTAs changes which CTA takes which item, never a value."""
    rng = np.random.default_rng(5)
    n, nrhs = 3000, 16
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, nrhs))
    x0 = _solve(lagpu, a, b, lagpu.ARITH_FAST, 0)
    x1 = _solve(lagpu, a, b, lagpu.ARITH_FAST, wave)
    assert np.array_equal(x0.view(np.uint64), x1.view(np.uint64))


def test_many_rhs_take_the_block_steps(lagpu):
    """More than 4 * 1024 right-hand sides exceed the progress counters and run
    the block-step schedule; the result is the reference's, bit for bit."""
    rng = np.random.default_rng(11)
    n, nrhs = 48, 4100
    a = rng.uniform(-1, 1, size=(n, n))
    b = rng.uniform(-1, 1, size=(n, nrhs))
    x = _solve(lagpu, a, b, lagpu.ARITH_EXACT, 2)
    ref = oracle.lu_factor(a)
    assert np.array_equal(x, oracle.solve(ref, b))


def test_solve_wave_option_range(lagpu):
    ctx = lagpu.Context()
    try:
        assert ctx.get_option(lagpu.OPT_SOLVE_WAVE) == 2
        with pytest.raises(Exception):
            ctx.set_option(lagpu.OPT_SOLVE_WAVE, 9)
        with pytest.raises(Exception):
            ctx.set_option(lagpu.OPT_SOLVE_WAVE, -1)
    finally:
        ctx.close()
