"""The allocation-free LU entry point (la_lu_factor_noalloc), called through the
C ABI, against the regular entry point (la_lu_new_device).

It exists for callers whose device memory is owned by someone else (a pool or
framework that forbids cudaMalloc) or that must keep a fixed footprint: they
pass the matrix and output buffers, and the factorization's own scratch sits in
a static device array. This file is collected last so that a failure here
comes after every other test has run.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lagpu, torch, a, stream):
    m, n = a.shape
    lda = n + (n % 2)
    da = torch.zeros((m, lda), dtype=torch.float64, device="cuda")
    da[:, :n] = torch.from_numpy(a)
    ipiv = torch.zeros(min(m, n), dtype=torch.int32, device="cuda")
    piv = torch.zeros(m, dtype=torch.int64, device="cuda")
    flags = torch.zeros(2, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lagpu.lib().la_lu_factor_noalloc(ctypes.c_void_p(stream), ctypes.c_void_p(da.data_ptr()),
                                          lda, m, n, ctypes.c_void_p(ipiv.data_ptr()),
                                          ctypes.c_void_p(piv.data_ptr()),
                                          ctypes.c_void_p(flags.data_ptr()))
    assert st == lagpu.OK
    return (da[:, :n].cpu().numpy(), piv.cpu().numpy().astype(np.uint64),
            flags.cpu().numpy())


def _regular(lagpu, ctx, a):
    lu = lagpu.LUDecomposition.new(a, ctx)
    try:
        singular = lu.is_singular()
    except lagpu.Panic:  # m < n and no zero pivot: the reference indexes past U (lu.rs:174-182)
        singular = False
    out = lu.get_packed().data, lu.get_piv(), lu.pospivsign(), singular
    lu.free()
    return out


def _check_same(lagpu, torch, ctx, a, stream):
    lu_na, piv_na, flags = _noalloc(lagpu, torch, a, stream)
    lu_ref, piv_ref, pos_ref, sing_ref = _regular(lagpu, ctx, a)
    # Both run the same FAST kernels, in which every element takes the same
    # fused multiply-adds in the same order, so the results are identical.
    assert np.array_equal(piv_na, piv_ref)
    assert np.array_equal(lu_na, lu_ref)
    assert bool(flags[0]) == pos_ref
    assert bool(flags[1]) == sing_ref


def test_noalloc_matches_regular_entry_point_twice(lagpu):
    torch = pytest.importorskip("torch")
    ctx = lagpu.Context(0, lagpu.ARITH_FAST)
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(2024)
    for n in (700, 513):  # two calls in a row share the static scratch
        _check_same(lagpu, torch, ctx, rng.standard_normal((n, n)), stream.cuda_stream)
    ctx.close()


@pytest.mark.parametrize("m,n", [(16384, 64), (300, 517), (517, 300), (1, 40), (40, 1)])
def test_noalloc_shapes_and_row_limit(lagpu, m, n):
    # The documented row limit (the 64-CTA panel's shared memory is sized for
    # it), wide matrices (columns right of the last panel) and tall ones.
    torch = pytest.importorskip("torch")
    ctx = lagpu.Context(0, lagpu.ARITH_FAST)
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(m * 7 + n)
    _check_same(lagpu, torch, ctx, rng.standard_normal((m, n)), stream.cuda_stream)
    ctx.close()


def test_noalloc_rejects_oversize_and_bad_arguments(lagpu):
    lib = lagpu.lib()
    fake = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    assert lib.la_lu_factor_noalloc(None, fake, 16, 16385, 16, fake, fake, fake) == lagpu.UNSUPPORTED
    assert lib.la_lu_factor_noalloc(None, None, 16, 16, 16, fake, fake, fake) == lagpu.INVALID
