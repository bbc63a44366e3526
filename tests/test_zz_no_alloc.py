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
    out = lu.get_packed().data, lu.get_piv(), lu.pospivsign(), lu.is_singular()
    lu.free()
    return out


def test_noalloc_matches_regular_entry_point_twice(lagpu):
    torch = pytest.importorskip("torch")
    ctx = lagpu.Context(0, lagpu.ARITH_FAST)
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(2024)
    for n in (700, 513):  # two calls in a row share the static scratch
        a = rng.standard_normal((n, n))
        lu_na, piv_na, flags = _noalloc(lagpu, torch, a, stream.cuda_stream)
        lu_ref, piv_ref, pos_ref, sing_ref = _regular(lagpu, ctx, a)
        assert np.array_equal(piv_na, piv_ref)
        assert np.allclose(lu_na, lu_ref, rtol=1e-12, atol=1e-12)
        assert bool(flags[0]) == pos_ref
        assert bool(flags[1]) == sing_ref
    ctx.close()


def test_noalloc_rejects_oversize_and_bad_arguments(lagpu):
    lib = lagpu.lib()
    fake = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    assert lib.la_lu_factor_noalloc(None, fake, 16, 16385, 16, fake, fake, fake) == lagpu.UNSUPPORTED
    assert lib.la_lu_factor_noalloc(None, None, 16, 16, 16, fake, fake, fake) == lagpu.INVALID
