"""ORACLE — test infrastructure only.

A CPU restatement of the `la` crate's LU path (xasmx/rust-la 0.2.0,
src/decomp/lu.rs:104-278, src/matrix/mod.rs:957-980 and :1025-1047) and of
its Cholesky decomposition (src/decomp/cholesky.rs:56-145), QR
decomposition (src/decomp/qr.rs:26-238, src/matrix/mod.rs:1049-1057) and
SVD::direct (src/decomp/svd.rs:454-497 with eigen.rs:33-247, 755-790) used by
the tests, the smoke check and the benchmark's CPU-baseline leg as the checker.
Nothing on the product path may import this package.

`liboracle.so` is built from lu_oracle.c / lu_oracle_mt.c / chol_oracle.c / qr_oracle.c / svd_oracle.c by `make` in this
directory (the repository's build step runs it). `pyref` holds an independent
pure-Python restatement used to cross-check the C one on small cases.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

OK, NONE, PANIC = 0, 1, 2


class ReferencePanic(Exception):
    """The reference would panic (a failed `assert!` or an index out of bounds)."""


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        S = ctypes.c_size_t
        I = ctypes.c_int
        L.oracle_lu_factor_partial.argtypes = [P, S, S, S, P, P, P]
        L.oracle_lu_factor.argtypes = [P, S, S, P, P, P]
        L.oracle_lu_is_non_singular.argtypes = [P, S, S]
        L.oracle_lu_is_non_singular.restype = I
        L.oracle_lu_det.argtypes = [P, S, S, I, P]
        L.oracle_lu_det.restype = I
        L.oracle_lu_solve.argtypes = [P, S, S, P, P, S, S, P]
        L.oracle_lu_solve.restype = I
        L.oracle_lu_get_l.argtypes = [P, S, S, P]
        L.oracle_lu_get_u.argtypes = [P, S, S, P]
        L.oracle_lu_get_p.argtypes = [P, S, P]
        L.oracle_matmul_rows.argtypes = [P, S, S, P, S, S, P, S, S]
        L.oracle_matmul_rows.restype = I
        L.oracle_matmul.argtypes = [P, S, S, P, S, S, P]
        L.oracle_matmul.restype = I
        L.oracle_inverse.argtypes = [P, S, S, P, P, P, P]
        L.oracle_inverse.restype = I
        L.oracle_backward_error.argtypes = [P, S, P, P, S]
        L.oracle_backward_error.restype = ctypes.c_double
        L.oracle_mt_max_threads.restype = I
        L.oracle_mt_lu_factor_partial.argtypes = [P, S, S, S, P, P, P, I]
        L.oracle_mt_lu_solve_nocheck.argtypes = [P, S, P, P, S, P, I]
        L.oracle_mt_matmul_rows.argtypes = [P, S, S, P, S, P, S, S, I]
        L.oracle_chol_new_partial.argtypes = [P, S, S, S, P]
        L.oracle_chol_new_partial.restype = I
        L.oracle_chol_solve.argtypes = [P, S, P, S, S, P]
        L.oracle_chol_solve.restype = I
        L.oracle_qr_new.argtypes = [P, S, S, P, P]
        L.oracle_qr_is_full_rank.argtypes = [P, S, S]
        L.oracle_qr_is_full_rank.restype = I
        L.oracle_qr_get_h.argtypes = [P, S, S, P]
        L.oracle_qr_get_r.argtypes = [P, P, S, S, P]
        L.oracle_qr_get_q.argtypes = [P, P, S, S, P]
        L.oracle_qr_solve.argtypes = [P, P, S, S, P, S, S, P]
        L.oracle_qr_solve.restype = I
        L.oracle_eig_sym.argtypes = [P, S, P, P, P]
        L.oracle_eig_sym.restype = I
        L.oracle_svd_direct.argtypes = [P, S, S, P, P, P]
        L.oracle_svd_direct.restype = I
        _LIB = L
    return _LIB


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class LU:
    """Packed LU factors exactly as LUDecomposition holds them (lu.rs:95-101)."""

    def __init__(self, lu, piv, pospivsign):
        self.lu = lu
        self.piv = piv
        self.pospivsign = bool(pospivsign)

    @property
    def m(self):
        return self.lu.shape[0]

    @property
    def n(self):
        return self.lu.shape[1]


def lu_factor(a, j_end=None, threads=0):
    """lu.rs:104-168. `j_end` stops after that many columns (a bounded sample)."""
    a = _c(a)
    m, n = a.shape
    lu = np.empty_like(a)
    piv = np.empty(m, dtype=np.uint64)
    pos = ctypes.c_int(1)
    je = n if j_end is None else min(int(j_end), n)
    if threads and threads > 1:
        lib().oracle_mt_lu_factor_partial(_p(a), m, n, je, _p(lu), _p(piv), ctypes.byref(pos), threads)
    else:
        lib().oracle_lu_factor_partial(_p(a), m, n, je, _p(lu), _p(piv), ctypes.byref(pos))
    return LU(lu, piv, pos.value)


def is_non_singular(f):
    r = lib().oracle_lu_is_non_singular(_p(f.lu), f.m, f.n)
    if r < 0:
        raise ReferencePanic("index out of bounds in is_non_singular (m < n)")
    return bool(r)


def det(f):
    d = ctypes.c_double()
    if lib().oracle_lu_det(_p(f.lu), f.m, f.n, int(f.pospivsign), ctypes.byref(d)) == PANIC:
        raise ReferencePanic("det of a non-square LU")
    return d.value


def solve(f, b):
    """lu.rs:237-278. Returns None where the reference returns None."""
    b = _c(b)
    if b.ndim == 1:
        b = b.reshape(-1, 1)
    x = np.empty((f.m, b.shape[1]), dtype=np.float64)
    r = lib().oracle_lu_solve(_p(f.lu), f.m, f.n, _p(f.piv), _p(b), b.shape[0], b.shape[1], _p(x))
    if r == PANIC:
        raise ReferencePanic("solve: right-hand side rows != LU rows, or is_non_singular out of bounds")
    if r == NONE:
        return None
    return x


def solve_mt(f, b, threads):
    """Same arithmetic as solve(), right-hand-side columns split across threads (no checks)."""
    b = _c(b)
    x = np.empty_like(b)
    lib().oracle_mt_lu_solve_nocheck(_p(f.lu), f.n, _p(f.piv), _p(b), b.shape[1], _p(x), threads)
    return x


def get_l(f):
    c = min(f.m, f.n)
    out = np.empty((f.m, c))
    lib().oracle_lu_get_l(_p(f.lu), f.m, f.n, _p(out))
    return out


def get_u(f):
    r = min(f.m, f.n)
    out = np.empty((r, f.n))
    lib().oracle_lu_get_u(_p(f.lu), f.m, f.n, _p(out))
    return out


def get_p(f):
    out = np.empty((f.m, f.m))
    lib().oracle_lu_get_p(_p(f.piv), f.m, _p(out))
    return out


def matmul(a, b, rows=None, threads=0):
    """mod.rs:957-980. `rows=(r0, r1)` computes only those output rows (a bounded sample)."""
    a = _c(a)
    b = _c(b)
    m, k = a.shape
    kb, n = b.shape
    if k != kb:
        raise ReferencePanic("matmul: a.cols != b.rows")
    c = np.zeros((m, n))
    r0, r1 = (0, m) if rows is None else rows
    if threads and threads > 1:
        lib().oracle_mt_matmul_rows(_p(a), m, k, _p(b), n, _p(c), r0, r1, threads)
    else:
        lib().oracle_matmul_rows(_p(a), m, k, _p(b), kb, n, _p(c), r0, r1)
    return c


def inverse(a):
    """mod.rs:1034-1037."""
    a = _c(a)
    m, n = a.shape
    if m != n:
        raise ReferencePanic("inverse of a non-square matrix")
    out = np.empty_like(a)
    lu = np.empty_like(a)
    piv = np.empty(n, dtype=np.uint64)
    idm = np.empty_like(a)
    r = lib().oracle_inverse(_p(a), m, n, _p(out), _p(lu), _p(piv), _p(idm))
    return None if r == NONE else out


def matrix_det(a):
    """mod.rs:1025-1028."""
    a = _c(a)
    if a.shape[0] != a.shape[1]:
        raise ReferencePanic("det of a non-square matrix")
    return det(lu_factor(a))


def matrix_is_non_singular(a):
    """mod.rs:1044-1047."""
    a = _c(a)
    if a.shape[0] != a.shape[1]:
        raise ReferencePanic("is_non_singular of a non-square matrix")
    return is_non_singular(lu_factor(a))


def backward_error(a, x, b):
    """Normwise backward error max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf)."""
    a = _c(a)
    x = _c(x)
    b = _c(b)
    if x.ndim == 1:
        x = x.reshape(-1, 1)
        b = b.reshape(-1, 1)
    return lib().oracle_backward_error(_p(a), a.shape[0], _p(x), _p(b), x.shape[1])


def max_threads():
    return lib().oracle_mt_max_threads()


def chol_new(a, j_end=None):
    """cholesky.rs:56-111: the n x n factor L (zeros above the diagonal), or
    None for a non-square, non-symmetric or not positive definite matrix.
    `j_end` stops after that many rows (a bounded sample; rows past it are
    left unset)."""
    a = _c(a)
    if a.ndim != 2:
        raise ValueError("a must be 2-D")
    m, n = a.shape
    lo = np.zeros((n, n), dtype=np.float64)
    je = n if j_end is None else min(int(j_end), n)
    r = lib().oracle_chol_new_partial(_p(a), m, n, je, _p(lo))
    return None if r == NONE else lo


def chol_solve(l, b):
    """cholesky.rs:116-145; ReferencePanic when b's row count differs from L's."""
    l = _c(l)
    b = _c(b)
    if b.ndim == 1:
        b = b.reshape(-1, 1)
    n = l.shape[0]
    x = np.empty((n, b.shape[1]), dtype=np.float64)
    if lib().oracle_chol_solve(_p(l), n, _p(b), b.shape[0], b.shape[1], _p(x)) == PANIC:
        raise ReferencePanic("assertion failed: l.rows() == b.rows()")
    return x


class QR:
    """QRDecomposition as the reference holds it (qr.rs:20-23): qr and rdiag."""

    def __init__(self, qr, rdiag):
        self.qr = qr
        self.rdiag = rdiag

    @property
    def m(self):
        return self.qr.shape[0]

    @property
    def n(self):
        return self.qr.shape[1]


def qr_new(a):
    """qr.rs:26-105."""
    a = _c(a)
    m, n = a.shape
    qr = np.empty_like(a)
    rd = np.empty(min(m, n))
    lib().oracle_qr_new(_p(a), m, n, _p(qr), _p(rd))
    return QR(qr, rd)


def qr_is_full_rank(f):
    """qr.rs:108-115; ReferencePanic where it indexes past rdiag (n > m)."""
    r = lib().oracle_qr_is_full_rank(_p(f.rdiag), f.m, f.n)
    if r < 0:
        raise ReferencePanic("index out of bounds in is_full_rank (n > m)")
    return bool(r)


def qr_get_h(f):
    out = np.empty((f.m, f.n))
    lib().oracle_qr_get_h(_p(f.qr), f.m, f.n, _p(out))
    return out


def qr_get_r(f):
    out = np.empty((f.m, f.n))
    lib().oracle_qr_get_r(_p(f.qr), _p(f.rdiag), f.m, f.n, _p(out))
    return out


def qr_get_q(f):
    out = np.empty((f.m, f.m))
    lib().oracle_qr_get_q(_p(f.qr), _p(f.rdiag), f.m, f.n, _p(out))
    return out


def qr_solve(f, b):
    """qr.rs:199-238: the solution, None (not full rank) or ReferencePanic."""
    b = _c(b)
    if b.ndim == 1:
        b = b.reshape(-1, 1)
    x = np.empty((f.n, b.shape[1]))
    r = lib().oracle_qr_solve(_p(f.qr), _p(f.rdiag), f.m, f.n, _p(b), b.shape[0], b.shape[1], _p(x))
    if r == PANIC:
        raise ReferencePanic("QRDecomposition::solve panics (shape)")
    if r == NONE:
        return None
    return x


def pinverse(a):
    """Matrix::pinverse (mod.rs:1049-1057): (R' R)^-1 A' with the crate's Mul
    (mod.rs:957-980) and inverse (LU, mod.rs:1034-1037); ReferencePanic where
    the inverse is None (unwrap)."""
    a = _c(a)
    r = qr_get_r(qr_new(a))
    rtr = matmul(np.ascontiguousarray(r.T), r)
    f = lu_factor(rtr)
    inv = solve(f, np.eye(rtr.shape[0]))
    if inv is None:
        raise ReferencePanic("called `Option::unwrap()` on a `None` value")
    return matmul(inv, np.ascontiguousarray(a.T))


UNSUPPORTED, NOT_FINITE = 3, 4


def eig_sym(a):
    """eigen.rs:755-790 symmetric branch (tred2 + tql2): (d, e, v), eigenvalues
    descending, eigenvectors as the columns of v."""
    a = _c(a)
    n = a.shape[0]
    d = np.empty(n)
    e = np.empty(n)
    v = np.empty((n, n))
    r = lib().oracle_eig_sym(_p(a), n, _p(d), _p(e), _p(v))
    if r != OK:
        raise ValueError("oracle_eig_sym status %d" % r)
    return d, e, v


def svd_direct(a):
    """svd.rs:454-497: (u m x m, s m x n, v n x n). ReferencePanic where the
    reference's s.inverse().unwrap() panics (a zero singular value)."""
    a = _c(a)
    m, n = a.shape
    u = np.empty((m, m))
    s = np.empty((m, n))
    v = np.empty((n, n))
    r = lib().oracle_svd_direct(_p(a), m, n, _p(u), _p(s), _p(v))
    if r == PANIC:
        raise ReferencePanic("SVD::direct: a zero singular value (inverse().unwrap() on None)")
    if r != OK:
        raise ValueError("oracle_svd_direct status %d" % r)
    return u, s, v
