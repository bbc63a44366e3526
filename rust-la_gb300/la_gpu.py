"""Python host mirror of the `la` crate's LU path over liblagpu.so (include/la_gpu.h).

The names, argument meaning and failure behaviour follow the reference crate
(xasmx/rust-la 0.2.0):

  Matrix.new(rows, cols, data)        src/matrix/mod.rs:207-211 (asserts len and dims > 0)
  Matrix.id(m, n)                     mod.rs:416-426
  a * b, a.mmul(b, dst)               mod.rs:957-998, mmatrix.rs:82-98
  a.det(), a.solve(b), a.inverse()    mod.rs:1025-1037
  a.is_singular(), a.is_non_singular() mod.rs:1039-1047
  LUDecomposition.new(a)              src/decomp/lu.rs:104-168
  SVD.direct(a)                       src/decomp/svd.rs:454-497
  lu.solve(b) / det / is_singular / is_non_singular / get_l / get_u / get_p / get_piv
                                      lu.rs:170-278

A reference `assert!` panic raises `Panic`; a reference `None` is returned as
`None`. All arithmetic runs in the CUDA library; there is no CPU path here, and
importing this module fails loudly when liblagpu.so is missing.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblagpu.so")

OK, SINGULAR, BADSHAPE, INVALID, NOMEM, CUDA_ERROR, TIMEOUT, NOT_CONVERGED, UNSUPPORTED = range(9)
OPT_ARITH, OPT_PANEL_WIDTH, OPT_PANEL_CTAS, OPT_PROFILE, OPT_LOOKAHEAD, OPT_CLUSTER_PANEL = 1, 2, 3, 4, 5, 6
OPT_BATCH_GMRES = 7
OPT_SOLVE_WAVE = 8
OPT_INJECT_ALLOC_FAIL, OPT_INJECT_IR_STALL = 10, 11
OPT_WAIT_LIMIT_US, OPT_INJECT_PANEL_STALL = 12, 13
OPT_PDL = 14
ARITH_FAST, ARITH_EXACT = 0, 1


class Panic(Exception):
    """The reference would panic here (failed assert! or out-of-bounds index)."""


class LaError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("liblagpu status %d%s" % (status, (": " + msg) if msg else ""))


_lib = None

# Every symbol declared in include/la_gpu.h, with its ctypes signature.
_P, _S, _I, _D = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_double
SIGNATURES = {
    "la_abi_version": ([], _I),
    "la_status_string": ([_I], ctypes.c_char_p),
    "la_ctx_create": ([_I, _P], _I),
    "la_ctx_destroy": ([_P], None),
    "la_ctx_set_stream": ([_P, _P], _I),
    "la_ctx_get_stream": ([_P], _P),
    "la_ctx_synchronize": ([_P], _I),
    "la_ctx_last_error": ([_P], ctypes.c_char_p),
    "la_ctx_set_option": ([_P, _I, ctypes.c_int64], _I),
    "la_ctx_get_option": ([_P, _I, _P], _I),
    "la_ctx_kernel_launches": ([_P], ctypes.c_uint64),
    "la_ctx_last_phase_ms": ([_P, _P], _I),
    "la_probe_fp64_peak": ([_P, _P], _I),
    "la_lu_new": ([_P, _P, _S, _S, _P], _I),
    "la_lu_new_device": ([_P, _P, _S, _S, _S, _P], _I),
    "la_lu_free": ([_P], None),
    "la_lu_shape": ([_P, _P, _P], _I),
    "la_lu_is_non_singular": ([_P, _P], _I),
    "la_lu_det": ([_P, _P], _I),
    "la_lu_get_piv": ([_P, _P, _P], _I),
    "la_lu_get_packed": ([_P, _P], _I),
    "la_lu_get_l": ([_P, _P], _I),
    "la_lu_get_u": ([_P, _P], _I),
    "la_lu_get_p": ([_P, _P], _I),
    "la_lu_device_data": ([_P, _P], _P),
    "la_lu_solve": ([_P, _P, _S, _S, _P], _I),
    "la_lu_solve_device": ([_P, _P, _S, _S, _S, _P, _S], _I),
    "la_matrix_det": ([_P, _P, _S, _S, _P], _I),
    "la_matrix_solve": ([_P, _P, _S, _S, _P, _S, _S, _P], _I),
    "la_matrix_inverse": ([_P, _P, _S, _S, _P], _I),
    "la_matrix_is_non_singular": ([_P, _P, _S, _S, _P], _I),
    "la_matrix_mul": ([_P, _P, _S, _S, _P, _S, _S, _P], _I),
    "la_matrix_mmul": ([_P, _P, _S, _S, _P, _S, _S, _P, _S, _S], _I),
    "la_matrix_mul_device": ([_P, _P, _S, _P, _S, _P, _S, _S, _S, _S], _I),
    "la_backward_error_device": ([_P, _P, _S, _P, _S, _P, _S, _S, _S, _P], _I),
    "la_backward_error": ([_P, _P, _P, _P, _S, _S, _P], _I),
    "la_lu_factor_noalloc": ([_P, _P, _S, _S, _S, _P, _P, _P], _I),
    "la_qr_new": ([_P, _P, _S, _S, _P], _I),
    "la_qr_new_device": ([_P, _P, _S, _S, _S, _P], _I),
    "la_qr_free": ([_P], None),
    "la_qr_is_full_rank": ([_P, _P], _I),
    "la_qr_get_h": ([_P, _P], _I),
    "la_qr_get_r": ([_P, _P], _I),
    "la_qr_get_q": ([_P, _P], _I),
    "la_qr_solve": ([_P, _P, _S, _S, _P], _I),
    "la_matrix_pinverse": ([_P, _P, _S, _S, _P], _I),
    "la_svd_direct": ([_P, _P, _S, _S, _P, _P, _P], _I),
    "la_read_csv_f64": ([ctypes.c_char_p, _P, _P, _P], _I),
    "la_host_free": ([_P], None),
    "la_chol_new": ([_P, _P, _S, _S, _P], _I),
    "la_chol_new_device": ([_P, _P, _S, _S, _P], _I),
    "la_chol_free": ([_P], None),
    "la_chol_n": ([_P, _P], _I),
    "la_chol_get_l": ([_P, _P], _I),
    "la_chol_solve": ([_P, _P, _S, _S, _P], _I),
    "la_chol_solve_device": ([_P, _P, _S, _S, _S, _P, _S], _I),
    "la_lu_mixed_new_device": ([_P, _P, _S, _S, _I, _P], _I),
    "la_lu_solve_refined_device": ([_P, _P, _S, _S, _P, _S, _I, _D, _P], _I),
    "la_lu_solve_auto_device": ([_P, _P, _S, _S, _P, _S, _S, _P, _S, _D, _P], _I),
    "la_lowp_update_device": ([_P, _I, _S, _S, _S, _P, _S, _P, _S, _P, _S, ctypes.c_float], _I),
    "la_batch_plan_create": ([_P, _P, _P, _P, _P, _I, _I, _I, _I, _D, _I, _P], _I),
    "la_batch_plan_run": ([_P], _I),
    "la_batch_plan_stats": ([_P, _P, _P, _P], _I),
    "la_batch_plan_destroy": ([_P], None),
    "la_batch_autotune": ([_P, _P, _P, _P, _P, _I, _I, _D, _I, ctypes.c_char_p, _P, _P, _P], _I),
    "la_batch_plan_cycles": ([_P, _P], _I),
    "la_batch_plan_select_device": ([_P, _P], _I),
    "la_batch_plan_pivots": ([_P, _P], _I),
    "la_batch_partition": ([_P, _I, _I, _P], _I),
    "la_batch_backward_error_device": ([_P, _P, _P, _P, _P, _I, _P, _P], _I),
    "la_batch_plan_phase_cycles": ([_P, _P], _I),
    "la_batch_features_device": ([_P, _P, _P, _I, _P], _I),
    "la_generate_conditioned_batch": ([_P, _P, _I, _D, _D, ctypes.c_ulonglong, _P, _P, _P], _I),
    "la_mlp_param_count": ([], _I),
    "la_mlp_create": ([_P, ctypes.c_ulonglong, _P], _I),
    "la_mlp_destroy": ([_P], None),
    "la_mlp_get_params": ([_P, _P], _I),
    "la_mlp_set_params": ([_P, _P], _I),
    "la_mlp_gradients": ([_P, _P, _P, _I, _P, _P], _I),
    "la_mlp_train_step": ([_P, _P, _P, _I, ctypes.c_float, _P], _I),
    "la_mlp_gradients_cost": ([_P, _P, _P, _I, _P, _P], _I),
    "la_mlp_train_step_cost": ([_P, _P, _P, _I, ctypes.c_float, _P], _I),
    "la_mlp_predict": ([_P, _P, _I, _P, _P], _I),
    "la_mlp_set_gate": ([_P, _P, ctypes.c_float], _I),
}

BATCH_FP64, BATCH_MIXED = 0, 1


class BatchSystem(ctypes.Structure):
    _fields_ = [("a_offset", ctypes.c_size_t), ("b_offset", ctypes.c_size_t),
                ("n", ctypes.c_int), ("nrhs", ctypes.c_int), ("precision", ctypes.c_int),
                ("reserved", ctypes.c_int)]

PREC_BF16, PREC_FP16, PREC_FP32, PREC_FP8, PREC_FP64, PREC_FP16X3 = 1, 2, 3, 4, 5, 6


class RefineStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("eta", ctypes.c_double), ("fell_back", ctypes.c_int),
                ("precision", ctypes.c_int), ("gmres_steps", ctypes.c_int)]


def lib():
    """Loads liblagpu.so (built by rust-la_gb300/build.py). Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("liblagpu.so not built: run python rust-la_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """One la_ctx: a device, a stream and the library's device scratch."""

    def __init__(self, device=0, arith=ARITH_FAST):
        self.h = ctypes.c_void_p()
        st = lib().la_ctx_create(device, ctypes.byref(self.h))
        if st != OK:
            raise LaError(st, "la_ctx_create")
        self.set_option(OPT_ARITH, arith)

    def close(self):
        if self.h:
            lib().la_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, opt, value):
        st = lib().la_ctx_set_option(self.h, opt, int(value))
        if st != OK:
            raise LaError(st, "set_option")

    def get_option(self, opt):
        v = ctypes.c_int64()
        st = lib().la_ctx_get_option(self.h, opt, ctypes.byref(v))
        if st != OK:
            raise LaError(st, "get_option")
        return v.value

    def set_stream(self, stream_handle):
        st = lib().la_ctx_set_stream(self.h, ctypes.c_void_p(stream_handle))
        if st != OK:
            raise LaError(st, "set_stream")

    def synchronize(self):
        _check(self, lib().la_ctx_synchronize(self.h))

    def last_error(self):
        return lib().la_ctx_last_error(self.h).decode()

    def kernel_launches(self):
        return lib().la_ctx_kernel_launches(self.h)

    def phase_ms(self):
        out = (ctypes.c_double * 5)()
        lib().la_ctx_last_phase_ms(self.h, out)
        return list(out)

    def fp64_peak_tflops(self):
        v = ctypes.c_double()
        _check(self, lib().la_probe_fp64_peak(self.h, ctypes.byref(v)))
        return v.value


_default = None


def default_context():
    global _default
    if _default is None:
        _default = Context()
    return _default


def _check(ctx, st, allow=(OK,)):
    if st in allow:
        return st
    if st == BADSHAPE:
        raise Panic("reference would panic (shape assertion)")
    msg = ctx.last_error() if ctx is not None else ""
    raise LaError(st, msg)


class Matrix:
    """Row-major f64 matrix, the mirror of Matrix<f64> (mod.rs:26-30)."""

    __slots__ = ("data", "ctx")

    def __init__(self, array, ctx=None):
        a = np.ascontiguousarray(array, dtype=np.float64)
        if a.ndim != 2 or a.shape[0] == 0 or a.shape[1] == 0:
            raise Panic("Matrix::new requires rows > 0 and cols > 0")
        self.data = a
        self.ctx = ctx

    @staticmethod
    def new(rows, cols, data, ctx=None):
        data = list(data) if not isinstance(data, np.ndarray) else data.ravel()
        if rows * cols != len(data) or rows == 0 or cols == 0:
            raise Panic("Matrix::new: len(data) != rows * cols or empty")
        return Matrix(np.asarray(data, dtype=np.float64).reshape(rows, cols), ctx)

    @staticmethod
    def id(m, n, ctx=None):
        return Matrix(np.eye(m, n), ctx)

    def _c(self):
        return self.ctx if self.ctx is not None else default_context()

    def rows(self):
        return self.data.shape[0]

    def cols(self):
        return self.data.shape[1]

    def get_data(self):
        return self.data.ravel()

    def pinverse(self):
        """mod.rs:1049-1057: (R' R)^-1 A' (Panic where inverse() is None)."""
        ctx = self._c()
        out = np.empty((self.cols(), self.rows()))
        _check(ctx, lib().la_matrix_pinverse(ctx.h, _ptr(self.data), self.rows(), self.cols(),
                                             _ptr(out)))
        return Matrix(out, self.ctx)

    def t(self):
        """mod.rs:653-662: the transpose (a host copy)."""
        return Matrix(np.ascontiguousarray(self.data.T), self.ctx)

    def get(self, r, c):
        if r >= self.rows() or c >= self.cols():
            raise Panic("Matrix::get out of range")
        return float(self.data[r, c])

    def __eq__(self, other):
        return (isinstance(other, Matrix) and self.data.shape == other.data.shape
                and bool(np.all(self.data == other.data)))

    def approx_eq(self, other):
        """mod.rs:1141-1147 with approxeq.rs:34-47 (|a-b| < 1e-6 for every entry)."""
        if self.data.shape != other.data.shape:
            return False
        return bool(np.all(np.abs(self.data - other.data) < 1e-6))

    def __mul__(self, other):
        ctx = self._c()
        if self.cols() != other.rows():
            raise Panic("Mul: self.cols() != m.rows() (mod.rs:961)")
        out = np.empty((self.rows(), other.cols()))
        _check(ctx, lib().la_matrix_mul(ctx.h, _ptr(self.data), self.rows(), self.cols(),
                                        _ptr(other.data), other.rows(), other.cols(), _ptr(out)))
        return Matrix(out, self.ctx)

    def mmul(self, m, dst):
        """mmatrix.rs:82-98: writes self * m into dst (asserts dims)."""
        ctx = self._c()
        st = lib().la_matrix_mmul(ctx.h, _ptr(self.data), self.rows(), self.cols(), _ptr(m.data),
                                  m.rows(), m.cols(), _ptr(dst.data), dst.rows(), dst.cols())
        _check(ctx, st)
        return dst

    def det(self):
        ctx = self._c()
        out = ctypes.c_double()
        _check(ctx, lib().la_matrix_det(ctx.h, _ptr(self.data), self.rows(), self.cols(),
                                        ctypes.byref(out)))
        return out.value

    def solve(self, b):
        ctx = self._c()
        x = np.empty((self.rows(), b.cols()))
        st = lib().la_matrix_solve(ctx.h, _ptr(self.data), self.rows(), self.cols(), _ptr(b.data),
                                   b.rows(), b.cols(), _ptr(x))
        if _check(ctx, st, (OK, SINGULAR)) == SINGULAR:
            return None
        return Matrix(x, self.ctx)

    def inverse(self):
        ctx = self._c()
        out = np.empty_like(self.data)
        st = lib().la_matrix_inverse(ctx.h, _ptr(self.data), self.rows(), self.cols(), _ptr(out))
        if _check(ctx, st, (OK, SINGULAR)) == SINGULAR:
            return None
        return Matrix(out, self.ctx)

    def is_non_singular(self):
        ctx = self._c()
        out = ctypes.c_int()
        _check(ctx, lib().la_matrix_is_non_singular(ctx.h, _ptr(self.data), self.rows(),
                                                    self.cols(), ctypes.byref(out)))
        return bool(out.value)

    def is_singular(self):
        return not self.is_non_singular()

    def __repr__(self):
        return "Matrix(%r)" % (self.data,)


def m(rows):
    """The m! macro (src/macros.rs:40-42): m([[1, 2], [3, 4]])."""
    return Matrix(np.array(rows, dtype=np.float64))


class LUDecomposition:
    """Device-resident LU factors, the mirror of LUDecomposition<f64> (lu.rs:95-101)."""

    def __init__(self, handle, ctx, m_, n_):
        self.h = handle
        self.ctx = ctx
        self.m = m_
        self.n = n_

    @staticmethod
    def new(a, ctx=None):
        """lu.rs:104-168. `a` is a Matrix or a 2-D array."""
        if not isinstance(a, Matrix):
            a = Matrix(a, ctx)
        ctx = ctx or a._c()
        h = ctypes.c_void_p()
        _check(ctx, lib().la_lu_new(ctx.h, _ptr(a.data), a.rows(), a.cols(), ctypes.byref(h)))
        return LUDecomposition(h, ctx, a.rows(), a.cols())

    @staticmethod
    def new_device(ptr, lda, m_, n_, ctx):
        h = ctypes.c_void_p()
        _check(ctx, lib().la_lu_new_device(ctx.h, ctypes.c_void_p(ptr), lda, m_, n_,
                                           ctypes.byref(h)))
        return LUDecomposition(h, ctx, m_, n_)

    def free(self):
        if self.h:
            lib().la_lu_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def is_non_singular(self):
        out = ctypes.c_int()
        _check(self.ctx, lib().la_lu_is_non_singular(self.h, ctypes.byref(out)))
        return bool(out.value)

    def is_singular(self):
        return not self.is_non_singular()

    def det(self):
        out = ctypes.c_double()
        _check(self.ctx, lib().la_lu_det(self.h, ctypes.byref(out)))
        return out.value

    def get_piv(self):
        piv = np.empty(self.m, dtype=np.uint64)
        _check(self.ctx, lib().la_lu_get_piv(self.h, _ptr(piv), None))
        return piv

    def pospivsign(self):
        s = ctypes.c_int()
        _check(self.ctx, lib().la_lu_get_piv(self.h, None, ctypes.byref(s)))
        return bool(s.value)

    def _get(self, fn, shape):
        out = np.empty(shape)
        _check(self.ctx, fn(self.h, _ptr(out)))
        return Matrix(out, self.ctx)

    def get_packed(self):
        return self._get(lib().la_lu_get_packed, (self.m, self.n))

    def get_l(self):
        return self._get(lib().la_lu_get_l, (self.m, min(self.m, self.n)))

    def get_u(self):
        return self._get(lib().la_lu_get_u, (min(self.m, self.n), self.n))

    def get_p(self):
        return self._get(lib().la_lu_get_p, (self.m, self.m))

    def solve(self, b):
        """lu.rs:237-278: None if singular, Panic if b.rows() != m."""
        if not isinstance(b, Matrix):
            b = Matrix(np.asarray(b, dtype=np.float64).reshape(self.m, -1)
                       if np.ndim(b) == 1 else b, self.ctx)
        x = np.empty((self.m, b.cols()))
        st = lib().la_lu_solve(self.h, _ptr(b.data), b.rows(), b.cols(), _ptr(x))
        if _check(self.ctx, st, (OK, SINGULAR)) == SINGULAR:
            return None
        return Matrix(x, self.ctx)

    def solve_device(self, b_ptr, ldb, brows, nrhs, x_ptr, ldx):
        st = lib().la_lu_solve_device(self.h, ctypes.c_void_p(b_ptr), ldb, brows, nrhs,
                                      ctypes.c_void_p(x_ptr), ldx)
        return _check(self.ctx, st, (OK, SINGULAR))


class QRDecomposition:
    """Mirror of QRDecomposition<f64> (src/decomp/qr.rs:20-238)."""

    def __init__(self, h, ctx, m, n):
        self.h = h
        self.ctx = ctx
        self.m = m
        self.n = n

    @staticmethod
    def new(a, ctx=None):
        """qr.rs:26-105."""
        if not isinstance(a, Matrix):
            a = Matrix(a, ctx)
        ctx = ctx or a._c()
        h = ctypes.c_void_p()
        _check(ctx, lib().la_qr_new(ctx.h, _ptr(a.data), a.rows(), a.cols(), ctypes.byref(h)))
        return QRDecomposition(h, ctx, a.rows(), a.cols())

    @staticmethod
    def new_device(ptr, lda, m_, n_, ctx):
        h = ctypes.c_void_p()
        _check(ctx, lib().la_qr_new_device(ctx.h, ctypes.c_void_p(ptr), lda, m_, n_,
                                           ctypes.byref(h)))
        return QRDecomposition(h, ctx, m_, n_)

    def free(self):
        if self.h:
            lib().la_qr_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def is_full_rank(self):
        """qr.rs:108-115 (Panic where it indexes past rdiag)."""
        out = ctypes.c_int()
        _check(self.ctx, lib().la_qr_is_full_rank(self.h, ctypes.byref(out)))
        return bool(out.value)

    def _get(self, fn, shape):
        out = np.empty(shape)
        _check(self.ctx, fn(self.h, _ptr(out)))
        return Matrix(out, self.ctx)

    def get_h(self):
        return self._get(lib().la_qr_get_h, (self.m, self.n))

    def get_r(self):
        return self._get(lib().la_qr_get_r, (self.m, self.n))

    def get_q(self):
        return self._get(lib().la_qr_get_q, (self.m, self.m))

    def solve(self, b):
        """qr.rs:199-238: None if not full rank, Panic where the reference panics."""
        if not isinstance(b, Matrix):
            b = Matrix(np.asarray(b, dtype=np.float64).reshape(-1, 1)
                       if np.ndim(b) == 1 else b, self.ctx)
        x = np.empty((self.n, b.cols()))
        st = lib().la_qr_solve(self.h, _ptr(b.data), b.rows(), b.cols(), _ptr(x))
        if _check(self.ctx, st, (OK, SINGULAR)) == SINGULAR:
            return None
        return Matrix(x, self.ctx)


class CholeskyDecomposition:
    """Mirror of CholeskyDecomposition<f64> (src/decomp/cholesky.rs:52-145)."""

    def __init__(self, h, ctx, n):
        self.h = h
        self.ctx = ctx
        self.n = n

    @staticmethod
    def new(a, ctx=None):
        """cholesky.rs:56-111: None for a non-square, non-symmetric or not
        positive definite matrix."""
        if not isinstance(a, Matrix):
            a = Matrix(a, ctx)
        ctx = ctx or a._c()
        h = ctypes.c_void_p()
        st = lib().la_chol_new(ctx.h, _ptr(a.data), a.rows(), a.cols(), ctypes.byref(h))
        if _check(ctx, st, (OK, SINGULAR)) == SINGULAR:
            return None
        return CholeskyDecomposition(h, ctx, a.rows())

    @staticmethod
    def new_device(ptr, lda, n, ctx):
        h = ctypes.c_void_p()
        st = lib().la_chol_new_device(ctx.h, ctypes.c_void_p(ptr), lda, n, ctypes.byref(h))
        if _check(ctx, st, (OK, SINGULAR)) == SINGULAR:
            return None
        return CholeskyDecomposition(h, ctx, n)

    def free(self):
        if self.h:
            lib().la_chol_free(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def get_l(self):
        """cholesky.rs:113."""
        out = np.empty((self.n, self.n))
        _check(self.ctx, lib().la_chol_get_l(self.h, _ptr(out)))
        return Matrix(out, self.ctx)

    def solve(self, b):
        """cholesky.rs:116-145: Panic when b's row count differs from L's."""
        if not isinstance(b, Matrix):
            b = Matrix(np.asarray(b, dtype=np.float64).reshape(-1, 1)
                       if np.ndim(b) == 1 else b, self.ctx)
        x = np.empty((b.rows(), b.cols()))
        _check(self.ctx, lib().la_chol_solve(self.h, _ptr(b.data), b.rows(), b.cols(), _ptr(x)))
        return Matrix(x, self.ctx)

    def solve_device(self, b_ptr, ldb, brows, nrhs, x_ptr, ldx):
        _check(self.ctx, lib().la_chol_solve_device(self.h, ctypes.c_void_p(b_ptr), ldb, brows,
                                                     nrhs, ctypes.c_void_p(x_ptr), ldx))


class SVD:
    """Mirror of SVD<f64>'s direct method (src/decomp/svd.rs:454-497, get_u / get_s /
    get_v at :427-437): U (m x m), S (m x n), V (n x n) with A = U S V'."""

    def __init__(self, u, s, v):
        self.u, self.s, self.v = u, s, v

    @staticmethod
    def direct(a, ctx=None):
        """svd.rs:454-497. Panic where the reference panics (a zero singular value)."""
        if not isinstance(a, Matrix):
            a = Matrix(a, ctx)
        ctx = ctx or a._c()
        m, n = a.rows(), a.cols()
        u = np.empty((m, m))
        s = np.empty((m, n))
        v = np.empty((n, n))
        _check(ctx, lib().la_svd_direct(ctx.h, _ptr(a.data), m, n, _ptr(u), _ptr(s), _ptr(v)))
        return SVD(Matrix(u, ctx), Matrix(s, ctx), Matrix(v, ctx))

    def get_u(self):
        return self.u

    def get_s(self):
        return self.s

    def get_v(self):
        return self.v


def read_csv(path):
    """util::read_csv (src/util.rs:9-35) with the f64 parser: a Matrix, or Panic
    where the reference panics (no file, not UTF-8, an item that is not an f64
    literal, ragged lines, an empty file)."""
    data = ctypes.c_void_p()
    rows = ctypes.c_size_t()
    cols = ctypes.c_size_t()
    st = lib().la_read_csv_f64(os.fsencode(path), ctypes.byref(data), ctypes.byref(rows),
                               ctypes.byref(cols))
    _check(None, st)
    try:
        n = rows.value * cols.value
        buf = (ctypes.c_double * n).from_address(data.value)
        out = np.frombuffer(buf, dtype=np.float64, count=n).reshape(rows.value, cols.value).copy()
    finally:
        lib().la_host_free(data)
    return Matrix(out)


def backward_error(ctx, a, x, b):
    """eta = max_j ||b_j - A x_j||_inf / (||A||_inf ||x_j||_inf + ||b_j||_inf), on the GPU."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(a.shape[0], -1)
    b = np.ascontiguousarray(b, dtype=np.float64).reshape(a.shape[0], -1)
    out = ctypes.c_double()
    _check(ctx, lib().la_backward_error(ctx.h, _ptr(a), _ptr(x), _ptr(b), a.shape[0], x.shape[1],
                                        ctypes.byref(out)))
    return out.value


def backward_error_device(ctx, a_ptr, lda, x_ptr, ldx, b_ptr, ldb, n, nrhs):
    out = ctypes.c_double()
    _check(ctx, lib().la_backward_error_device(ctx.h, ctypes.c_void_p(a_ptr), lda,
                                               ctypes.c_void_p(x_ptr), ldx, ctypes.c_void_p(b_ptr),
                                               ldb, n, nrhs, ctypes.byref(out)))
    return out.value


def batch_backward_error_device(ctx, a_ptr, b_ptr, x_ptr, systems, eta_ptr):
    """Every system's backward error into the device buffer eta_ptr (count
    doubles, caller's order); returns the largest."""
    worst = ctypes.c_double()
    _check(ctx, lib().la_batch_backward_error_device(ctx.h, ctypes.c_void_p(a_ptr),
                                                     ctypes.c_void_p(b_ptr),
                                                     ctypes.c_void_p(x_ptr), systems,
                                                     len(systems), ctypes.c_void_p(eta_ptr),
                                                     ctypes.byref(worst)))
    return worst.value


def lu_mixed_new_device(ctx, a_ptr, lda, n, prec):
    h = ctypes.c_void_p()
    _check(ctx, lib().la_lu_mixed_new_device(ctx.h, ctypes.c_void_p(a_ptr), lda, n, prec,
                                             ctypes.byref(h)))
    return LUDecomposition(h, ctx, n, n)


def lu_solve_refined_device(lu, b_ptr, ldb, nrhs, x_ptr, ldx, max_iters=50, tol=1e-14):
    stats = RefineStats()
    st = lib().la_lu_solve_refined_device(lu.h, ctypes.c_void_p(b_ptr), ldb, nrhs,
                                          ctypes.c_void_p(x_ptr), ldx, max_iters, tol,
                                          ctypes.byref(stats))
    _check(lu.ctx, st, (OK, NOT_CONVERGED, SINGULAR))
    return st, stats


def lu_solve_auto_device(ctx, a_ptr, lda, n, b_ptr, ldb, nrhs, x_ptr, ldx, tol=1e-14):
    """Automatic precision (la_lu_solve_auto_device): split-FP16 factors with
    refinement and then GMRES-IR, then the plain FP64 LU for whatever they
    could not answer. Returns (status, RefineStats)."""
    stats = RefineStats()
    st = lib().la_lu_solve_auto_device(ctx.h, ctypes.c_void_p(a_ptr), lda, n,
                                       ctypes.c_void_p(b_ptr), ldb, nrhs, ctypes.c_void_p(x_ptr),
                                       ldx, ctypes.c_double(tol), ctypes.byref(stats))
    _check(ctx, st, (OK, SINGULAR))
    return st, stats


def lowp_update_device(ctx, fmt, m_, n, k, a_ptr, lda, b_ptr, ldb, c_ptr, ldc, alpha):
    st = lib().la_lowp_update_device(ctx.h, fmt, m_, n, k, ctypes.c_void_p(a_ptr), lda,
                                     ctypes.c_void_p(b_ptr), ldb, ctypes.c_void_p(c_ptr), ldc,
                                     ctypes.c_float(alpha))
    return _check(ctx, st)


def batch_systems(ns, nrhss, precisions=None):
    """Packs per-system sizes (and factor precisions) into la_batch_system
    records with dense offsets."""
    arr = (BatchSystem * len(ns))()
    ao = bo = 0
    for i, (n, r) in enumerate(zip(ns, nrhss)):
        arr[i].a_offset, arr[i].b_offset, arr[i].n, arr[i].nrhs = ao, bo, int(n), int(r)
        arr[i].precision = int(precisions[i]) if precisions is not None else 0
        ao += int(n) * int(n)
        bo += int(n) * int(r)
    return arr, ao, bo


def batch_partition(systems, parts):
    """Cost-balanced contiguous slices of a batch for `parts` GPUs
    (la_batch_partition): bounds[0] = 0 <= ... <= bounds[parts] = count."""
    bounds = np.empty(parts + 1, dtype=np.int32)
    st = lib().la_batch_partition(systems, len(systems), parts, _ptr(bounds))
    _check(None, st)
    return [int(b) for b in bounds]


def batch_slice(systems, lo, hi):
    """Systems [lo, hi) of a densely packed batch (batch_systems) as their own
    batch: (systems with offsets rebased to the slice, a_base, a_len, b_base,
    b_len), so that a GPU holding only A[a_base : a_base + a_len] and
    B, X[b_base : b_base + b_len] can build its plan over them."""
    count = hi - lo
    arr = (BatchSystem * max(count, 0))()
    if count <= 0:
        return arr, 0, 0, 0, 0
    a_base, b_base = systems[lo].a_offset, systems[lo].b_offset
    last = systems[hi - 1]
    for i in range(count):
        s = systems[lo + i]
        arr[i].a_offset = s.a_offset - a_base
        arr[i].b_offset = s.b_offset - b_base
        arr[i].n, arr[i].nrhs, arr[i].precision = s.n, s.nrhs, s.precision
    a_len = last.a_offset + last.n * last.n - a_base
    b_len = last.b_offset + last.n * last.nrhs - b_base
    return arr, a_base, a_len, b_base, b_len


def set_precisions(systems, precisions):
    for i, p in enumerate(precisions):
        systems[i].precision = int(p)


class BatchPlan:
    """A captured batched factor + solve (la_batch_plan)."""

    def __init__(self, ctx, a_ptr, b_ptr, x_ptr, systems, mode, ctas_per_sm=1, warps_per_system=8,
                 tol=1e-14, max_iters=10):
        self.ctx = ctx
        self.count = len(systems)
        self.h = ctypes.c_void_p()
        _check(ctx, lib().la_batch_plan_create(ctx.h, ctypes.c_void_p(a_ptr), ctypes.c_void_p(b_ptr),
                                               ctypes.c_void_p(x_ptr), systems, self.count, mode,
                                               ctas_per_sm, warps_per_system, tol, max_iters,
                                               ctypes.byref(self.h)))

    def run(self):
        _check(self.ctx, lib().la_batch_plan_run(self.h))

    def stats(self):
        its = np.empty(self.count, dtype=np.int32)
        eta = np.empty(self.count, dtype=np.float64)
        fb = np.empty(self.count, dtype=np.int32)
        _check(self.ctx, lib().la_batch_plan_stats(self.h, _ptr(its), _ptr(eta), _ptr(fb)))
        return its, eta, fb

    def select_device(self, class_ptr):
        """Per-system factor storage from selector classes (device int32: 0 FP8,
        1 BF16, 2 FP32, 3 straight to the FP64 pass)."""
        _check(self.ctx, lib().la_batch_plan_select_device(self.h, ctypes.c_void_p(class_ptr)))

    def pivots(self, ns):
        """Row order (lu.rs piv) of each system's factors in the last run, as a
        list of arrays in the caller's order; ns are the systems' sizes."""
        total = int(np.sum(ns))
        p = np.empty(total, dtype=np.uint64)
        _check(self.ctx, lib().la_batch_plan_pivots(self.h, _ptr(p)))
        out, o = [], 0
        for n in ns:
            out.append(p[o:o + int(n)])
            o += int(n)
        return out

    def phase_cycles(self):
        """[load, factor, solves, residuals] cycles of the first pass, then of the FP64 redo."""
        c = np.empty(8, dtype=np.int64)
        _check(self.ctx, lib().la_batch_plan_phase_cycles(self.h, _ptr(c)))
        return c

    def cycles(self):
        c = np.empty(self.count, dtype=np.int64)
        _check(self.ctx, lib().la_batch_plan_cycles(self.h, _ptr(c)))
        return c

    def free(self):
        if self.h:
            lib().la_batch_plan_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def batch_autotune(ctx, a_ptr, b_ptr, x_ptr, systems, mode, tol=1e-14, max_iters=10,
                   table_path=None):
    """Returns (ctas_per_sm, warps_per_system, ms) of the fastest plan shape."""
    best = ctypes.c_int()
    warps = ctypes.c_int()
    ms = ctypes.c_double()
    _check(ctx, lib().la_batch_autotune(ctx.h, ctypes.c_void_p(a_ptr), ctypes.c_void_p(b_ptr),
                                        ctypes.c_void_p(x_ptr), systems, len(systems), mode, tol,
                                        max_iters, table_path.encode() if table_path else None,
                                        ctypes.byref(best), ctypes.byref(warps), ctypes.byref(ms)))
    return best.value, warps.value, ms.value


def batch_features_device(ctx, a_ptr, systems, f_ptr):
    """16 selector features per system into the device buffer f_ptr ([count][16] FP32)."""
    _check(ctx, lib().la_batch_features_device(ctx.h, ctypes.c_void_p(a_ptr), systems,
                                               len(systems), ctypes.c_void_p(f_ptr)))


def generate_conditioned_batch(ctx, systems, log10_kappa_min, log10_kappa_max, seed, a_ptr, b_ptr,
                               kappa_ptr=None):
    """Householder-conditioned systems A = H1 diag(s) H2 written on the device."""
    _check(ctx, lib().la_generate_conditioned_batch(
        ctx.h, systems, len(systems), log10_kappa_min, log10_kappa_max, seed,
        ctypes.c_void_p(a_ptr), ctypes.c_void_p(b_ptr),
        ctypes.c_void_p(kappa_ptr) if kappa_ptr else None))


SELECTOR_CLASSES = (PREC_FP8, PREC_BF16, PREC_FP32)  # MLP class index -> factor precision


class Mlp:
    """The selector network (la_mlp): 16 -> 64 -> 64 -> 3, FP32, trained on the GPU."""

    N_FEATURES = 16

    def __init__(self, ctx, seed=0):
        self.ctx = ctx
        self.h = ctypes.c_void_p()
        _check(ctx, lib().la_mlp_create(ctx.h, ctypes.c_ulonglong(seed), ctypes.byref(self.h)))
        self.nparam = lib().la_mlp_param_count()

    def get_params(self):
        p = np.empty(self.nparam + 32, dtype=np.float32)
        _check(self.ctx, lib().la_mlp_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.nparam + 32:
            raise ValueError("expected %d floats" % (self.nparam + 32))
        _check(self.ctx, lib().la_mlp_set_params(self.h, _ptr(p)))

    def gradients(self, x_ptr, y_ptr, count):
        g = np.empty(self.nparam, dtype=np.float32)
        loss = ctypes.c_float()
        _check(self.ctx, lib().la_mlp_gradients(self.h, ctypes.c_void_p(x_ptr),
                                                ctypes.c_void_p(y_ptr), count, _ptr(g),
                                                ctypes.byref(loss)))
        return g, loss.value

    def train_step(self, x_ptr, y_ptr, count, lr, want_loss=False):
        loss = ctypes.c_float()
        _check(self.ctx, lib().la_mlp_train_step(self.h, ctypes.c_void_p(x_ptr),
                                                 ctypes.c_void_p(y_ptr), count, ctypes.c_float(lr),
                                                 ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def gradients_cost(self, x_ptr, cost_ptr, count):
        """Mean expected cost (cost [count, 3] device FP32) and its gradient."""
        g = np.empty(self.nparam, dtype=np.float32)
        loss = ctypes.c_float()
        _check(self.ctx, lib().la_mlp_gradients_cost(self.h, ctypes.c_void_p(x_ptr),
                                                     ctypes.c_void_p(cost_ptr), count, _ptr(g),
                                                     ctypes.byref(loss)))
        return g, loss.value

    def train_step_cost(self, x_ptr, cost_ptr, count, lr, want_loss=False):
        loss = ctypes.c_float()
        _check(self.ctx, lib().la_mlp_train_step_cost(self.h, ctypes.c_void_p(x_ptr),
                                                      ctypes.c_void_p(cost_ptr), count,
                                                      ctypes.c_float(lr),
                                                      ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def set_gate(self, coef, bias=0.0):
        """Class 3 (straight to the FP64 pass) where coef[:16] . x + coef[16:] . p
        + bias >= 0 (x raw features, p class probabilities); coef None turns
        the gate off."""
        if coef is None:
            _check(self.ctx, lib().la_mlp_set_gate(self.h, None, ctypes.c_float(0.0)))
            return
        c = np.ascontiguousarray(coef, dtype=np.float32)
        if c.size != 19:
            raise ValueError("the gate has 19 coefficients")
        _check(self.ctx, lib().la_mlp_set_gate(self.h, _ptr(c), ctypes.c_float(bias)))

    def predict(self, x_ptr, count, probs_ptr=None, class_ptr=None):
        _check(self.ctx, lib().la_mlp_predict(self.h, ctypes.c_void_p(x_ptr), count,
                                              ctypes.c_void_p(probs_ptr) if probs_ptr else None,
                                              ctypes.c_void_p(class_ptr) if class_ptr else None))

    def free(self):
        if self.h:
            lib().la_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def matrix_mul_device(ctx, a_ptr, lda, b_ptr, ldb, c_ptr, ldc, m_, k, n):
    st = lib().la_matrix_mul_device(ctx.h, ctypes.c_void_p(a_ptr), lda, ctypes.c_void_p(b_ptr),
                                    ldb, ctypes.c_void_p(c_ptr), ldc, m_, k, n)
    return _check(ctx, st)
