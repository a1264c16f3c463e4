"""Host-side mirror of rulinalg's interface for the GPU path, over the C ABI.

Names, argument meaning and error behaviour follow the reference crate:
  * `mat_mul(a, b)`                     <- `&a * &b` (src/matrix/mat_mul.rs:17-143)
  * `PartialPivLu.decompose(m)` ...     <- src/matrix/decomposition/lu.rs:130-300
  * `Cholesky.decompose(m)` ...         <- src/matrix/decomposition/cholesky.rs:93-246
  * `HouseholderQr.decompose(m)` ...    <- src/matrix/decomposition/qr.rs:171-315
  * `HouseholderQr.q().left_multiply_into(x)` <- householder.rs:203-227
  * `solve_u_triangular / solve_l_triangular` <- src/matrix/base/mod.rs:1015-1067
  * `solve/inverse/det(m, ...)`         <- Matrix::solve/inverse/det (src/matrix/impl_mat.rs:354-427)
A numerical failure raises `RulinalgError` with the reference's ErrorKind; a dimension
misuse raises `RulinalgPanic` (the reference panics via assert!). Matrices are numpy
arrays (row-major, like Matrix<T>); float64 and float32 select the f64 and f32 paths.
All arithmetic happens in librulinalg_gb300.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import lib

# status codes (include/rulinalg_gb300.h)
OK = 0
ERROR_KINDS = {
    1: "InvalidArg",
    2: "DecompFailure",
    3: "AlgebraFailure",
    4: "DivByZero",
    5: "ScalarConversionFailure",
    6: "InvalidPermutation",
}
DIV_BY_ZERO = 4
RL_ERR_SHAPE = 16
RL_ERR_NO_DEVICE = 33


class RulinalgError(Exception):
    """A reference `Err(Error)`: `kind` is the ErrorKind name (src/error.rs:21-34)."""

    def __init__(self, status: int):
        self.status = status
        self.kind = ERROR_KINDS.get(status, "Device")
        super().__init__(f"{self.kind}: {lib.rl_status_string(status).decode()}")


class RulinalgPanic(AssertionError):
    """Where the reference panics (assert! on dimensions)."""


class DeviceError(RuntimeError):
    """CUDA failure, no usable GPU, out of memory or a device wait that timed out."""

    def __init__(self, status: int):
        self.status = status
        super().__init__(lib.rl_status_string(status).decode())


def _check(status: int) -> None:
    if status == OK:
        return
    if status in ERROR_KINDS:
        raise RulinalgError(status)
    if status == RL_ERR_SHAPE:
        raise RulinalgPanic(lib.rl_status_string(status).decode())
    raise DeviceError(status)


def _ptr(a: np.ndarray):
    if a.dtype == np.float64:
        return a.ctypes.data_as(C.POINTER(C.c_double))
    if a.dtype == np.float32:
        return a.ctypes.data_as(C.POINTER(C.c_float))
    if a.dtype == np.uint64:
        return a.ctypes.data_as(C.POINTER(C.c_uint64))
    if a.dtype == np.int32:
        return a.ctypes.data_as(C.POINTER(C.c_int32))
    if a.dtype == np.uint8:
        return a.ctypes.data_as(C.POINTER(C.c_uint8))
    raise TypeError(f"unsupported dtype {a.dtype}")


def _prefix(a: np.ndarray) -> str:
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "s"
    raise TypeError("rulinalg_gb300 computes in f32 or f64 (Matrix<f32> / Matrix<f64>)")


def _fn(prefix: str, name: str):
    return getattr(lib, f"rl_{prefix}{name}")


def _mat(a, dtype=None) -> np.ndarray:
    a = np.asarray(a, dtype=dtype)
    if a.ndim != 2:
        raise RulinalgPanic("expected a matrix")
    if a.dtype not in (np.float32, np.float64):
        a = a.astype(np.float64)
    return np.ascontiguousarray(a)


def _row_stride(a: np.ndarray) -> int:
    """Row stride in elements of a 2D array whose rows are contiguous (MatrixSlice)."""
    if a.size == 0:
        return max(a.shape[1], 1)
    if a.shape[1] > 1 and a.strides[1] != a.itemsize:
        raise ValueError("rows must be contiguous")
    return a.strides[0] // a.itemsize if a.shape[0] > 1 else max(a.shape[1], 1)


def mat_mul(a, b) -> np.ndarray:
    """`&a * &b` for Matrix<f32>/Matrix<f64> (mat_mul.rs:17-143); strided row views
    (MatrixSlice with row_stride > cols) are passed through without a copy."""
    a = np.asarray(a)
    b = np.asarray(b)
    if a.ndim != 2 or b.ndim != 2:
        raise RulinalgPanic("expected matrices")
    if a.shape[1] != b.shape[0]:
        raise RulinalgPanic("Matrix dimensions do not agree.")  # mat_mul.rs:21
    if a.dtype != b.dtype:
        raise TypeError("operands must share a dtype")
    if a.dtype not in (np.float32, np.float64):
        raise TypeError("GPU mat_mul covers f32 and f64")
    if a.size == 0 or (a.shape[1] > 1 and a.strides[1] != a.itemsize):
        a = np.ascontiguousarray(a)
    if b.size == 0 or (b.shape[1] > 1 and b.strides[1] != b.itemsize):
        b = np.ascontiguousarray(b)
    m, k = a.shape
    n = b.shape[1]
    c = np.empty((m, n), dtype=a.dtype)
    _check(_fn(_prefix(a), "gemm")(m, k, n, _ptr(a), _row_stride(a), _ptr(b), _row_stride(b), _ptr(c), max(n, 1)))
    return c


# ------------------------------------------------------------------ permutations --
@dataclass
class PermutationMatrix:
    """`PermutationMatrix{perm}` (permutation_matrix.rs:102-111): row i -> perm[i]."""
    perm: np.ndarray

    def size(self) -> int:
        return len(self.perm)

    def as_matrix(self, dtype=np.float64) -> np.ndarray:
        n = len(self.perm)
        m = np.zeros((n, n), dtype=dtype)
        m[np.arange(n), self.perm.astype(np.int64)] = 1
        return m

    def inverse(self) -> "PermutationMatrix":
        inv = np.empty_like(self.perm)
        inv[self.perm.astype(np.int64)] = np.arange(len(self.perm), dtype=self.perm.dtype)
        return PermutationMatrix(inv)

    def det(self) -> float:
        """PermutationMatrix::det (permutation_matrix.rs:254-260): +1 for an even
        permutation, -1 for an odd one (parity by cycle resolution, :216-234)."""
        perm = [int(v) for v in self.perm]
        odd = False
        for i in range(len(perm)):
            target = perm[i]
            while i != target:
                nxt = perm[target]
                odd = not odd
                perm[target] = target
                target = nxt
            perm[i] = i
        return -1.0 if odd else 1.0


@dataclass
class LUP:
    l: np.ndarray
    u: np.ndarray
    p: PermutationMatrix


class PartialPivLu:
    """PA = LU with partial pivoting (lu.rs:130-300), factored on the GPU."""

    def __init__(self, lu: np.ndarray, perm: np.ndarray):
        self.lu = lu
        self.p = PermutationMatrix(perm)

    @staticmethod
    def decompose(matrix) -> "PartialPivLu":
        a = _mat(matrix).copy()
        n = a.shape[1]
        if a.shape[0] != n:
            raise RulinalgPanic("Matrix must be square for LU decomposition.")  # lu.rs:165
        perm = np.arange(n, dtype=np.uint64)
        _check(_fn(_prefix(a), "lu_decompose")(n, _ptr(a), max(n, 1), _ptr(perm)))
        return PartialPivLu(a, perm)

    def solve(self, b) -> np.ndarray:
        n = self.lu.shape[0]
        b = np.array(b, dtype=self.lu.dtype, copy=True, order="C")
        if b.shape[0] != n:
            raise RulinalgPanic("Right-hand side vector must have compatible size.")  # lu.rs:232
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        _check(_fn(_prefix(self.lu), "lu_solve")(n, nrhs, _ptr(self.lu), max(n, 1), _ptr(self.p.perm), _ptr(b),
                                                max(nrhs, 1)))
        return b

    def inverse(self) -> np.ndarray:
        n = self.lu.shape[0]
        inv = np.zeros((n, n), dtype=self.lu.dtype)
        _check(_fn(_prefix(self.lu), "lu_inverse")(n, _ptr(self.lu), max(n, 1), _ptr(self.p.perm), _ptr(inv),
                                                  max(n, 1)))
        return inv

    def det(self) -> float:
        n = self.lu.shape[0]
        out = np.zeros(1, dtype=self.lu.dtype)
        _check(_fn(_prefix(self.lu), "lu_det")(n, _ptr(self.lu), max(n, 1), _ptr(self.p.perm), _ptr(out)))
        return out[0].item()

    def unpack(self) -> LUP:
        """`Decomposition::unpack` (lu.rs:138-149): unit lower L, upper U, P."""
        l = np.tril(self.lu, -1)
        np.fill_diagonal(l, 1)
        u = np.triu(self.lu)
        return LUP(l, u, self.p)


@dataclass
class LUPQ:
    l: np.ndarray
    u: np.ndarray
    p: "PermutationMatrix"
    q: "PermutationMatrix"


class FullPivLu:
    """PAQ = LU with complete pivoting (lu.rs:303-599), factored on the GPU; the factors
    and permutations are bit-identical to the reference's."""

    def __init__(self, lu: np.ndarray, p: np.ndarray, q: np.ndarray):
        self.lu = lu
        self.p = PermutationMatrix(p)
        self.q = PermutationMatrix(q)

    @staticmethod
    def decompose(matrix) -> "FullPivLu":
        a = _mat(matrix).copy()
        n = a.shape[1]
        if a.shape[0] != n:
            raise RulinalgPanic("Matrix must be square for LU decomposition.")  # lu.rs:386-388
        p = np.arange(n, dtype=np.uint64)
        q = np.arange(n, dtype=np.uint64)
        _check(_fn(_prefix(a), "full_lu_decompose")(n, _ptr(a), max(n, 1), _ptr(p), _ptr(q)))
        return FullPivLu(a, p, q)

    def solve(self, b) -> np.ndarray:
        n = self.lu.shape[0]
        b = np.array(b, dtype=self.lu.dtype, copy=True, order="C")
        if b.shape[0] != n:
            raise RulinalgPanic("Right-hand side vector must have compatible size.")  # lu.rs:481
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        _check(_fn(_prefix(self.lu), "full_lu_solve")(n, nrhs, _ptr(self.lu), max(n, 1), _ptr(self.p.perm),
                                                     _ptr(self.q.perm), _ptr(b), max(nrhs, 1)))
        return b

    def _epsilon(self) -> float:
        """|lu[0, 0]| eps (lu.rs:595-597); 1 eps for an empty matrix."""
        n = self.lu.shape[0]
        return abs(float(self.lu[0, 0]) if n else 1.0) * float(np.finfo(self.lu.dtype).eps)

    def rank(self) -> int:
        """FullPivLu::rank (lu.rs:547-561)."""
        eps, r = self._epsilon(), 0
        for i in range(self.lu.shape[0]):
            if abs(float(self.lu[i, i])) > eps:
                r += 1
            else:
                break
        return r

    def is_invertible(self) -> bool:
        """FullPivLu::is_invertible (lu.rs:582-593)."""
        n = self.lu.shape[0]
        return True if n == 0 else abs(float(self.lu[n - 1, n - 1])) > self._epsilon()

    def det(self) -> float:
        """FullPivLu::det (lu.rs:512-524): p_det * (fold of diag(U)) * q_det."""
        u_det = self.lu.dtype.type(1)
        with np.errstate(over="ignore"):  # the reference's fold overflows to inf the same way
            for i in range(self.lu.shape[0]):
                u_det = u_det * self.lu[i, i]
            return float(self.p.det() * u_det * self.q.det())

    def inverse(self) -> np.ndarray:
        """FullPivLu::inverse (lu.rs:493-509): DivByZero when not invertible."""
        n = self.lu.shape[0]
        if not self.is_invertible():
            raise RulinalgError(DIV_BY_ZERO)
        return self.solve(np.eye(n, dtype=self.lu.dtype))

    def unpack(self) -> LUPQ:
        """`Decomposition::unpack` (lu.rs:345-361): unit lower L, upper U, P, Q."""
        l = np.tril(self.lu, -1)
        np.fill_diagonal(l, 1)
        return LUPQ(l, np.triu(self.lu), self.p, self.q)


class Cholesky:
    """A = L L^T (cholesky.rs:93-246), factored on the GPU."""

    def __init__(self, l: np.ndarray):
        self.l = l

    @staticmethod
    def decompose(matrix) -> "Cholesky":
        a = _mat(matrix).copy()
        n = a.shape[0]
        if a.shape[1] != n:
            raise RulinalgPanic("Matrix must be square for Cholesky decomposition.")  # cholesky.rs:117
        _check(_fn(_prefix(a), "cholesky_decompose")(n, _ptr(a), max(n, 1)))
        return Cholesky(a)

    def solve(self, b) -> np.ndarray:
        n = self.l.shape[0]
        b = np.array(b, dtype=self.l.dtype, copy=True, order="C")
        if b.shape[0] != n:
            raise RulinalgPanic("RHS vector and coefficient matrix must be dimensionally compatible.")
        nrhs = 1 if b.ndim == 1 else b.shape[1]
        _check(_fn(_prefix(self.l), "cholesky_solve")(n, nrhs, _ptr(self.l), max(n, 1), _ptr(b), max(nrhs, 1)))
        return b

    def inverse(self) -> np.ndarray:
        n = self.l.shape[0]
        inv = np.zeros((n, n), dtype=self.l.dtype)
        _check(_fn(_prefix(self.l), "cholesky_inverse")(n, _ptr(self.l), max(n, 1), _ptr(inv), max(n, 1)))
        return inv

    def det(self) -> float:
        n = self.l.shape[0]
        out = np.zeros(1, dtype=self.l.dtype)
        _check(_fn(_prefix(self.l), "cholesky_det")(n, _ptr(self.l), max(n, 1), _ptr(out)))
        return out[0].item()

    def unpack(self) -> np.ndarray:
        """cholesky.rs:237-246: L with the strict upper triangle zeroed."""
        return np.tril(self.l)


@dataclass
class QR:
    q: np.ndarray
    r: np.ndarray


@dataclass
class ThinQR:
    q1: np.ndarray
    r1: np.ndarray


class HouseholderQr:
    """Compact Householder QR (qr.rs:171-315), factored on the GPU."""

    def __init__(self, qr: np.ndarray, tau: np.ndarray):
        self.qr = qr
        self.tau = tau

    @staticmethod
    def decompose(matrix) -> "HouseholderQr":
        a = _mat(matrix).copy()
        m, n = a.shape
        tau = np.zeros(min(m, n), dtype=a.dtype)
        _check(_fn(_prefix(a), "qr_decompose")(m, n, _ptr(a), max(n, 1), _ptr(tau)))
        return HouseholderQr(a, tau)

    def first_k_columns(self, k: int) -> np.ndarray:
        """HouseholderComposition::first_k_columns (householder.rs:235-268)."""
        m, n = self.qr.shape
        if k > m:
            raise RulinalgPanic("k cannot exceed m, the number of rows of Q")
        q = np.zeros((m, k), dtype=self.qr.dtype)
        tau = self.tau if len(self.tau) else np.zeros(1, dtype=self.qr.dtype)
        _check(_fn(_prefix(self.qr), "qr_first_k_columns")(m, n, _ptr(self.qr), max(n, 1), _ptr(tau), k, _ptr(q),
                                                          max(k, 1)))
        return q

    def q(self) -> "HouseholderComposition":
        """HouseholderQr::q (qr.rs:228-230): Q as a composition of the stored reflectors."""
        return HouseholderComposition(self)

    def unpack(self) -> QR:
        m = self.qr.shape[0]
        return QR(self.first_k_columns(m), np.triu(self.qr))

    def unpack_thin(self) -> ThinQR:
        m, n = self.qr.shape
        if m <= n:
            qr = self.unpack()
            return ThinQR(qr.q, qr.r)
        return ThinQR(self.first_k_columns(n), np.triu(self.qr[:n, :]))


class HouseholderComposition:
    """Q = H_0 H_1 ... H_{p-1} of a compact QR (householder.rs:177-284), applied on the GPU
    without forming Q."""

    def __init__(self, qr: HouseholderQr):
        self._qr = qr

    def _apply(self, x, trans: bool) -> None:
        st = self._qr
        m, n = st.qr.shape
        if not isinstance(x, np.ndarray) or x.dtype != st.qr.dtype or x.ndim != 2 or not x.flags.c_contiguous:
            raise RulinalgPanic("expected a C-contiguous matrix of the factor's type")
        if x.shape[0] != m:
            raise RulinalgPanic("Number of rows of Q and X must agree")  # householder.rs:205
        tau = st.tau if len(st.tau) else np.zeros(1, dtype=st.qr.dtype)
        name = "qr_q_apply_t" if trans else "qr_q_apply"
        _check(_fn(_prefix(st.qr), name)(m, n, _ptr(st.qr), max(n, 1), _ptr(tau), x.shape[1], _ptr(x),
                                        max(x.shape[1], 1)))

    def left_multiply_into(self, x: np.ndarray) -> None:
        """HouseholderComposition::left_multiply_into (householder.rs:203-227): x <- Q x in place."""
        self._apply(x, False)

    def left_multiply_into_transposed(self, x: np.ndarray) -> None:
        """x <- Q^T x in place (the q1^T b of least squares, without forming Q)."""
        self._apply(x, True)

    def first_k_columns(self, k: int) -> np.ndarray:
        """HouseholderComposition::first_k_columns (householder.rs:235-268)."""
        return self._qr.first_k_columns(k)


def _triangular(t, b, upper: bool) -> np.ndarray:
    t = _mat(t)
    n = t.shape[0]
    if t.shape[1] != n:
        raise RulinalgPanic("Matrix must be square to solve a triangular system.")
    x = np.array(b, dtype=t.dtype, copy=True, order="C")
    if x.shape[0] != n:
        raise RulinalgPanic("Vector size must match the number of rows of the matrix.")
    nrhs = 1 if x.ndim == 1 else x.shape[1]
    _check(_fn(_prefix(t), "trsv_upper" if upper else "trsv_lower")(n, nrhs, _ptr(t), max(n, 1), _ptr(x),
                                                                   max(nrhs, 1)))
    return x


def solve_u_triangular(u, y) -> np.ndarray:
    """BaseMatrix::solve_u_triangular (base/mod.rs:1015-1024): back substitution with the
    upper triangle of u (its strict lower part is ignored); DivByZero for |u_ii| < eps."""
    return _triangular(u, y, True)


def solve_l_triangular(l, y) -> np.ndarray:
    """BaseMatrix::solve_l_triangular (base/mod.rs:1058-1067): forward substitution with the
    lower triangle of l; DivByZero for |l_ii| < eps."""
    return _triangular(l, y, False)


class ResidentFactor:
    """A device-resident factorisation (rl_factor_*) for repeated f64-accurate solves:
    `a` and each `b` / `x` are device buffers given as torch CUDA tensors (float64,
    row-major contiguous); `kind` is "lu" or "cholesky"."""

    def __init__(self, a, kind: str = "lu", stream: int = 0):
        n = a.shape[0]
        if a.shape != (n, n) or not a.is_contiguous():
            raise RulinalgPanic("Matrix must be square and contiguous")
        self.n = n
        h = C.c_void_p()
        _check(lib.rl_factor_create(C.byref(h), 1 if kind == "cholesky" else 0, n, a.data_ptr(), n, stream or None))
        self._h = h

    def solve(self, b, x, stream: int = 0) -> dict:
        from ._lib import SolveInfo
        nrhs = 1 if b.dim() == 1 else b.shape[1]
        if b.shape[0] != self.n or x.shape != b.shape or not b.is_contiguous() or not x.is_contiguous():
            raise RulinalgPanic("Right-hand side and solution must be n x nrhs and contiguous")
        info = SolveInfo()
        _check(lib.rl_factor_solve(self._h, nrhs, b.data_ptr(), nrhs, x.data_ptr(), nrhs, C.byref(info),
                                   stream or None))
        return {"iters": info.iters, "gmres_iters": info.gmres_iters, "path": PATHS.get(info.path, info.path),
                "berr": info.berr}

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.rl_factor_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def least_squares(matrix, b) -> np.ndarray:
    """min ||A x - b|| through Householder QR (m >= n); no reference routine exists, it is
    the composition unpack_thin -> q1^T b -> r1.solve_u_triangular."""
    a = _mat(matrix).copy()
    m, n = a.shape
    b = np.ascontiguousarray(b, dtype=a.dtype)
    if b.shape != (m,):
        raise RulinalgPanic("right-hand side must have m entries")
    x = np.zeros(n, dtype=a.dtype)
    _check(_fn(_prefix(a), "qr_least_squares")(m, n, _ptr(a), max(n, 1), _ptr(b), _ptr(x)))
    return x


def solve(matrix, y) -> np.ndarray:
    """Matrix::solve (impl_mat.rs:354-356)."""
    a = _mat(matrix).copy()
    n = a.shape[0]
    if a.shape[1] != n:
        raise RulinalgPanic("Matrix must be square for LU decomposition.")
    y = np.array(y, dtype=a.dtype, copy=True)
    if y.shape != (n,):
        raise RulinalgPanic("Right-hand side vector must have compatible size.")
    _check(_fn(_prefix(a), "matrix_solve")(n, _ptr(a), max(n, 1), _ptr(y)))
    return y


def inverse(matrix) -> np.ndarray:
    """Matrix::inverse (impl_mat.rs:386-388)."""
    a = _mat(matrix).copy()
    n = a.shape[0]
    if a.shape[1] != n:
        raise RulinalgPanic("Matrix must be square for LU decomposition.")
    inv = np.zeros((n, n), dtype=a.dtype)
    _check(_fn(_prefix(a), "matrix_inverse")(n, _ptr(a), max(n, 1), _ptr(inv), max(n, 1)))
    return inv


def det(matrix) -> float:
    """Matrix::det (impl_mat.rs:407-427)."""
    a = _mat(matrix).copy()
    n = a.shape[0]
    if a.shape[1] != n:
        raise RulinalgPanic("Matrix is not square.")
    out = np.zeros(1, dtype=a.dtype)
    _check(_fn(_prefix(a), "matrix_det")(n, _ptr(a), max(n, 1), _ptr(out)))
    return out[0].item()


PATHS = {0: "refinement", 1: "gmres-ir", 2: "fp64"}


def solve_mixed(matrix, b, kind: str = "lu"):
    """f64 solve through the mixed-precision single-system solver (FP32 factor, FP64
    refinement, GMRES-IR, FP64 refactor as needed). Returns (x, info) where info has
    iters, gmres_iters, path and berr (max normwise backward error over the columns)."""
    from ._lib import SolveInfo
    a = np.ascontiguousarray(matrix, dtype=np.float64)
    n = a.shape[0]
    if a.shape != (n, n):
        raise RulinalgPanic("Matrix must be square.")
    bb = np.ascontiguousarray(b, dtype=np.float64)
    vec = bb.ndim == 1
    bb = bb.reshape(n, -1)
    nrhs = bb.shape[1]
    x = np.zeros_like(bb)
    info = SolveInfo()
    k = 1 if kind == "cholesky" else 0
    _check(lib.rl_dsolve_mixed(n, nrhs, k, _ptr(a), max(n, 1), _ptr(bb), max(nrhs, 1), _ptr(x), max(nrhs, 1),
                               C.byref(info)))
    out = {"iters": info.iters, "gmres_iters": info.gmres_iters, "path": PATHS.get(info.path, info.path),
           "berr": info.berr}
    return (x[:, 0] if vec else x), out


def lstsq_mixed(matrix, b):
    """min ||A x - b||_2 (m >= n) through the mixed-precision least-squares solver (FP32
    Householder QR, FP64 corrected semi-normal-equation refinement, FP64 QR fallback).
    Returns (x, info) with iters, path and berr (the scaled normal-equations residual)."""
    from ._lib import SolveInfo
    a = np.ascontiguousarray(matrix, dtype=np.float64)
    if a.ndim != 2:
        raise RulinalgPanic("Matrix must be two-dimensional.")
    m, n = a.shape
    bb = np.ascontiguousarray(b, dtype=np.float64).reshape(-1)
    if bb.shape[0] != m:
        raise RulinalgPanic("Matrix and vector dimensions are not compatible.")
    x = np.zeros(n, dtype=np.float64)
    info = SolveInfo()
    _check(lib.rl_dlstsq_mixed(m, n, _ptr(a), max(n, 1), _ptr(bb), _ptr(x), C.byref(info)))
    return x, {"iters": info.iters, "gmres_iters": info.gmres_iters, "path": PATHS.get(info.path, info.path),
               "berr": info.berr}
