"""The oracle: numpy-facing ctypes wrapper of liboracle.so, the plain-C restatement of
rulinalg 0.4.2's dense hot path (see rulinalg_oracle.c / oracle_impl.h for the
file:line of every function it follows).

TEST INFRASTRUCTURE ONLY. The tests, the smoke check and the benchmark's CPU-baseline
leg use it as the checker or the timed CPU reference; the product (rulinalg_gb300)
never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
_SO = _DIR / "liboracle.so"
_SRC = [_DIR / "rulinalg_oracle.c", _DIR / "oracle_impl.h"]

if not _SO.exists() or _SO.stat().st_mtime < max(p.stat().st_mtime for p in _SRC):
    subprocess.run(["make", "-s", "-C", str(_DIR)], check=True)

_lib = C.CDLL(str(_SO))

OK, DIV_BY_ZERO, DECOMP_FAILURE, INVALID_PERMUTATION = 0, 4, 2, 6


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


_sz, _vp = C.c_size_t, C.c_void_p
for sfx, ct in (("d", C.c_double), ("s", C.c_float)):
    for name, res, args in (
        ("or_dot", ct, [_sz, _vp, _vp]),
        ("or_gemm", None, [_sz, _sz, _sz, _vp, _sz, _vp, _sz, _vp, _sz]),
        ("or_matvec", None, [_sz, _sz, _vp, _sz, _vp, _vp]),
        ("or_norm_frobenius", ct, [_sz, _sz, _vp, _sz]),
        ("or_lu_decompose", C.c_int, [_sz, _vp, _sz, _vp, _vp]),
        ("or_lu_solve", C.c_int, [_sz, _vp, _sz, _vp, _vp]),
        ("or_lu_inverse", C.c_int, [_sz, _vp, _sz, _vp, _vp, _sz]),
        ("or_lu_det", ct, [_sz, _vp, _sz, _vp]),
        ("or_matrix_det", ct, [_sz, _vp, _sz]),
        ("or_back_substitution", C.c_int, [_sz, _vp, _sz, _vp]),
        ("or_forward_substitution", C.c_int, [_sz, _vp, _sz, _vp]),
        ("or_chol_decompose", C.c_int, [_sz, _vp, _sz]),
        ("or_chol_solve", C.c_int, [_sz, _vp, _sz, _vp]),
        ("or_chol_det", ct, [_sz, _vp, _sz]),
        ("or_chol_inverse", C.c_int, [_sz, _vp, _sz, _vp, _sz]),
        ("or_transpose_back_substitution", C.c_int, [_sz, _vp, _sz, _vp]),
        ("or_house_compute", ct, [_sz, _vp]),
        ("or_house_apply", None, [_sz, _sz, _vp, _sz, _vp, ct, _vp]),
        ("or_qr_decompose", None, [_sz, _sz, _vp, _sz, _vp]),
        ("or_qr_first_k_columns", None, [_sz, _sz, _vp, _sz, _vp, _sz, _vp, _sz]),
        ("or_qr_q_left_multiply", None, [_sz, _sz, _vp, _sz, _vp, _sz, _vp, _sz]),
        ("or_qr_qt_left_multiply", None, [_sz, _sz, _vp, _sz, _vp, _sz, _vp, _sz]),
        ("or_full_lu_decompose", None, [_sz, _vp, _sz, _vp, _vp, _vp, _vp]),
        ("or_full_lu_solve", C.c_int, [_sz, _vp, _sz, _vp, _vp, _vp]),
        ("or_qr_lstsq", C.c_int, [_sz, _sz, _vp, _sz, _vp, _vp]),
        ("or_gemm_mt", None, [_sz, _sz, _sz, _vp, _sz, _vp, _sz, _vp, _sz, C.c_int]),
        ("or_lu_decompose_mt", C.c_int, [_sz, _vp, _sz, _vp, _vp, C.c_int]),
        ("or_solve_columns_mt", C.c_int, [_sz, _vp, _sz, _vp, _sz, _vp, _sz, C.c_int]),
    ):
        f = getattr(_lib, f"{name}_{sfx}")
        f.restype = res
        f.argtypes = args
_lib.or_perm_parity_odd.restype = C.c_int
_lib.or_perm_parity_odd.argtypes = [_sz, _vp]
_lib.or_perm_validate.restype = C.c_int
_lib.or_perm_validate.argtypes = [_sz, _vp]
_lib.or_batch_solve_d.restype = None
_lib.or_batch_solve_d.argtypes = [_sz, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int]


def _sfx(a):
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "s"
    raise TypeError(a.dtype)


def _f(a, name):
    return getattr(_lib, f"{name}_{_sfx(a)}")


def _m(a, dtype=None):
    return np.array(a, dtype=dtype if dtype is not None else np.asarray(a).dtype, copy=True, order="C")


def dot(u, v):
    u = _m(u)
    v = _m(v, u.dtype)
    return _f(u, "or_dot")(min(len(u), len(v)), _p(u), _p(v))


def gemm(a, b, threads=1):
    """The i-k-j GEMM; threads > 1 splits the rows of C (bit-identical results)."""
    a = _m(a)
    b = _m(b, a.dtype)
    m, k = a.shape
    n = b.shape[1]
    c = np.zeros((m, n), dtype=a.dtype)
    if threads > 1:
        _f(a, "or_gemm_mt")(m, k, n, _p(a), max(k, 1), _p(b), max(n, 1), _p(c), max(n, 1), threads)
    else:
        _f(a, "or_gemm")(m, k, n, _p(a), max(k, 1), _p(b), max(n, 1), _p(c), max(n, 1))
    return c


def matvec(a, x):
    a = _m(a)
    x = _m(x, a.dtype)
    y = np.zeros(a.shape[0], dtype=a.dtype)
    _f(a, "or_matvec")(a.shape[0], a.shape[1], _p(a), max(a.shape[1], 1), _p(x), _p(y))
    return y


def norm_frobenius(a):
    a = _m(a)
    return _f(a, "or_norm_frobenius")(a.shape[0], a.shape[1], _p(a), max(a.shape[1], 1))


def lu_decompose(a, gaps=False, threads=1):
    """Returns (lu, perm, status[, gap per step]); threads > 1 splits every step's
    elimination rows over threads (bit-identical results)."""
    lu = _m(a)
    n = lu.shape[0]
    perm = np.zeros(max(n, 1), dtype=np.uint64)
    gap = np.zeros(max(n, 1), dtype=lu.dtype)
    if threads > 1:
        st = _f(lu, "or_lu_decompose_mt")(n, _p(lu), max(n, 1), _p(perm), _p(gap) if gaps else None, threads)
    else:
        st = _f(lu, "or_lu_decompose")(n, _p(lu), max(n, 1), _p(perm), _p(gap) if gaps else None)
    if gaps:
        return lu, perm[:n], st, gap[:n]
    return lu, perm[:n], st


def lu_solve(lu, perm, b):
    lu = _m(lu)
    perm = _m(perm, np.uint64)
    x = _m(b, lu.dtype)
    st = _f(lu, "or_lu_solve")(lu.shape[0], _p(lu), max(lu.shape[0], 1), _p(perm), _p(x))
    return x, st


def solve_columns(lu, perm, b, threads=1):
    """PartialPivLu::solve (perm given) or Cholesky::solve (perm None) of every column of
    the n x nrhs array b, columns split over threads. Returns (x, status)."""
    lu = _m(lu)
    n = lu.shape[0]
    x = _m(np.asarray(b).reshape(n, -1), lu.dtype)
    pp = _m(perm, np.uint64) if perm is not None else None
    st = _f(lu, "or_solve_columns_mt")(n, _p(lu), max(n, 1), _p(pp) if pp is not None else None, x.shape[1], _p(x),
                                       max(x.shape[1], 1), threads)
    return x, st


def full_lu_decompose(a):
    """FullPivLu::decompose: returns (lu, p, q, piv_r, piv_c) (stored permutations and
    the per-step pivot positions, -1 after a zero pivot ended the elimination)."""
    lu = _m(a)
    n = lu.shape[0]
    p = np.zeros(max(n, 1), dtype=np.uint64)
    q = np.zeros(max(n, 1), dtype=np.uint64)
    pr = np.zeros(max(n, 1), dtype=np.int64)
    pc = np.zeros(max(n, 1), dtype=np.int64)
    _f(lu, "or_full_lu_decompose")(n, _p(lu), max(n, 1), _p(p), _p(q), _p(pr), _p(pc))
    return lu, p[:n], q[:n], pr[:n], pc[:n]


def full_lu_solve(lu, p, q, b):
    lu = _m(lu)
    x = _m(b, lu.dtype)
    st = _f(lu, "or_full_lu_solve")(lu.shape[0], _p(lu), max(lu.shape[0], 1), _p(_m(p, np.uint64)),
                                    _p(_m(q, np.uint64)), _p(x))
    return x, st


def full_lu_rank(lu):
    """FullPivLu::rank (lu.rs:547-561): diagonal entries above |lu[0,0]| eps, counted up
    to the first that is not."""
    n = lu.shape[0]
    eps = abs(lu[0, 0] if n else lu.dtype.type(1)) * np.finfo(lu.dtype).eps
    r = 0
    for i in range(n):
        if abs(lu[i, i]) > eps:
            r += 1
        else:
            break
    return r


def full_lu_is_invertible(lu):
    """FullPivLu::is_invertible (lu.rs:582-593)."""
    n = lu.shape[0]
    if n == 0:
        return True
    return abs(lu[n - 1, n - 1]) > abs(lu[0, 0]) * np.finfo(lu.dtype).eps


def lu_inverse(lu, perm):
    lu = _m(lu)
    n = lu.shape[0]
    perm = _m(perm, np.uint64)
    inv = np.zeros((n, n), dtype=lu.dtype)
    st = _f(lu, "or_lu_inverse")(n, _p(lu), max(n, 1), _p(perm), _p(inv), max(n, 1))
    return inv, st


def lu_det(lu, perm):
    lu = _m(lu)
    perm = _m(perm, np.uint64)
    return _f(lu, "or_lu_det")(lu.shape[0], _p(lu), max(lu.shape[0], 1), _p(perm))


def matrix_det(a):
    a = _m(a)
    return _f(a, "or_matrix_det")(a.shape[0], _p(a), max(a.shape[0], 1))


def perm_parity_odd(perm):
    perm = _m(perm, np.uint64)
    return _lib.or_perm_parity_odd(len(perm), _p(perm))


def perm_validate(perm):
    perm = _m(perm, np.uint64)
    return _lib.or_perm_validate(len(perm), _p(perm))


def back_substitution(u, y):
    u = _m(u)
    x = _m(y, u.dtype)
    return x, _f(u, "or_back_substitution")(u.shape[0], _p(u), max(u.shape[0], 1), _p(x))


def forward_substitution(l, y):
    l = _m(l)
    x = _m(y, l.dtype)
    return x, _f(l, "or_forward_substitution")(l.shape[0], _p(l), max(l.shape[0], 1), _p(x))


def transpose_back_substitution(l, y):
    l = _m(l)
    x = _m(y, l.dtype)
    return x, _f(l, "or_transpose_back_substitution")(l.shape[0], _p(l), max(l.shape[0], 1), _p(x))


def chol_decompose(a):
    """Returns (l_storage, status); the strict upper triangle keeps the input's values."""
    l = _m(a)
    st = _f(l, "or_chol_decompose")(l.shape[0], _p(l), max(l.shape[0], 1))
    return l, st


def chol_solve(l, b):
    l = _m(l)
    x = _m(b, l.dtype)
    return x, _f(l, "or_chol_solve")(l.shape[0], _p(l), max(l.shape[0], 1), _p(x))


def chol_det(l):
    l = _m(l)
    return _f(l, "or_chol_det")(l.shape[0], _p(l), max(l.shape[0], 1))


def chol_inverse(l):
    l = _m(l)
    n = l.shape[0]
    inv = np.zeros((n, n), dtype=l.dtype)
    return inv, _f(l, "or_chol_inverse")(n, _p(l), max(n, 1), _p(inv), max(n, 1))


def house_compute(x):
    x = _m(x)
    tau = _f(x, "or_house_compute")(len(x), _p(x))
    return x, tau


def house_apply(a, v, tau):
    a = _m(a)
    v = _m(v, a.dtype)
    u = np.zeros(max(a.shape[1], 1), dtype=a.dtype)
    _f(a, "or_house_apply")(a.shape[0], a.shape[1], _p(a), max(a.shape[1], 1), _p(v), tau, _p(u))
    return a


def qr_decompose(a):
    qr = _m(a)
    m, n = qr.shape
    tau = np.zeros(max(min(m, n), 1), dtype=qr.dtype)
    _f(qr, "or_qr_decompose")(m, n, _p(qr), max(n, 1), _p(tau))
    return qr, tau[:min(m, n)]


def qr_first_k_columns(qr, tau, k):
    qr = _m(qr)
    m, n = qr.shape
    tau = _m(tau if len(tau) else np.zeros(1), qr.dtype)
    q = np.zeros((m, k), dtype=qr.dtype)
    _f(qr, "or_qr_first_k_columns")(m, n, _p(qr), max(n, 1), _p(tau), k, _p(q), max(k, 1))
    return q


def qr_q_left_multiply(qr, tau, x):
    qr = _m(qr)
    m, n = qr.shape
    tau = _m(tau if len(tau) else np.zeros(1), qr.dtype)
    x = _m(x, qr.dtype)
    _f(qr, "or_qr_q_left_multiply")(m, n, _p(qr), max(n, 1), _p(tau), x.shape[1], _p(x), max(x.shape[1], 1))
    return x


def qr_qt_left_multiply(qr, tau, x):
    qr = _m(qr)
    m, n = qr.shape
    tau = _m(tau if len(tau) else np.zeros(1), qr.dtype)
    x = _m(x, qr.dtype)
    _f(qr, "or_qr_qt_left_multiply")(m, n, _p(qr), max(n, 1), _p(tau), x.shape[1], _p(x), max(x.shape[1], 1))
    return x


def qr_lstsq(a, b):
    a = _m(a)
    m, n = a.shape
    b = _m(b, a.dtype)
    x = np.zeros(max(n, 1), dtype=a.dtype)
    st = _f(a, "or_qr_lstsq")(m, n, _p(a), max(n, 1), _p(b), _p(x))
    return x[:n], st


def batch_solve(n, kind, a_off, a, b_off, b, threads=1):
    """Loops the reference's decompose + solve over a packed f64 batch (a, b consumed)."""
    n = _m(n, np.int32)
    kind = _m(kind, np.uint8)
    a_off = _m(a_off, np.int64)
    b_off = _m(b_off, np.int64)
    info = np.zeros(max(len(n), 1), dtype=np.int32)
    _lib.or_batch_solve_d(len(n), _p(n), _p(kind), _p(a_off), _p(a), _p(b_off), _p(b), _p(info), threads)
    return info[:len(n)]
