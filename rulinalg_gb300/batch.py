"""Batched solves over the C ABI (rl_batch_plan_*): many independent LU / Cholesky
systems with n <= 512 in one GPU launch sequence. The reference has no batched routine;
this replaces a caller's loop over `PartialPivLu::decompose(a)?.solve(b)` /
`Cholesky::decompose(a)?.solve(b)` (src/matrix/decomposition/lu.rs:163-244,
cholesky.rs:116-202)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import lib
from .api import _check, _ptr

KIND_LU = 0
KIND_CHOLESKY = 1
PREC_FP64 = 0    # plain FP64 factor and solve
PREC_MIXED = 1   # FP32 factor + FP64 iterative refinement, FP64 refactor fallback
PREC_FP32 = 2    # f32 systems, FP32 throughout


class BatchPlan:
    """Sizes, kinds and precision of a batch; owns the device schedule and workspace."""

    def __init__(self, n, kind=None, precision: int = PREC_MIXED):
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.count = len(self.n)
        self.kind = (np.zeros(self.count, dtype=np.uint8) if kind is None
                     else np.ascontiguousarray(kind, dtype=np.uint8))
        self.precision = precision
        self.dtype = np.float32 if precision == PREC_FP32 else np.float64
        h = C.c_void_p()
        _check(lib.rl_batch_plan_create(C.byref(h), self.count, _ptr(self.n) if self.count else None,
                                        _ptr(self.kind) if self.count else None, precision))
        self._h = h
        self.a_offset = np.zeros(max(self.count, 1), dtype=np.int64)
        self.b_offset = np.zeros(max(self.count, 1), dtype=np.int64)
        at, bt = C.c_int64(), C.c_int64()
        _check(lib.rl_batch_plan_layout(h, self.a_offset.ctypes.data_as(C.POINTER(C.c_int64)),
                                        self.b_offset.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(at), C.byref(bt)))
        self.a_total, self.b_total = at.value, bt.value

    def pack(self, mats, rhs):
        """Packs lists of square matrices and right-hand sides into the plan's layout."""
        a = np.empty(self.a_total, dtype=self.dtype)
        b = np.empty(self.b_total, dtype=self.dtype)
        for i, (m, v) in enumerate(zip(mats, rhs)):
            k = int(self.n[i])
            a[self.a_offset[i]:self.a_offset[i] + k * k] = np.asarray(m, dtype=self.dtype).reshape(-1)
            b[self.b_offset[i]:self.b_offset[i] + k] = v
        return a, b

    def unpack(self, x):
        return [x[self.b_offset[i]:self.b_offset[i] + int(self.n[i])] for i in range(self.count)]

    def solve(self, a, b):
        """Host buffers in, host buffers out (blocking). Returns x, info, iters, berr."""
        a = np.ascontiguousarray(a, dtype=self.dtype)
        b = np.ascontiguousarray(b, dtype=self.dtype)
        x = np.zeros(max(self.b_total, 1), dtype=self.dtype)
        info = np.zeros(max(self.count, 1), dtype=np.int32)
        iters = np.zeros(max(self.count, 1), dtype=np.int32)
        berr = np.zeros(max(self.count, 1), dtype=np.float64)
        fn = lib.rl_sbatch_solve if self.precision == PREC_FP32 else lib.rl_dbatch_solve
        _check(fn(self._h, _ptr(a), _ptr(b), _ptr(x), _ptr(info), _ptr(iters), _ptr(berr)))
        c = self.count
        return x[:self.b_total], info[:c], iters[:c], berr[:c]

    def solve_dev(self, a_ptr: int, b_ptr: int, x_ptr: int, info_ptr: int, iters_ptr: int = 0, berr_ptr: int = 0,
                  stream: int = 0) -> None:
        """Device pointers (e.g. torch tensor data_ptr()); asynchronous on `stream`."""
        fn = lib.rl_sbatch_solve_dev if self.precision == PREC_FP32 else lib.rl_dbatch_solve_dev
        _check(fn(self._h, a_ptr, b_ptr, x_ptr, info_ptr, iters_ptr or None, berr_ptr or None, stream or None))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.rl_batch_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
