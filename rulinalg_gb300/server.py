"""The serving loop (rl_server_*): continuous batching of f64-accurate LU / Cholesky
solves, device-resident factors for re-solves, QR least squares, admission by device
memory footprint, p50/p99 latency. All work runs in librulinalg_gb300.so."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import REQUEST_DTYPE, RESULT_DTYPE, Request, Result, ServerConfig, ServerStats, lib
from .api import _check

REQ_LU, REQ_CHOLESKY, REQ_LSTSQ, REQ_RESOLVE = 0, 1, 2, 3
PATHS = {0: "refinement", 1: "gmres-ir", 2: "fp64"}


def _vp(a: np.ndarray) -> int:
    return a.ctypes.data


class Server:
    def __init__(self, hbm_budget_bytes: int = 0, workers: int = 0, max_batch: int = 0, small_n: int = 0,
                 max_pending: int = 0):
        cfg = ServerConfig(hbm_budget_bytes, workers, max_batch, small_n, max_pending)
        h = C.c_void_p()
        _check(lib.rl_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = {}  # ticket -> host buffers that must outlive the request

    def submit(self, kind: int, a=None, b=None, retain: bool = False, factor: int = 0, n: int | None = None) -> tuple:
        """Returns (ticket, x) where x is filled when the ticket completes."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        if kind == REQ_RESOLVE:
            nn = len(b) if n is None else n
            m = nn
            a_arr = None
        else:
            a_arr = np.ascontiguousarray(a, dtype=np.float64)
            m, nn = a_arr.shape
        x = np.zeros(nn, dtype=np.float64)
        req = Request(kind, int(retain), factor, m, nn, _vp(a_arr) if a_arr is not None else None, _vp(b), _vp(x))
        t = C.c_uint64()
        _check(lib.rl_server_submit(self._h, C.byref(req), C.byref(t)))
        self._keep[t.value] = (a_arr, b, x)
        return t.value, x

    def wait(self, ticket: int, timeout_s: float = -1.0) -> dict:
        r = Result()
        _check(lib.rl_server_wait(self._h, ticket, timeout_s, C.byref(r)))
        _, _, x = self._keep.pop(ticket)
        return {"status": r.status, "iters": r.iters, "path": PATHS.get(r.path, r.path), "berr": r.berr,
                "factor": r.factor, "queue_us": r.queue_us, "latency_us": r.latency_us, "x": x}

    def release_factor(self, factor: int) -> None:
        _check(lib.rl_server_release_factor(self._h, factor))

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib.rl_server_stats_get(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        _check(lib.rl_server_reset_stats(self._h))

    def replay(self, arrivals_s, requests) -> list:
        """requests: list of (kind, a, b, factor) with host arrays; submitted at the given
        arrival times by the library's replay thread. Returns per-request result dicts."""
        count = len(requests)
        reqs = (Request * count)()
        xs = []
        keep = []
        for i, (kind, a, b, factor) in enumerate(requests):
            b = np.ascontiguousarray(b, dtype=np.float64)
            if kind == REQ_RESOLVE:
                m = nn = len(b)
                ap = None
            else:
                a = np.ascontiguousarray(a, dtype=np.float64)
                m, nn = a.shape
                ap = _vp(a)
            x = np.zeros(nn, dtype=np.float64)
            keep.append((a, b))
            xs.append(x)
            reqs[i] = Request(kind, 0, factor, m, nn, ap, _vp(b), _vp(x))
        arr = np.ascontiguousarray(arrivals_s, dtype=np.float64)
        res = (Result * count)()
        _check(lib.rl_server_replay(self._h, count, arr.ctypes.data_as(C.c_void_p), reqs, res))
        return [{"status": r.status, "iters": r.iters, "path": PATHS.get(r.path, r.path), "berr": r.berr,
                 "latency_us": r.latency_us, "queue_us": r.queue_us, "x": xs[i]} for i, r in enumerate(res)]

    def replay_arrays(self, arrivals_s, requests: np.ndarray) -> np.ndarray:
        """A request stream as a numpy array of REQUEST_DTYPE records (host pointers in the
        a / b / x fields; the caller keeps those buffers alive), submitted at arrivals_s by
        the library's replay thread. Returns a RESULT_DTYPE array (status RL_ERR_BUSY = 37
        for requests refused by backpressure)."""
        reqs = np.ascontiguousarray(requests, dtype=REQUEST_DTYPE)
        arr = np.ascontiguousarray(arrivals_s, dtype=np.float64)
        res = np.zeros(len(reqs), dtype=RESULT_DTYPE)
        _check(lib.rl_server_replay(self._h, len(reqs), arr.ctypes.data_as(C.c_void_p),
                                    reqs.ctypes.data_as(C.c_void_p), res.ctypes.data_as(C.c_void_p)))
        return res

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib.rl_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
