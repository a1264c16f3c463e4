"""Autotuner of the batched solver (rl_batch_plan_*).

For a given batch (sizes, kinds, precision) it picks, by timing candidate plans on the
device, the launch shape and the size classes of the one persistent launch:

  * CTAs per SM of the solver kernel (RL_TUNE_BATCH_CTAS_PER_SM; more CTAs hide more of
    each system's latency chain, fewer leave each CTA more L1 and issue slots);
  * the cost threshold of the one-warp class (RL_TUNE_BATCH_WARP_COST: systems of cost
    n^3, x2 for LU, up to it are solved by one warp each once the largest-first queue
    reaches them; the rest by a whole CTA);
  * for the host-pointer path, the number of upload chunks overlapped with the solve
    (RL_TUNE_UPLOAD_CHUNKS).

The search is coordinate descent from the library defaults: one knob at a time, each
candidate timed over `reps` graph launches after a warm-up (CUDA events), the best kept
only if it beats the incumbent by more than 1% (so the tuned plan is never slower than
the defaults by more than the timing noise). The choice is cached in a JSON file keyed
by the GPU, the precision and the batch's size histogram (counts per octave of n and
kind), so a later batch of the same shape reuses it without timing. Device buffers are
torch CUDA tensors (the library itself keeps no timing API).
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import numpy as np

from . import _lib as L
from ._lib import lib
from .batch import BatchPlan, PREC_FP32

KNOBS = {
    "ctas_per_sm": L.TUNE_BATCH_CTAS_PER_SM,
    "warp_cost": L.TUNE_BATCH_WARP_COST,
    "upload_chunks": L.TUNE_UPLOAD_CHUNKS,
}
CANDIDATES = {
    "ctas_per_sm": [0, 1, 2],  # 0: as many as fit (the kernel's occupancy: 3 FP32, 2 FP64)
    "warp_cost": [32768, 24 ** 3, 16 ** 3, 0],
    "upload_chunks": [32, 8, 16, 64],
}


def default_cache_path() -> Path:
    return Path(os.environ.get("RULINALG_GB300_TUNE_CACHE",
                               Path.home() / ".cache" / "rulinalg_gb300" / "autotune.json"))


def batch_key(n, kind, precision: int, device_name: str) -> str:
    """GPU, precision and the size histogram: counts per octave of n ([2^k, 2^(k+1))) and kind."""
    n = np.asarray(n, dtype=np.int64)
    kind = np.asarray(kind, dtype=np.int64)
    octave = np.floor(np.log2(np.maximum(n, 1))).astype(np.int64)
    hist = {f"{k}:{o}": int(np.sum((kind == k) & (octave == o))) for k in (0, 1) for o in range(0, 11)}
    hist = {key: v for key, v in hist.items() if v}
    blob = json.dumps({"gpu": device_name, "precision": precision, "hist": hist}, sort_keys=True)
    return hashlib.sha256(blob.encode()).hexdigest()[:24]


def _get():
    return {name: int(_tune_get(key)) for name, key in KNOBS.items()}


def _tune_get(key):
    import ctypes as C
    v = C.c_int64(0)
    if lib.rl_tune_get(key, C.byref(v)) != 0:
        raise ValueError(key)
    return v.value


def _set(choice: dict) -> None:
    for name, value in choice.items():
        st = lib.rl_tune_set(KNOBS[name], int(value))
        if st != 0:
            raise ValueError(f"rl_tune_set({name}, {value}) = {st}")


def apply(choice: dict) -> None:
    """Sets the tunables of a stored choice for the plans created after this call."""
    _set({k: v for k, v in choice.items() if k in KNOBS})


def _time_plan(n, kind, precision, a, b, reps: int, host: bool) -> float:
    """Mean ms per solve of a plan created under the current tunables."""
    import time

    import torch
    plan = BatchPlan(n, kind, precision)
    try:
        count = len(plan.n)
        if host:
            import ctypes as C
            dt = np.float32 if precision == PREC_FP32 else np.float64
            ah, bh = a.cpu().numpy().astype(dt), b.cpu().numpy().astype(dt)
            x = np.zeros_like(bh)
            info = np.zeros(count, dtype=np.int32)
            fp = C.POINTER(C.c_float if dt == np.float32 else C.c_double)
            fn = lib.rl_sbatch_solve if precision == PREC_FP32 else lib.rl_dbatch_solve
            args = (plan._h, ah.ctypes.data_as(fp), bh.ctypes.data_as(fp), x.ctypes.data_as(fp),
                    info.ctypes.data_as(C.POINTER(C.c_int32)), None, None)
            fn(*args)
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                if fn(*args) != 0:
                    raise RuntimeError("batched solve failed while tuning")
                ts.append(time.perf_counter() - t0)
            return 1e3 * float(np.mean(ts))
        x = torch.zeros_like(b)
        info = torch.zeros(count, dtype=torch.int32, device=b.device)
        stream = torch.cuda.current_stream()
        call = lambda: plan.solve_dev(a.data_ptr(), b.data_ptr(), x.data_ptr(), info.data_ptr(), 0, 0,
                                      stream.cuda_stream)
        call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        e1.synchronize()
        if not bool((info == 0).all()):
            raise RuntimeError("batched solve failed while tuning")
        return e0.elapsed_time(e1) / reps
    finally:
        plan.close()


def tune(n, kind, precision: int, a, b, reps: int = 3, host: bool = False, cache: Path | None = None,
         device_name: str | None = None) -> dict:
    """Tunes the batched plan for this batch (a, b: the packed device buffers, torch CUDA
    tensors) and leaves the chosen tunables set. host = True also tunes the upload chunks
    of the host-pointer path (timed through rl_dbatch_solve with host copies of a, b).
    Returns {"choice", "ms", "default_ms", "trials", "cached", "key"}."""
    import torch
    name = device_name or torch.cuda.get_device_name()
    key = batch_key(n, kind, precision, name) + (":host" if host else "")
    path = Path(cache) if cache else default_cache_path()
    store = json.loads(path.read_text()) if path.exists() else {}
    if key in store:
        apply(store[key]["choice"])
        return {**store[key], "cached": True, "key": key}
    saved = _get()
    knobs = ["ctas_per_sm", "warp_cost"] + (["upload_chunks"] if host else [])
    best = {k: CANDIDATES[k][0] for k in knobs}
    _set(best)
    best_ms = default_ms = _time_plan(n, kind, precision, a, b, reps, host)
    trials = [{"choice": dict(best), "ms": best_ms}]
    try:
        for k in knobs:
            for v in CANDIDATES[k][1:]:
                cand = dict(best, **{k: v})
                _set(cand)
                ms = _time_plan(n, kind, precision, a, b, reps, host)
                trials.append({"choice": cand, "ms": ms})
                if ms < 0.99 * best_ms:
                    best, best_ms = cand, ms
    except Exception:
        _set(saved)
        raise
    _set(best)
    out = {"choice": best, "ms": best_ms, "default_ms": default_ms, "trials": trials}
    store[key] = out
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text(json.dumps(store, indent=1, sort_keys=True))
    except OSError:
        pass  # a read-only cache location only costs the next run its tuning time
    return {**out, "cached": False, "key": key}
