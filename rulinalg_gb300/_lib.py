"""ctypes binding of librulinalg_gb300.so (the C ABI declared in include/rulinalg_gb300.h).

The library is the product: there is no Python or CPU implementation behind these
names. If the shared object has not been built, importing raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("RULINALG_GB300_LIB", _PKG / "librulinalg_gb300.so"))

if not LIB_PATH.exists():
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA library first "
        "(python -c 'import __graft_entry__ as g; g.build()' or python rulinalg_gb300/build.py)")

lib = C.CDLL(str(LIB_PATH))

sz = C.c_size_t
i64 = C.c_int64
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)
i64p = C.POINTER(C.c_int64)
vp = C.c_void_p
st = C.c_int

# name -> (restype, argtypes). Every function the header declares appears here, and
# tests check the two lists against each other.
SIGNATURES = {
    "rl_status_string": (C.c_char_p, [st]),
    "rl_version": (C.c_int, []),
    "rl_device_check": (st, []),
    "rl_launch_count": (C.c_uint64, []),
    "rl_tune_set": (st, [C.c_int, C.c_int64]),
    "rl_tune_get": (st, [C.c_int, i64p]),
    "rl_sgemm": (st, [sz, sz, sz, f32p, sz, f32p, sz, f32p, sz]),
    "rl_dgemm": (st, [sz, sz, sz, f64p, sz, f64p, sz, f64p, sz]),
    "rl_sgemm_dev": (st, [sz, sz, sz, vp, sz, vp, sz, vp, sz, vp]),
    "rl_dgemm_dev": (st, [sz, sz, sz, vp, sz, vp, sz, vp, sz, vp]),
    "rl_slu_decompose": (st, [sz, f32p, sz, u64p]),
    "rl_dlu_decompose": (st, [sz, f64p, sz, u64p]),
    "rl_slu_solve": (st, [sz, sz, f32p, sz, u64p, f32p, sz]),
    "rl_dlu_solve": (st, [sz, sz, f64p, sz, u64p, f64p, sz]),
    "rl_slu_inverse": (st, [sz, f32p, sz, u64p, f32p, sz]),
    "rl_dlu_inverse": (st, [sz, f64p, sz, u64p, f64p, sz]),
    "rl_slu_det": (st, [sz, f32p, sz, u64p, f32p]),
    "rl_dlu_det": (st, [sz, f64p, sz, u64p, f64p]),
    "rl_sfull_lu_decompose": (st, [sz, f32p, sz, u64p, u64p]),
    "rl_dfull_lu_decompose": (st, [sz, f64p, sz, u64p, u64p]),
    "rl_sfull_lu_solve": (st, [sz, sz, f32p, sz, u64p, u64p, f32p, sz]),
    "rl_dfull_lu_solve": (st, [sz, sz, f64p, sz, u64p, u64p, f64p, sz]),
    "rl_scholesky_decompose": (st, [sz, f32p, sz]),
    "rl_dcholesky_decompose": (st, [sz, f64p, sz]),
    "rl_scholesky_solve": (st, [sz, sz, f32p, sz, f32p, sz]),
    "rl_dcholesky_solve": (st, [sz, sz, f64p, sz, f64p, sz]),
    "rl_scholesky_inverse": (st, [sz, f32p, sz, f32p, sz]),
    "rl_dcholesky_inverse": (st, [sz, f64p, sz, f64p, sz]),
    "rl_scholesky_det": (st, [sz, f32p, sz, f32p]),
    "rl_dcholesky_det": (st, [sz, f64p, sz, f64p]),
    "rl_sqr_decompose": (st, [sz, sz, f32p, sz, f32p]),
    "rl_dqr_decompose": (st, [sz, sz, f64p, sz, f64p]),
    "rl_sqr_first_k_columns": (st, [sz, sz, f32p, sz, f32p, sz, f32p, sz]),
    "rl_dqr_first_k_columns": (st, [sz, sz, f64p, sz, f64p, sz, f64p, sz]),
    "rl_sqr_q_apply": (st, [sz, sz, f32p, sz, f32p, sz, f32p, sz]),
    "rl_dqr_q_apply": (st, [sz, sz, f64p, sz, f64p, sz, f64p, sz]),
    "rl_sqr_q_apply_t": (st, [sz, sz, f32p, sz, f32p, sz, f32p, sz]),
    "rl_dqr_q_apply_t": (st, [sz, sz, f64p, sz, f64p, sz, f64p, sz]),
    "rl_strsv_upper": (st, [sz, sz, f32p, sz, f32p, sz]),
    "rl_dtrsv_upper": (st, [sz, sz, f64p, sz, f64p, sz]),
    "rl_strsv_lower": (st, [sz, sz, f32p, sz, f32p, sz]),
    "rl_dtrsv_lower": (st, [sz, sz, f64p, sz, f64p, sz]),
    "rl_factor_create": (st, [C.POINTER(vp), C.c_int, sz, vp, sz, vp]),
    "rl_factor_solve": (st, [vp, sz, vp, sz, vp, sz, vp, vp]),
    "rl_factor_destroy": (st, [vp]),
    "rl_sqr_least_squares": (st, [sz, sz, f32p, sz, f32p, f32p]),
    "rl_dqr_least_squares": (st, [sz, sz, f64p, sz, f64p, f64p]),
    "rl_smatrix_solve": (st, [sz, f32p, sz, f32p]),
    "rl_dmatrix_solve": (st, [sz, f64p, sz, f64p]),
    "rl_smatrix_inverse": (st, [sz, f32p, sz, f32p, sz]),
    "rl_dmatrix_inverse": (st, [sz, f64p, sz, f64p, sz]),
    "rl_smatrix_det": (st, [sz, f32p, sz, f32p]),
    "rl_dmatrix_det": (st, [sz, f64p, sz, f64p]),
    "rl_batch_plan_create": (st, [C.POINTER(vp), sz, i32p, u8p, C.c_int]),
    "rl_batch_plan_destroy": (st, [vp]),
    "rl_batch_plan_layout": (st, [vp, i64p, i64p, i64p, i64p]),
    "rl_dbatch_solve_dev": (st, [vp, vp, vp, vp, vp, vp, vp, vp]),
    "rl_sbatch_solve_dev": (st, [vp, vp, vp, vp, vp, vp, vp, vp]),
    "rl_dbatch_solve": (st, [vp, f64p, f64p, f64p, i32p, i32p, f64p]),
    "rl_sbatch_solve": (st, [vp, f32p, f32p, f32p, i32p, i32p, f64p]),
    "rl_dsolve_mixed_noalloc_dev": (st, [sz, C.c_int, vp, vp, vp, vp, vp, vp, vp]),
    "rl_dsolve_mixed_dev": (st, [sz, sz, C.c_int, vp, sz, vp, sz, vp, sz, vp, vp]),
    "rl_dsolve_mixed": (st, [sz, sz, C.c_int, f64p, sz, f64p, sz, f64p, sz, vp]),
    "rl_dsolve_fp64_dev": (st, [sz, sz, C.c_int, vp, sz, vp, sz, vp, sz, vp, vp]),
    "rl_dlstsq_mixed_dev": (st, [sz, sz, vp, sz, vp, vp, vp, vp]),
    "rl_dlstsq_mixed": (st, [sz, sz, f64p, sz, f64p, f64p, vp]),
    "rl_server_create": (st, [vp, C.POINTER(vp)]),
    "rl_server_submit": (st, [vp, vp, C.POINTER(C.c_uint64)]),
    "rl_server_wait": (st, [vp, C.c_uint64, C.c_double, vp]),
    "rl_server_release_factor": (st, [vp, C.c_uint64]),
    "rl_server_stats_get": (st, [vp, vp]),
    "rl_server_reset_stats": (st, [vp]),
    "rl_server_replay": (st, [vp, sz, vp, vp, vp]),
    "rl_server_destroy": (st, [vp]),
}


class ServerConfig(C.Structure):
    """rl_server_config"""
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("workers", C.c_int), ("max_batch", C.c_int), ("small_n", C.c_int),
                ("max_pending", C.c_int)]


class Request(C.Structure):
    """rl_request"""
    _fields_ = [("kind", C.c_int), ("retain", C.c_int), ("factor", C.c_uint64), ("m", C.c_size_t), ("n", C.c_size_t),
                ("a", C.c_void_p), ("b", C.c_void_p), ("x", C.c_void_p)]


class Result(C.Structure):
    """rl_result"""
    _fields_ = [("status", C.c_int), ("iters", C.c_int32), ("path", C.c_int32), ("reserved", C.c_int32),
                ("berr", C.c_double), ("factor", C.c_uint64), ("queue_us", C.c_double), ("latency_us", C.c_double)]


class ServerStats(C.Structure):
    """rl_server_stats"""
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64), ("batches", C.c_uint64),
                ("batched_requests", C.c_uint64), ("bytes_in_use", C.c_uint64), ("bytes_peak", C.c_uint64),
                ("bytes_budget", C.c_uint64), ("resident_factors", C.c_uint64), ("p50_us", C.c_double),
                ("p99_us", C.c_double), ("mean_us", C.c_double), ("solves_per_s", C.c_double),
                ("rejected", C.c_uint64)]


# numpy layouts of rl_request and rl_result, for request streams built without a Python
# loop (Server.replay_arrays)
import numpy as _np  # noqa: E402
REQUEST_DTYPE = _np.dtype([("kind", "<i4"), ("retain", "<i4"), ("factor", "<u8"), ("m", "<u8"), ("n", "<u8"),
                           ("a", "<u8"), ("b", "<u8"), ("x", "<u8")])
RESULT_DTYPE = _np.dtype([("status", "<i4"), ("iters", "<i4"), ("path", "<i4"), ("reserved", "<i4"),
                          ("berr", "<f8"), ("factor", "<u8"), ("queue_us", "<f8"), ("latency_us", "<f8")])
assert REQUEST_DTYPE.itemsize == C.sizeof(Request) and RESULT_DTYPE.itemsize == C.sizeof(Result)


class SolveInfo(C.Structure):
    """rl_solve_info"""
    _fields_ = [("iters", C.c_int32), ("gmres_iters", C.c_int32), ("path", C.c_int32), ("reserved", C.c_int32),
                ("berr", C.c_double)]

# RL_TUNE_* keys (rulinalg_gb300.h)
TUNE_WAIT_TIMEOUT_NS = 1
TUNE_PANEL_CLUSTER_MAX = 2
TUNE_BATCH_CTAS_PER_SM = 3
TUNE_BATCH_WARP_COST = 4
TUNE_UPLOAD_CHUNKS = 5
TUNE_MIXED_REFINE_STEPS = 6
TUNE_LU_OUTER_NB = 7
TUNE_MIXED_SWEEP_INV = 8
TUNE_PANEL_LOOKAHEAD = 9
TUNE_FULLPIV_CTAS_PER_SM = 10
TUNE_TEST_WITHHOLD_CHUNK = 100
TUNE_TEST_WITHHOLD_SWEEP_BLOCK = 101

for _name, (_res, _args) in SIGNATURES.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args
