"""rulinalg_gb300: rulinalg's dense hot path (GEMM, PartialPivLu, Cholesky,
HouseholderQr with solve/det/inverse) as hand-written sm_103a CUDA behind a C ABI
(include/rulinalg_gb300.h). Importing loads librulinalg_gb300.so; there is no CPU path."""
from ._lib import lib, LIB_PATH  # noqa: F401  (raises ImportError when the library is not built)
from .api import (  # noqa: F401
    Cholesky, DeviceError, FullPivLu, HouseholderComposition, HouseholderQr, LUP, LUPQ, PartialPivLu, PermutationMatrix, QR,
    ResidentFactor, RulinalgError, RulinalgPanic, ThinQR, det, inverse, least_squares, lstsq_mixed, mat_mul, solve,
    solve_l_triangular, solve_mixed, solve_u_triangular,
)
from .batch import BatchPlan, KIND_CHOLESKY, KIND_LU, PREC_FP32, PREC_FP64, PREC_MIXED  # noqa: F401
from .server import REQ_CHOLESKY, REQ_LSTSQ, REQ_LU, REQ_RESOLVE, Server  # noqa: F401


def device_available() -> bool:
    return lib.rl_device_check() == 0


def launch_count() -> int:
    return int(lib.rl_launch_count())


def tune_set(key: int, value: int) -> None:
    """Sets a process-wide tunable (rl_tune_set; keys TUNE_* in rulinalg_gb300._lib)."""
    st = lib.rl_tune_set(key, value)
    if st != 0:
        raise ValueError(f"rl_tune_set({key}, {value}): {lib.rl_status_string(st).decode()}")


def tune_get(key: int) -> int:
    import ctypes as C
    v = C.c_int64(0)
    st = lib.rl_tune_get(key, C.byref(v))
    if st != 0:
        raise ValueError(f"rl_tune_get({key}): {lib.rl_status_string(st).decode()}")
    return int(v.value)
