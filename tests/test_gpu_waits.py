"""Bounded device waits run out cleanly: the kernel returns RL_ERR_TIMEOUT through the
host, the context stays usable and the next call on the same objects succeeds.

No GPU is faulted, trapped or hung: each test shortens the wait limit
(RL_TUNE_WAIT_TIMEOUT_NS, 50 ms) and makes one flag that nothing sets
(RL_TUNE_TEST_WITHHOLD_*), so the waits for it expire by their own wall-time bound.
"""
import ctypes as C

import numpy as np
import pytest

from comparators import backward_error

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53
RL_ERR_TIMEOUT = 35


@pytest.fixture
def tunables(gpu):
    from rulinalg_gb300 import _lib as L
    saved = {k: gpu.tune_get(k) for k in (L.TUNE_WAIT_TIMEOUT_NS, L.TUNE_UPLOAD_CHUNKS, L.TUNE_TEST_WITHHOLD_CHUNK,
                                          L.TUNE_TEST_WITHHOLD_SWEEP_BLOCK)}
    yield L
    for k, v in saved.items():
        gpu.tune_set(k, v)


def _batch(rng, count):
    sizes = rng.integers(8, 200, count).astype(np.int32)
    kinds = rng.integers(0, 2, count).astype(np.uint8)
    mats, rhs = [], []
    for n, k in zip(sizes, kinds):
        if k:
            g = rng.standard_normal((n, n))
            mats.append(g @ g.T + n * np.eye(n))
        else:
            mats.append(rng.uniform(-1, 1, (n, n)) + n * np.eye(n))
        rhs.append(rng.standard_normal(n))
    return sizes, kinds, mats, rhs


def test_gated_upload_wait_runs_out_then_recovers(gpu, tunables):
    """The host-pointer batched path: chunk 3's arrival flag is withheld, the CTAs that
    reach its systems wait 50 ms and stop, rl_dbatch_solve returns RL_ERR_TIMEOUT; with
    the flag restored the same plan solves the batch."""
    L = tunables
    rng = np.random.default_rng(31)
    sizes, kinds, mats, rhs = _batch(rng, 400)
    gpu.tune_set(L.TUNE_UPLOAD_CHUNKS, 8)
    plan = gpu.BatchPlan(sizes, kinds, gpu.PREC_MIXED)
    a, b = plan.pack(mats, rhs)
    x = np.zeros(plan.b_total)
    info = np.zeros(len(sizes), dtype=np.int32)
    f64p, i32p = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    args = (plan._h, a.ctypes.data_as(f64p), b.ctypes.data_as(f64p), x.ctypes.data_as(f64p),
            info.ctypes.data_as(i32p), None, None)
    gpu.tune_set(L.TUNE_WAIT_TIMEOUT_NS, 50_000_000)
    gpu.tune_set(L.TUNE_TEST_WITHHOLD_CHUNK, 3)
    assert gpu.lib.rl_dbatch_solve(*args) == RL_ERR_TIMEOUT
    gpu.tune_set(L.TUNE_TEST_WITHHOLD_CHUNK, -1)
    gpu.tune_set(L.TUNE_WAIT_TIMEOUT_NS, 1_000_000_000)
    assert gpu.lib.rl_dbatch_solve(*args) == 0
    assert (info == 0).all()
    for i, (m, r) in enumerate(zip(mats, rhs)):
        xi = plan.unpack(x)[i]
        assert backward_error(m, xi, r) <= sizes[i] * U64 * 10
    plan.close()


def test_triangular_sweep_wait_runs_out_then_recovers(gpu, tunables):
    """The one-launch few-right-hand-side triangular sweep (n > 512): block 5 is solved
    but never published, the blocks after it wait 50 ms, publish anyway and the solve
    returns RL_ERR_TIMEOUT; the next solve with the same factor is correct."""
    L = tunables
    rng = np.random.default_rng(32)
    n = 1024
    a = rng.uniform(-1, 1, (n, n)) + np.eye(n)
    bvec = rng.uniform(-1, 1, n)
    lu = gpu.PartialPivLu.decompose(a)
    gpu.tune_set(L.TUNE_WAIT_TIMEOUT_NS, 50_000_000)
    gpu.tune_set(L.TUNE_TEST_WITHHOLD_SWEEP_BLOCK, 5)
    with pytest.raises(gpu.DeviceError) as e:
        lu.solve(bvec)
    assert e.value.status == RL_ERR_TIMEOUT
    gpu.tune_set(L.TUNE_TEST_WITHHOLD_SWEEP_BLOCK, -1)
    gpu.tune_set(L.TUNE_WAIT_TIMEOUT_NS, 1_000_000_000)
    x = lu.solve(bvec)
    assert backward_error(a, x, bvec) <= n * U64 * 10
