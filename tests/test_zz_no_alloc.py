"""The allocation-free entry point, checked against the existing batched entry point.

rl_dsolve_mixed_noalloc_dev exists for callers that cannot allocate device memory (a
serving process that reserved all GPU memory at start-up, or a framework whose own pool
owns the device memory): it takes all scratch from one fixed array inside the library.
Here it is called through the C ABI twice in a row (the second call must not be
disturbed by what the first left in the shared array) and each result is compared with
a one-system RL_PREC_MIXED batch solved through rl_dbatch_solve_dev. This file is
collected last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53


def _system(rng, n, kind):
    if kind:
        g = rng.standard_normal((n, n))
        return g @ g.T + n * np.eye(n), rng.standard_normal(n)
    return rng.uniform(-1, 1, (n, n)) + n * np.eye(n), rng.standard_normal(n)


def _noalloc(gpu, torch, a, b, kind):
    dev = torch.device("cuda:0")
    ta = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    tb = torch.from_numpy(b).to(dev)
    tx = torch.full_like(tb, np.nan)
    info = torch.full((1,), -7, dtype=torch.int32, device=dev)
    iters = torch.zeros(1, dtype=torch.int32, device=dev)
    berr = torch.zeros(1, dtype=torch.float64, device=dev)
    st = gpu.lib.rl_dsolve_mixed_noalloc_dev(a.shape[0], kind, ta.data_ptr(), tb.data_ptr(), tx.data_ptr(),
                                             info.data_ptr(), iters.data_ptr(), berr.data_ptr(),
                                             torch.cuda.current_stream().cuda_stream)
    assert st == 0, gpu.lib.rl_status_string(st)
    torch.cuda.synchronize()
    return tx.cpu().numpy(), int(info.item()), int(iters.item()), float(berr.item())


def _batched(gpu, a, b, kind):
    plan = gpu.BatchPlan([a.shape[0]], [kind], gpu.PREC_MIXED)
    pa, pb = plan.pack([a], [b])
    x, info, iters, berr = plan.solve(pa, pb)
    plan.close()
    return x, int(info[0]), int(iters[0]), float(berr[0])


def test_noalloc_matches_batched_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    # two calls in a row with different sizes and kinds: the larger first, so that the
    # second call runs on scratch that still holds the first call's factor
    for n, kind in ((300, 0), (97, 1)):
        a, b = _system(rng, n, kind)
        x, info, iters, berr = _noalloc(gpu, torch, a, b, kind)
        xr, info_r, iters_r, berr_r = _batched(gpu, a, b, kind)
        assert info == 0 and info_r == 0
        assert iters == iters_r
        assert np.max(np.abs(x - xr)) <= 1e-12 * n * np.max(np.abs(xr))
        assert berr <= n * U64 * 10


def _noalloc_no_outputs(gpu, torch, a, b, kind):
    """The same call with NULL iters and berr (both optional)."""
    dev = torch.device("cuda:0")
    ta = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    tb = torch.from_numpy(b).to(dev)
    tx = torch.full_like(tb, np.nan)
    info = torch.full((1,), -7, dtype=torch.int32, device=dev)
    st = gpu.lib.rl_dsolve_mixed_noalloc_dev(a.shape[0], kind, ta.data_ptr(), tb.data_ptr(), tx.data_ptr(),
                                             info.data_ptr(), None, None, torch.cuda.current_stream().cuda_stream)
    assert st == 0, gpu.lib.rl_status_string(st)
    torch.cuda.synchronize()
    return tx.cpu().numpy(), int(info.item())


def test_noalloc_fallback_then_warp_path(gpu):
    """The launches only this entry point wires to the fixed array: an ill-conditioned
    LU system (kappa = 1e10, n = 100) whose FP32 refinement cannot converge goes to the
    FP64 fallback launch (iters == -1) and leaves a fallback count of one in the shared
    array; the next calls, a small LU system on the one-warp path (n = 20) and a
    Cholesky system with NULL iters / berr, must not see that stale count. Each result
    is compared with a one-system RL_PREC_MIXED batch."""
    torch = pytest.importorskip("torch")
    from rulinalg_gb300.workloads import conditioned_system
    rng = np.random.default_rng(2025)
    a, b = conditioned_system(100, 1e10, 1, seed=7)
    b = np.ascontiguousarray(b[:, 0])
    x, info, iters, berr = _noalloc(gpu, torch, a, b, 0)
    xr, info_r, iters_r, berr_r = _batched(gpu, a, b, 0)
    assert info == 0 and info_r == 0
    assert iters == -1 and iters_r == -1  # solved by the FP64 fallback launch
    assert np.array_equal(x, xr)
    assert berr <= 100 * U64 * 10
    a, b = _system(rng, 20, 0)
    x, info, iters, berr = _noalloc(gpu, torch, a, b, 0)
    xr, info_r, iters_r, _ = _batched(gpu, a, b, 0)
    assert info == 0 and iters == iters_r >= 0
    assert np.max(np.abs(x - xr)) <= 1e-12 * 20 * np.max(np.abs(xr))
    a, b = _system(rng, 40, 1)
    x, info = _noalloc_no_outputs(gpu, torch, a, b, 1)
    xr, info_r, _, _ = _batched(gpu, a, b, 1)
    assert info == 0 and info_r == 0
    assert np.max(np.abs(x - xr)) <= 1e-12 * 40 * np.max(np.abs(xr))


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu):
    z = C.c_void_p(0)
    assert gpu.lib.rl_dsolve_mixed_noalloc_dev(513, 0, z, z, z, z, z, z, z) == 1  # RL_ERR_INVALID_ARG
