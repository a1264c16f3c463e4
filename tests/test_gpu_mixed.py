"""Mixed-precision single-system solves (FP32 factor + FP64 refinement / GMRES-IR /
FP64 refactor) on A = U diag(sigma) V^T systems with kappa in {1e2, 1e6, 1e10}: every
solution f64-accurate (normwise backward error <= n 2^-53 10) and close to the FP64
oracle's solution within kappa-scaled forward error."""
import numpy as np
import pytest

import oracle as O
from comparators import backward_error

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53


@pytest.mark.parametrize("kappa", [1e2, 1e6, 1e10])
@pytest.mark.parametrize("n,nrhs", [(700, 1), (1024, 3)])
def test_mixed_lu_conditioned(gpu, kappa, n, nrhs):
    from rulinalg_gb300.workloads import conditioned_system
    a, b = conditioned_system(n, kappa, nrhs, seed=int(np.log10(kappa)) + n)
    x, info = gpu.solve_mixed(a, b, "lu")
    lu, perm, st = O.lu_decompose(a)
    assert st == O.OK
    bes = []
    # ||A||_2 = 1, kappa_2 = kappa by construction: each solution's forward error is at
    # most 2 kappa eta (eta its 2-norm backward error), so two solutions differ by at most
    # the sum of the two bounds
    eta = lambda v, c: np.linalg.norm(b[:, c] - a @ v) / (np.linalg.norm(v) + np.linalg.norm(b[:, c]))
    for c in range(nrhs):
        be = backward_error(a, x[:, c], b[:, c])
        bes.append(be)
        assert be <= n * U64 * 10, (c, be, info)
        xo, _ = O.lu_solve(lu, perm, b[:, c])
        fe = np.linalg.norm(x[:, c] - xo) / np.linalg.norm(xo)
        assert fe <= 2 * kappa * (eta(x[:, c], c) + eta(xo, c)), (c, fe, info)
    assert info["berr"] <= n * U64 * 10
    # the reported backward error is the solution's, not a placeholder: it agrees with
    # the host's to within the rounding of the two residual evaluations
    assert 0.0 < info["berr"] and max(bes) <= 10 * info["berr"] + U64 * 1e-3, (bes, info)
    assert info["berr"] <= 10 * max(bes) + U64, (bes, info)
    if kappa == 1e2:
        assert info["path"] == "refinement" and 1 <= info["iters"] <= 4, info
    print(f"n={n} kappa={kappa:.0e} nrhs={nrhs}: {info}")


def test_mixed_cholesky_and_many_rhs(gpu):
    rng = np.random.default_rng(5)
    n = 600
    g = rng.standard_normal((n, n))
    a = g @ g.T + n * np.eye(n)
    b = rng.standard_normal((n, 12))  # more than 4 columns: the GEMM residual path
    x, info = gpu.solve_mixed(a, b, "cholesky")
    for c in range(12):
        assert backward_error(a, x[:, c], b[:, c]) <= n * U64 * 10
    assert info["path"] == "refinement"


def test_mixed_singular_reports_div_by_zero(gpu):
    a = np.ones((600, 600))
    with pytest.raises(gpu.RulinalgError) as e:
        gpu.solve_mixed(a, np.ones(600), "lu")
    assert e.value.kind == "DivByZero"


def test_fp64_dev_path(gpu):
    import torch
    from rulinalg_gb300._lib import SolveInfo
    import ctypes as C
    rng = np.random.default_rng(6)
    n = 900
    a = rng.uniform(-1, 1, (n, n)) + np.eye(n) * 3
    b = rng.standard_normal((n, 2))
    dev = torch.device("cuda:0")
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    tx = torch.zeros_like(tb)
    info = SolveInfo()
    st = gpu.lib.rl_dsolve_fp64_dev(n, 2, 0, ta.data_ptr(), n, tb.data_ptr(), 2, tx.data_ptr(), 2, C.byref(info),
                                    torch.cuda.current_stream().cuda_stream)
    assert st == 0
    x = tx.cpu().numpy()
    for c in range(2):
        assert backward_error(a, x[:, c], b[:, c]) <= n * U64 * 10
    assert info.path == 2 and info.berr <= n * U64 * 10


@pytest.mark.parametrize("m,n", [(600, 300), (2000, 1000)])
def test_lstsq_mixed_matches_fp64(gpu, m, n):
    rng = np.random.default_rng(m)
    a = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    x, info = gpu.lstsq_mixed(a, b)
    want = np.linalg.lstsq(a, b, rcond=None)[0]
    assert np.max(np.abs(x - want)) <= 1e-12 * np.max(np.abs(want)), info
    assert info["path"] == "refinement" and 1 <= info["iters"] <= 6, info
    # the reported quality is the normal-equations residual of x (never a placeholder)
    r = b - a @ x
    ne = np.max(np.abs(a.T @ r)) / (np.max(np.sum(np.abs(a), 1)) * (np.max(np.sum(np.abs(a), 1)) * np.max(np.abs(x)) + np.max(np.abs(b))))
    assert 0.0 < info["berr"] <= 1e-14 and ne <= 1e-14, (info, ne)


def test_lstsq_mixed_ill_conditioned_falls_back(gpu):
    rng = np.random.default_rng(9)
    m, n = 800, 400
    u, _ = np.linalg.qr(rng.standard_normal((m, n)))
    v, _ = np.linalg.qr(rng.standard_normal((n, n)))
    a = (u * np.logspace(0, -9, n)) @ v.T  # kappa 1e9: beyond what the FP32 R can precondition
    x_true = rng.standard_normal(n)
    b = a @ x_true  # consistent, so the solution is kappa u (not kappa^2 u) sensitive
    x, info = gpu.lstsq_mixed(a, b)
    assert info["path"] == "fp64", info
    assert np.max(np.abs(x - x_true)) <= 1e-5 * np.max(np.abs(x_true)), info


def test_gmres_ir_taken_and_converges(gpu):
    """GMRES-IR itself: with iterative refinement held to one step
    (RL_TUNE_MIXED_REFINE_STEPS = 1) a kappa = 1e6 system, which refinement would finish
    in several steps, goes on to GMRES-IR (restarted FP64 GMRES with the FP32 factor
    applied in FP64 through inverted diagonal blocks). The path is gmres-ir, GMRES
    converges inside its budget, and the solution is f64-accurate and within the
    kappa-scaled forward-error bound of the FP64 oracle's solution."""
    from rulinalg_gb300 import _lib as L
    from rulinalg_gb300.workloads import conditioned_system
    n, kappa = 2048, 1e6
    a, b = conditioned_system(n, kappa, 1, seed=2048 + 6)
    b = b[:, 0]
    gpu.tune_set(L.TUNE_MIXED_REFINE_STEPS, 1)
    try:
        x, info = gpu.solve_mixed(a, b, "lu")
    finally:
        gpu.tune_set(L.TUNE_MIXED_REFINE_STEPS, 30)
    assert info["path"] == "gmres-ir" and info["gmres_iters"] > 0, info
    assert backward_error(a, x, b) <= n * U64 * 10
    lu, perm, st = O.lu_decompose(a, threads=8)
    xo, _ = O.lu_solve(lu, perm, b)
    eta = lambda v: np.linalg.norm(b - a @ v) / (np.linalg.norm(v) + np.linalg.norm(b))
    fe = np.linalg.norm(x - xo) / np.linalg.norm(xo)
    assert fe <= 2 * kappa * (eta(x) + eta(xo)), (fe, info)
    print(f"GMRES-IR n={n} kappa={kappa:.0e}: {info}, forward error vs oracle {fe:.2e}")


@pytest.mark.parametrize("kind", ["lu", "cholesky"])
@pytest.mark.parametrize("kappa", [1e2, 1e6])
def test_mixed_sweeps_with_inverted_diagonal_blocks(gpu, kind, kappa):
    """RL_TUNE_MIXED_SWEEP_INV = 1: the refinement's triangular sweeps apply each 64 x 64
    diagonal block as its FP32 inverse. The solution is as accurate as with substitution
    (f64 backward error, forward error within the oracle bound); at kappa = 1e2 it takes
    the same path in at most two more refinement steps."""
    from rulinalg_gb300 import _lib as L
    from rulinalg_gb300.workloads import conditioned_system
    n = 1500
    a, b = conditioned_system(n, kappa, 2, seed=77 + int(np.log10(kappa)))
    if kind == "cholesky":
        a = a @ a.T  # SPD with kappa^2
    saved = gpu.tune_get(L.TUNE_MIXED_SWEEP_INV)
    try:
        gpu.tune_set(L.TUNE_MIXED_SWEEP_INV, 0)
        x0, i0 = gpu.solve_mixed(a, b, kind)
        gpu.tune_set(L.TUNE_MIXED_SWEEP_INV, 1)
        x1, i1 = gpu.solve_mixed(a, b, kind)
    finally:
        gpu.tune_set(L.TUNE_MIXED_SWEEP_INV, saved)
    if kind == "lu":
        f, perm, st = O.lu_decompose(a, threads=8)
    else:
        f, st = O.chol_decompose(a)
        perm = None
    assert st == O.OK
    xo, _ = O.solve_columns(f, perm, b, threads=8)
    k = kappa if kind == "lu" else kappa ** 2
    eta = lambda v, c: np.linalg.norm(b[:, c] - a @ v) / (np.linalg.norm(a, 2) * np.linalg.norm(v) + np.linalg.norm(b[:, c]))
    for c in range(2):
        assert backward_error(a, x1[:, c], b[:, c]) <= n * U64 * 10, (c, i1)
        fe = np.linalg.norm(x1[:, c] - xo[:, c]) / np.linalg.norm(xo[:, c])
        assert fe <= 2 * k * (eta(x1[:, c], c) + eta(xo[:, c], c)), (c, fe, i1)
    if kappa == 1e2:
        assert i0["path"] == i1["path"] == "refinement" and i1["iters"] <= i0["iters"] + 2, (i0, i1)
    print(f"{kind} kappa={kappa:.0e}: substitution {i0}, inverted blocks {i1}")
