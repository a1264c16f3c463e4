"""HouseholderComposition application (Q X, Q^T X) without forming Q, the triangular
solves (solve_u_triangular / solve_l_triangular) and device-resident factors, through
the C ABI, against the oracle and the reference's own known answers."""
import numpy as np
import pytest

import oracle as O
from comparators import assert_matrix_float_eq, backward_error

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53
U32 = 2.0 ** -24


def A(x, dtype=np.float64):
    return np.array(x, dtype=dtype).reshape(len(x), -1)


def fro(x):
    return float(np.sqrt(np.sum(np.asarray(x, dtype=np.float64) ** 2)))


def test_left_multiply_into_golden(gpu, golden):
    """householder.rs:382-430: the reference's left_multiply_into known answers (1e-15)."""
    c = golden["householder_composition"]
    h = gpu.HouseholderQr(A(c["storage"]), np.array(c["tau"]))
    for x, e in (("x_square", "e_square"), ("x_tall", "e_tall"), ("x_short", "e_short")):
        got = np.ascontiguousarray(A(c[x]))
        h.q().left_multiply_into(got)
        assert_matrix_float_eq(got, A(c[e]), eps=c["eps"])


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,q", [(5, 3, 2), (64, 64, 7), (200, 100, 1), (300, 600, 5), (1100, 520, 64),
                                   (4096, 300, 3)])
def test_q_and_qt_apply_against_oracle(gpu, dtype, m, n, q):
    """Q X against the oracle's left_multiply_into restatement and Q^T X against its
    forward-order counterpart, on a GPU factor (so both sides use the same reflectors):
    normwise within 10 max(m, n) eps ||X||."""
    rng = np.random.default_rng(m + 3 * n + q)
    a = rng.standard_normal((m, n)).astype(dtype)
    h = gpu.HouseholderQr.decompose(a)
    x = rng.standard_normal((m, q)).astype(dtype)
    eps = U64 if dtype == np.float64 else U32
    qr64, tau64 = h.qr.astype(np.float64), h.tau.astype(np.float64)
    for trans in (False, True):
        got = x.copy()
        if trans:
            h.q().left_multiply_into_transposed(got)
            want = O.qr_qt_left_multiply(qr64, tau64, x.astype(np.float64))
        else:
            h.q().left_multiply_into(got)
            want = O.qr_q_left_multiply(qr64, tau64, x.astype(np.float64))
        assert fro(got.astype(np.float64) - want) <= 10 * max(m, n) * eps * fro(x), trans
    # Q^T Q X = X
    y = x.copy()
    h.q().left_multiply_into(y)
    h.q().left_multiply_into_transposed(y)
    assert fro(y.astype(np.float64) - x) <= 20 * max(m, n) * eps * fro(x)


def test_q_apply_shape_panics(gpu):
    h = gpu.HouseholderQr.decompose(np.eye(4))
    with pytest.raises(gpu.RulinalgPanic):
        h.q().left_multiply_into(np.zeros((3, 2)))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n,nrhs", [(1, 1), (37, 1), (300, 3), (1000, 1), (1000, 12), (2500, 5), (700, 64),
                                    (1100, 100), (600, 129)])
def test_triangular_solves_against_oracle(gpu, dtype, n, nrhs):
    """solve_u_triangular / solve_l_triangular against the oracle's back_substitution /
    forward_substitution (src/matrix/mod.rs:318-398), column by column: backward error
    within 10 n eps and the other triangle ignored (filled with NaN). Up to 128
    right-hand sides take the one-launch sweep in groups of 8 columns (100: a partial
    last group), 129 the blocked path."""
    rng = np.random.default_rng(n + nrhs)
    t = rng.uniform(-1, 1, (n, n)) / np.sqrt(n) + np.diag(rng.uniform(1, 2, n))
    eps = U64 if dtype == np.float64 else U32
    for upper in (True, False):
        tri = (np.triu(t) if upper else np.tril(t)).astype(dtype)
        given = tri.copy()
        given[np.tril_indices(n, -1) if upper else np.triu_indices(n, 1)] = np.nan
        b = rng.standard_normal((n, nrhs)).astype(dtype)
        x = (gpu.solve_u_triangular if upper else gpu.solve_l_triangular)(given, b)
        for c in range(nrhs):
            xo, st = (O.back_substitution if upper else O.forward_substitution)(tri.astype(np.float64),
                                                                               b[:, c].astype(np.float64))
            assert st == O.OK
            assert backward_error(tri.astype(np.float64), x[:, c].astype(np.float64), b[:, c]) <= 10 * n * eps
            assert np.max(np.abs(x[:, c] - xo)) <= 100 * n * eps * np.max(np.abs(xo))


def test_triangular_div_by_zero(gpu):
    """|u_ii| < epsilon is the reference's Err(DivByZero) (src/matrix/mod.rs:333-336)."""
    u = np.triu(np.ones((70, 70)))
    u[40, 40] = 1e-17
    with pytest.raises(gpu.RulinalgError) as e:
        gpu.solve_u_triangular(u, np.ones(70))
    assert e.value.kind == "DivByZero"


@pytest.mark.parametrize("kind,n", [("lu", 300), ("lu", 1500), ("cholesky", 800)])
def test_resident_factor_repeated_solves(gpu, kind, n):
    """rl_factor_create once, rl_factor_solve with several right-hand-side sets: every
    column f64-accurate and equal to the oracle's decompose + solve within the forward
    error that the two backward errors allow (well-conditioned systems, kappa < 10)."""
    import torch
    rng = np.random.default_rng(n)
    if kind == "lu":
        a = rng.uniform(-1, 1, (n, n)) + n * np.eye(n) / 2
        f, perm, st = O.lu_decompose(a, threads=8)
    else:
        g = rng.standard_normal((n, n))
        a = g @ g.T / n + np.eye(n)
        f, st = O.chol_decompose(a)
        perm = None
    assert st == O.OK
    dev = torch.device("cuda:0")
    rf = gpu.ResidentFactor(torch.from_numpy(a).to(dev), kind)
    try:
        for nrhs in (1, 3, 16):
            b = rng.standard_normal((n, nrhs))
            tb = torch.from_numpy(b).to(dev)
            tx = torch.zeros_like(tb)
            info = rf.solve(tb, tx)
            x = tx.cpu().numpy()
            xo, _ = O.solve_columns(f, perm, b, threads=8)
            for c in range(nrhs):
                assert backward_error(a, x[:, c], b[:, c]) <= n * U64 * 10
                assert np.max(np.abs(x[:, c] - xo[:, c])) <= 1e-11 * np.max(np.abs(xo[:, c]))
            assert info["berr"] <= n * U64 * 10 and info["path"] == "refinement"
    finally:
        rf.close()
