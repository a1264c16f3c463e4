"""FullPivLu (complete pivoting, src/matrix/decomposition/lu.rs:303-599) on the GPU
against the reference's own known answers and, bit for bit, against the oracle's
restatement of the same algorithm: the GPU elimination uses the reference's operations
(multiplier by division, a - m * u without FMA), so factors and both permutations agree
exactly on every input, ties and rank deficiency included."""
import numpy as np
import pytest

import oracle as O
from comparators import assert_matrix_float_eq, assert_ulp_eq, backward_error

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53


def A(x, dtype=np.float64):
    return np.array(x, dtype=dtype).reshape(len(x), -1)


def reconstruct(lupq):
    """p.inverse() * L * U * q.inverse() (lu.rs:903-907) in numpy: (L U)[p][:, q]."""
    lu = lupq.l @ lupq.u
    return lu[lupq.p.perm.astype(np.int64)][:, lupq.q.perm.astype(np.int64)]


def test_full_lu_golden(gpu, golden):
    for name in ("full_lu_reconstruct_4x4", "full_lu_singular_rank3"):
        c = golden[name]
        lu = gpu.FullPivLu.decompose(A(c["a"]))
        if "rank" in c:
            assert lu.rank() == c["rank"]
        assert_matrix_float_eq(reconstruct(lu.unpack()), A(c["a"]))
    c = golden["full_lu_doc_rank2"]
    lu = gpu.FullPivLu.decompose(A(c["a"]))
    assert lu.rank() == 2 and not lu.is_invertible()
    c = golden["full_lu_solve_4x4"]
    x = gpu.FullPivLu.decompose(A(c["a"])).solve(np.array(c["b"]))
    assert_ulp_eq(x, np.array(c["x"]), c["ulp_tol"])
    c = golden["full_lu_inverse_4x4"]
    assert_matrix_float_eq(gpu.FullPivLu.decompose(A(c["a"])).inverse(), A(c["inv"]))
    c = golden["full_lu_noninvertible_3x3"]
    with pytest.raises(gpu.RulinalgError) as e:
        gpu.FullPivLu.decompose(A(c["a"])).inverse()
    assert e.value.kind == "DivByZero"
    # the empty matrix (lu.rs:992-1018) and the identity of the solve doc (lu.rs:459-466)
    lu = gpu.FullPivLu.decompose(np.zeros((0, 0)))
    assert lu.is_invertible() and lu.rank() == 0 and lu.det() == 1.0 and lu.inverse().shape == (0, 0)
    y = gpu.FullPivLu.decompose(np.eye(4)).solve(np.array([3.0, 4.0, 2.0, 1.0]))
    assert np.array_equal(y, [3.0, 4.0, 2.0, 1.0])
    with pytest.raises(gpu.RulinalgPanic):
        gpu.FullPivLu.decompose(np.zeros((4, 3)))


def _inputs(rng, n, dtype):
    yield "uniform", rng.uniform(-1, 1, (n, n)).astype(dtype)
    yield "ties", rng.integers(-3, 4, (n, n)).astype(dtype)  # many equal |a|: the tie rule decides
    r = max(1, n // 3)
    yield "rank_deficient", (rng.standard_normal((n, r)) @ rng.standard_normal((r, n))).astype(dtype)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [1, 2, 5, 33, 64, 130, 257, 500])
def test_full_lu_bit_identical_to_oracle(gpu, dtype, n):
    rng = np.random.default_rng(n + (0 if dtype == np.float64 else 1000))
    for name, a in _inputs(rng, n, dtype):
        lu = gpu.FullPivLu.decompose(a)
        olu, op, oq, _, _ = O.full_lu_decompose(a)
        assert np.array_equal(lu.p.perm, op), name
        assert np.array_equal(lu.q.perm, oq), name
        assert np.array_equal(lu.lu.view(np.uint8), olu.view(np.uint8)), (name, np.nanmax(np.abs(lu.lu - olu)))
        assert lu.rank() == O.full_lu_rank(olu)


def corrected_solve(olu, op, oq, b):
    """The oracle's FullPivLu::solve with the column permutation applied by gather
    (x[i] = y[q[i]]): the reference's scatter (`&self.q * x`, lu.rs:485) is right only
    when q is its own inverse. The oracle's solve with the identity q gives y."""
    y, st = O.full_lu_solve(olu, op, np.arange(len(oq), dtype=np.uint64), b)
    return y[oq.astype(np.int64)], st


@pytest.mark.parametrize("n", [300, 1024])
def test_full_lu_solve_and_det_against_oracle(gpu, n):
    rng = np.random.default_rng(n)
    a = rng.uniform(-1, 1, (n, n)) + np.eye(n)
    b = rng.standard_normal((n, 3))
    lu = gpu.FullPivLu.decompose(a)
    x = lu.solve(b)
    olu, op, oq, _, _ = O.full_lu_decompose(a)
    for c in range(3):
        xo, st = corrected_solve(olu, op, oq, b[:, c])
        assert st == O.OK
        assert backward_error(a, x[:, c], b[:, c]) <= n * U64 * 10
        assert np.max(np.abs(x[:, c] - xo)) <= 1e-10 * np.max(np.abs(xo))
    # det (lu.rs:512-524): p_det * fold(diag U) * q_det on the oracle's (bit-identical)
    # factors; at n = 1024 the product overflows to inf there as in the reference
    u_det = np.float64(1.0)
    for i in range(n):
        u_det = u_det * olu[i, i]
    par = lambda perm: -1.0 if O.perm_parity_odd(perm) else 1.0
    with np.errstate(over="ignore"):
        want = par(op) * u_det * par(oq)
        assert lu.det() == want
    sign, logdet = np.linalg.slogdet(a)
    if np.isfinite(want):
        assert np.sign(want) == sign and abs(np.log(abs(want)) - logdet) <= 1e-9 * max(1.0, abs(logdet))


def test_full_lu_singular_solve_div_by_zero(gpu):
    a = np.ones((70, 70))
    lu = gpu.FullPivLu.decompose(a)
    assert lu.rank() == 1 and not lu.is_invertible()
    with pytest.raises(gpu.RulinalgError) as e:
        lu.solve(np.ones(70))
    assert e.value.kind == "DivByZero"
