"""The oracle pinned against the reference's own known-answer tests (CPU only).

Every case comes from tests/golden/reference_cases.json, which make_golden.py extracted
from the reference's test sources; the comparators are the reference's (comparators.py).
"""
import numpy as np
import pytest

import oracle as O
from comparators import (assert_abs_eq, assert_matrix_float_eq, assert_ulp_eq, backward_error, float_eq,
                         perm_from_matrix)


def A(x, dtype=np.float64):
    return np.array(x, dtype=dtype).reshape(len(x), -1) if len(x) else np.zeros((0, 0), dtype=dtype)


def reconstruct_lu(lu, perm):
    n = lu.shape[0]
    l = np.tril(lu, -1) + np.eye(n)
    u = np.triu(lu)
    # p.inverse() * l * u: `P * X` sends row i of X to row q[i] (permute_rows_in_place,
    # permutation_matrix.rs:479-509) with q = p.inverse(), so row j of the result is
    # row p[j] of L U.
    return (l @ u)[perm.astype(np.int64)]


def test_dot_order(golden):
    # utils::dot's 8-lane order is observable in f32 with cancellation
    u = np.array([1e8, 1, -1e8, 1, 1, 1, 1, 1, 3], dtype=np.float32)
    v = np.ones(9, dtype=np.float32)
    p = [0.0] * 8
    for i in range(8):
        p[i] = np.float32(p[i] + u[i] * v[i])
    s = np.float32(0)
    for a, b in ((0, 4), (1, 5), (2, 6), (3, 7)):
        s = np.float32(np.float32(s + p[a]) + p[b])
    s = np.float32(s + u[8] * v[8])
    assert O.dot(u, v) == s


def test_lu_exact_3x3(golden):
    c = golden["lu_exact_3x3"]
    lu, perm, st = O.lu_decompose(A(c["a"]))
    assert st == O.OK
    l = np.tril(lu, -1) + np.eye(3)
    u = np.triu(lu)
    assert_matrix_float_eq(l, A(c["l"]))
    assert_matrix_float_eq(u, A(c["u"]))
    assert np.array_equal(perm, perm_from_matrix(c["p"]))


@pytest.mark.parametrize("name", ["lu_reconstruct_5x5", "lu_reconstruct_9x9", "lu_reconstruct_4x4_d",
                                  "lu_reconstruct_4x4_x"])
def test_lu_reconstruction(golden, name):
    a = A(golden[name]["a"])
    lu, perm, st = O.lu_decompose(a)
    assert st == O.OK
    assert_matrix_float_eq(reconstruct_lu(lu, perm), a)


def test_lu_inverse(golden):
    c = golden["lu_inverse_4x4"]
    lu, perm, st = O.lu_decompose(A(c["a"]))
    inv, st = O.lu_inverse(lu, perm)
    assert st == O.OK
    assert_matrix_float_eq(inv, A(c["inv"]))


def test_lu_det(golden):
    c = golden["lu_det_4x4"]
    lu, perm, _ = O.lu_decompose(A(c["a"]))
    assert float_eq(O.lu_det(lu, perm), c["det"])


def test_lu_solve(golden):
    c = golden["lu_solve_4x4"]
    lu, perm, _ = O.lu_decompose(A(c["a"]))
    x, st = O.lu_solve(lu, perm, np.array(c["b"]))
    assert st == O.OK
    assert_ulp_eq(x, c["x"], c["ulp_tol"])


def test_lu_singular(golden):
    _, _, st = O.lu_decompose(A(golden["lu_singular_4x4"]["a"]))
    assert st == O.DIV_BY_ZERO


def test_lu_forward_substitution(golden):
    # lu_forward_substitution is private; through solve with the identity permutation
    # and an identity-U factor the unit-lower part is what is exercised.
    c = golden["lu_forward_substitution"]
    for lu_, b, x in ((c["lu1"], c["b1"], c["x1"]), (c["lu2"], c["b2"], c["x2"])):
        lu = A(lu_)
        n = lu.shape[0]
        f = np.tril(lu, -1) + np.eye(n)
        y, st = O.lu_solve(f, np.arange(n, dtype=np.uint64), np.array(b))
        assert st == O.OK and np.array_equal(y, np.array(x))


def test_solve_poisson(golden):
    c = golden["solve_poisson_9x9"]
    lu, perm, _ = O.lu_decompose(A(c["a"]))
    x, st = O.lu_solve(lu, perm, np.array(c["b"]))
    assert_abs_eq(x, c["x"], c["abs_tol"])


def test_matrix_det(golden):
    c = golden["matrix_det"]
    for key, want in zip(["a2", "c3", "e5", "g4"], c["dets"]):
        got = O.matrix_det(A(c[key]))
        assert float_eq(got, want), (key, got, want)


def test_matrix_solve(golden):
    for name in ("matrix_solve_2x2", "matrix_solve_doc"):
        c = golden[name]
        lu, perm, _ = O.lu_decompose(A(c["a"]))
        x, st = O.lu_solve(lu, perm, np.array(c["y"]))
        assert st == O.OK and np.array_equal(x, np.array(c["x"]))


def test_cholesky_unpack(golden):
    c = golden["cholesky_unpack_1x1_2x2"]
    for a, l in ((c["a1"], c["l1"]), (c["a2"], c["l2"])):
        ls, st = O.chol_decompose(A(a))
        assert st == O.OK
        assert_matrix_float_eq(np.tril(ls), A(l))
    ls, st = O.chol_decompose(np.zeros((0, 0)))
    assert st == O.OK


def test_cholesky_failures(golden):
    c = golden["cholesky_fails"]
    for k in ("a1", "a2", "a3", "a4"):
        _, st = O.chol_decompose(A(c[k]))
        assert st == O.DECOMP_FAILURE, k


def test_cholesky_det(golden):
    c = golden["cholesky_det"]
    for k, want in zip(("a1", "a2"), c["dets"]):
        l, _ = O.chol_decompose(A(c[k]))
        assert float_eq(O.chol_det(l), want)
    assert O.chol_det(np.zeros((0, 0))) == 1.0


def test_cholesky_solve_inverse(golden):
    c = golden["cholesky_solve"]
    for a, b, x in ((c["a1"], c["b1"], c["x1"]), (c["a2"], c["b2"], c["x2"])):
        l, _ = O.chol_decompose(A(a))
        y, st = O.chol_solve(l, np.array(b))
        assert st == O.OK
        assert_matrix_float_eq(y, np.array(x))
    c = golden["cholesky_inverse"]
    for a, inv in ((c["a1"], c["inv1"]), (c["a2"], c["inv2"]), (c["a3"], c["inv3"])):
        l, _ = O.chol_decompose(A(a))
        got, st = O.chol_inverse(l)
        assert st == O.OK
        # the third case's expectation carries 16 significant digits only
        assert_matrix_float_eq(got, A(inv), eps=1e-15 if len(inv) < 3 else 1e-14)


def test_cholesky_doc(golden):
    c = golden["cholesky_doc"]
    l, st = O.chol_decompose(A(c["a"]))
    assert_matrix_float_eq(np.tril(l), A(c["l"]))
    for b, x in ((c["b1"], c["x1"]), (c["b2"], c["x2"])):
        y, st = O.chol_solve(l, np.array(b))
        assert_matrix_float_eq(y, np.array(x), eps=1e-12)


def test_cholesky_legacy(golden):
    c = golden["cholesky_legacy_3x3"]
    l, _ = O.chol_decompose(A(c["a"]))
    assert np.array_equal(np.tril(l).reshape(-1), np.array(c["l_flat"]))


def test_transpose_back_substitution(golden):
    c = golden["transpose_back_substitution"]
    for i in (1, 2, 3):
        x, st = O.transpose_back_substitution(A(c[f"l{i}"]), np.array(c[f"b{i}"]))
        assert st == O.OK
        assert_matrix_float_eq(x, np.array(c[f"x{i}"]))


def test_qr_reconstruction(golden):
    for mat in golden["qr_reconstruct_shapes"]["mats"]:
        a = A(mat)
        m, n = a.shape
        qr, tau = O.qr_decompose(a)
        q = O.qr_first_k_columns(qr, tau, m)
        r = np.triu(qr)
        assert_matrix_float_eq(q @ r, a, ulp=100)
        # qr.rs:413-416 checks q^T q with its own matrixmultiply product; numpy's product
        # rounds differently by up to one ulp of 1, hence 4 eps instead of eps here.
        assert_matrix_float_eq(q.T @ q, np.eye(m), eps=4 * np.finfo(np.float64).eps, ulp=100)
        # thin
        k = min(m, n)
        q1 = O.qr_first_k_columns(qr, tau, k)
        assert_matrix_float_eq(q1 @ np.triu(qr[:k, :]), a, ulp=100)


def test_qr_legacy_sign_convention(golden):
    c = golden["qr_legacy_3x3"]
    qr, tau = O.qr_decompose(A(c["a"]))
    q = O.qr_first_k_columns(qr, tau, 3)
    assert_abs_eq(q, A(c["q"]), c["abs_tol"])
    assert_abs_eq(np.triu(qr), A(c["r"]), c["abs_tol"])


def test_householder_compute(golden):
    c = golden["householder_compute"]
    for k in ("x1", "x2", "x3"):
        x = np.array(c[k])
        v, tau = O.house_compute(x)
        h = np.eye(len(x)) - tau * np.outer(v, v)
        y = h @ x
        assert_matrix_float_eq(y[1:], np.zeros(len(x) - 1), eps=1e-12)
        assert_matrix_float_eq(h @ y, x)
    _, tau = O.house_compute(np.array([2.0]))
    assert tau == 0.0


def test_householder_left_multiply(golden):
    c = golden["householder_left_multiply"]
    got = O.house_apply(A(c["a"]), np.array(c["v"]), c["tau"])
    assert_abs_eq(got, A(c["expected"]), c["abs_tol"])


def test_householder_composition(golden):
    c = golden["householder_composition"]
    s, tau = A(c["storage"]), np.array(c["tau"])
    for x, e in (("x_square", "e_square"), ("x_tall", "e_tall"), ("x_short", "e_short")):
        got = O.qr_q_left_multiply(s, tau, A(c[x]))
        assert_matrix_float_eq(got, A(c[e]), eps=c["eps"])
    c = golden["householder_first_k_columns"]
    q = A(c["q"])
    for k in (1, 2, 3):
        got = O.qr_first_k_columns(A(c["storage"]), np.array(c["tau"]), k)
        assert_matrix_float_eq(got, q[:, :k])
    assert O.qr_first_k_columns(A(c["storage"]), np.array(c["tau"]), 0).shape == (3, 0)


def test_qt_left_multiply_inverts_q():
    """Q^T (Q X) = X for the oracle's two reflector orders, and Q^T X equals the
    least-squares composition's q1^T X (first_k_columns, transposed, times X)."""
    rng = np.random.default_rng(8)
    for m, n in ((7, 4), (9, 9), (5, 8)):
        qr, tau = O.qr_decompose(rng.standard_normal((m, n)))
        x = rng.standard_normal((m, 3))
        back = O.qr_qt_left_multiply(qr, tau, O.qr_q_left_multiply(qr, tau, x))
        assert np.max(np.abs(back - x)) <= 1e-14 * m
        q = O.qr_first_k_columns(qr, tau, m)
        assert np.max(np.abs(O.qr_qt_left_multiply(qr, tau, x) - q.T @ x)) <= 1e-14 * m


@pytest.mark.parametrize("name,dtype", [("gemm_f32_3x2_2x3", np.float32), ("gemm_f64_3x2_2x3", np.float64)])
def test_gemm_golden(golden, name, dtype):
    c = golden[name]
    got = O.gemm(A(c["a"], dtype), A(c["b"], dtype))
    assert np.array_equal(got.reshape(-1), np.array(c["c"], dtype=dtype))


def test_permutation_golden(golden):
    p = list(range(4))
    for i, j in golden["perm_swap_rows"]["swaps"]:
        p[i], p[j] = p[j], p[i]
    assert p == [int(v) for v in golden["perm_swap_rows"]["expected"]]
    c = golden["perm_parity"]
    assert O.perm_parity_odd(np.array(c["even"])) == 0
    assert O.perm_parity_odd(np.array(c["odd"])) == 1
    c = golden["perm_invalid"]
    for k in ("a", "b", "c"):
        assert O.perm_validate(np.array(c[k])) == O.INVALID_PERMUTATION
    c = golden["perm_inverse"]
    p = np.array(c["p"], dtype=np.int64)
    inv = np.empty_like(p)
    inv[p] = np.arange(len(p))
    assert np.array_equal(inv, np.array(c["inverse"], dtype=np.int64))


def test_lstsq_composition():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((12, 5))
    b = rng.standard_normal(12)
    x, st = O.qr_lstsq(a, b)
    assert st == O.OK
    want = np.linalg.lstsq(a, b, rcond=None)[0]
    assert np.max(np.abs(x - want)) < 1e-12


def test_lu_random_backward_error():
    rng = np.random.default_rng(1)
    for n in (1, 7, 33, 100):
        a = rng.uniform(-1, 1, (n, n)) + np.eye(n)
        b = rng.uniform(-1, 1, n)
        lu, perm, st = O.lu_decompose(a)
        x, st = O.lu_solve(lu, perm, b)
        assert st == O.OK
        assert backward_error(a, x, b) < n * 2.0 ** -53 * 10
        assert np.allclose(reconstruct_lu(lu, perm), a, atol=1e-13 * n)


def test_batch_loop_matches_single_calls():
    rng = np.random.default_rng(2)
    ns = np.array([3, 8, 1, 20], dtype=np.int32)
    kind = np.array([0, 1, 0, 1], dtype=np.uint8)
    mats, rhs = [], []
    for n, k in zip(ns, kind):
        g = rng.standard_normal((n, n))
        mats.append(g @ g.T + n * np.eye(n) if k else rng.uniform(-1, 1, (n, n)) + n * np.eye(n))
        rhs.append(rng.standard_normal(n))
    a_off = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]])
    b_off = np.concatenate([[0], np.cumsum(ns.astype(np.int64))[:-1]])
    a = np.concatenate([m.reshape(-1) for m in mats])
    b = np.concatenate(rhs)
    info = O.batch_solve(ns, kind, a_off, a, b_off, b, threads=2)
    assert (info == 0).all()
    for i, (m, r) in enumerate(zip(mats, rhs)):
        if kind[i]:
            l, _ = O.chol_decompose(m)
            want, _ = O.chol_solve(l, r)
        else:
            lu, perm, _ = O.lu_decompose(m)
            want, _ = O.lu_solve(lu, perm, r)
        assert np.array_equal(b[b_off[i]:b_off[i] + ns[i]], want)


def _corrected_full_lu_solve(olu, op, oq, b):
    y, st = O.full_lu_solve(olu, op, np.arange(len(oq), dtype=np.uint64), b)
    return y[oq.astype(np.int64)], st


def test_full_lu_reference_solve_scatter_differs_only_for_non_involutions():
    """The reference's FullPivLu::solve applies q by scatter (`&self.q * x`, lu.rs:485): on
    its own 4 x 4 case that agrees with the gather x[i] = y[q[i]]; on a random 40 x 40
    matrix the scatter's x does not solve A x = b and the gather's is f64-accurate (the
    GPU path gathers)."""
    from comparators import backward_error
    a = np.array([[5.0, 0, 0, 1], [2, 2, 2, 1], [4, 5, 5, 5], [1, 6, 4, 5]])
    b = np.array([9.0, 16, 49, 45])
    olu, op, oq, _, _ = O.full_lu_decompose(a)
    assert np.array_equal(O.full_lu_solve(olu, op, oq, b)[0], _corrected_full_lu_solve(olu, op, oq, b)[0])
    rng = np.random.default_rng(40)
    a = rng.uniform(-1, 1, (40, 40))
    b = rng.standard_normal(40)
    olu, op, oq, _, _ = O.full_lu_decompose(a)
    assert backward_error(a, O.full_lu_solve(olu, op, oq, b)[0], b) > 1e-3
    assert backward_error(a, _corrected_full_lu_solve(olu, op, oq, b)[0], b) <= 40 * 2.0 ** -53 * 10


def test_full_lu_oracle_golden(golden):
    """FullPivLu restatement against the reference's known answers (lu.rs:892-1018, the
    rank doc example lu.rs:537-541): reconstruction (L U)[p][:, q] = A, ranks, the 4 x 4
    solve within 100 ULP, the inverse, and a singular matrix that is not invertible."""
    for name in ("full_lu_reconstruct_4x4", "full_lu_singular_rank3", "full_lu_doc_rank2"):
        c = golden[name]
        a = A(c["a"])
        lu, p, q, _, _ = O.full_lu_decompose(a)
        n = len(a)
        rec = ((np.tril(lu, -1) + np.eye(n)) @ np.triu(lu))[p.astype(np.int64)][:, q.astype(np.int64)]
        assert_matrix_float_eq(rec, a)
        if "rank" in c:
            assert O.full_lu_rank(lu) == c["rank"]
    c = golden["full_lu_solve_4x4"]
    lu, p, q, _, _ = O.full_lu_decompose(A(c["a"]))
    x, st = O.full_lu_solve(lu, p, q, np.array(c["b"]))
    assert st == O.OK
    assert_ulp_eq(x, np.array(c["x"]), c["ulp_tol"])
    c = golden["full_lu_noninvertible_3x3"]
    lu, _, _, _, _ = O.full_lu_decompose(A(c["a"]))
    assert not O.full_lu_is_invertible(lu)


def test_backward_error_flags_non_finite():
    """The test-side backward error is inf for a solution with a NaN or inf entry, so a
    NaN produced by a kernel can never pass a backward-error bound."""
    from comparators import backward_error
    a = np.eye(3)
    assert backward_error(a, np.array([np.nan, 1.0, 1.0]), np.ones(3)) == float("inf")
    assert backward_error(a, np.array([np.inf, 1.0, 1.0]), np.ones(3)) == float("inf")
    assert backward_error(a, np.ones(3), np.ones(3)) == 0.0
