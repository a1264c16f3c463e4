"""Parity of the CUDA single-matrix paths with the oracle, through the C ABI.

GEMM: normwise ||C - C_ref||_F <= n eps ||A||_F ||B||_F against the f64 oracle (eps of
the computing type). Factorisations: permutations bit-identical to the oracle where
the oracle's pivot choice is unique by a margin, factors normwise close, every solve's
normwise backward error <= n 2^-53 10 (f64) and forward error reported against the
oracle. Known answers use the reference's comparators.
"""
import os

import numpy as np
import pytest

import oracle as O
from comparators import (assert_abs_eq, assert_matrix_float_eq, assert_ulp_eq, backward_error, float_eq,
                         perm_from_matrix)

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53
U32 = 2.0 ** -24


def A(x, dtype=np.float64):
    return np.array(x, dtype=dtype).reshape(len(x), -1) if len(x) else np.zeros((0, 0), dtype=dtype)


def fro(x):
    return float(np.sqrt(np.sum(np.asarray(x, dtype=np.float64) ** 2)))


# ----------------------------------------------------------------------- GEMM --
@pytest.mark.parametrize("name,dtype", [("gemm_f32_3x2_2x3", np.float32), ("gemm_f64_3x2_2x3", np.float64)])
def test_gemm_golden(gpu, golden, name, dtype):
    c = golden[name]
    got = gpu.mat_mul(A(c["a"], dtype), A(c["b"], dtype))
    assert np.array_equal(got.reshape(-1), np.array(c["c"], dtype=dtype))


def test_gemm_slice_uneven(gpu, golden):
    c = golden["gemm_slice_uneven"]
    full = A(c["c"])
    d = full[0:2, 0:2]  # a MatrixSlice: row stride 3 > cols 2
    assert d.strides[0] == 3 * 8
    got = gpu.mat_mul(d, A(c["a"]))
    assert np.array_equal(got.reshape(-1), np.array(c["e"]))
    ones = 2 * np.ones((3, 3))
    s = ones[1:3, 1:3]
    assert np.array_equal(gpu.mat_mul(s, s), np.full((2, 2), 8.0))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,k,n", [(1, 1, 1), (7, 3, 5), (64, 64, 64), (129, 65, 257), (300, 1, 2), (1, 500, 1),
                                   (513, 257, 130), (1000, 1000, 1000)])
def test_gemm_normwise(gpu, dtype, m, k, n):
    rng = np.random.default_rng(m * 7 + k * 3 + n)
    a = rng.standard_normal((m, k)).astype(dtype)
    b = rng.standard_normal((k, n)).astype(dtype)
    got = gpu.mat_mul(a, b)
    ref = O.gemm(a.astype(np.float64), b.astype(np.float64))
    eps = U64 if dtype == np.float64 else U32
    assert fro(got.astype(np.float64) - ref) <= max(k, 1) * eps * fro(a) * fro(b)


@pytest.mark.parametrize("m,k,n", [(128, 256, 128), (256, 256, 256), (200, 300, 300), (130, 270, 131),
                                   (64, 1000, 256), (1024, 512, 768), (2048, 2048, 2048)])
def test_sgemm_tensor_core_elementwise(gpu, m, k, n):
    """Shapes that take the tcgen05 3xTF32 path (a 128 x 128 tile's worth of C, k >= 256;
    ragged edges and a half-height tile included): every element within the FP32
    dot-product bound 2 k eps (|A| |B|)."""
    rng = np.random.default_rng(m + 3 * k + 7 * n)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((k, n)).astype(np.float32)
    got = gpu.mat_mul(a, b).astype(np.float64)
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    ref = a64 @ b64
    bound = 2 * k * U32 * (np.abs(a64) @ np.abs(b64))
    assert np.all(np.abs(got - ref) <= bound), np.max(np.abs(got - ref) / bound)


@pytest.mark.parametrize("m,k,n,dtype", [(128, 4096, 128, np.float32), (64, 3000, 300, np.float32),
                                         (50, 5000, 60, np.float32), (64, 4096, 64, np.float64),
                                         (100, 3000, 130, np.float64)])
def test_gemm_split_k(gpu, m, k, n, dtype):
    """Products with few output tiles and a long K run as K slices at once (tensor-core
    and SIMT paths, ragged slices): every element within the dot-product bound of the
    type, 2 k eps (|A| |B|)."""
    rng = np.random.default_rng(m + k + n)
    a = rng.standard_normal((m, k)).astype(dtype)
    b = rng.standard_normal((k, n)).astype(dtype)
    got = gpu.mat_mul(a, b).astype(np.float64)
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    eps = U32 if dtype == np.float32 else U64
    bound = 2 * k * eps * (np.abs(a64) @ np.abs(b64))
    assert np.all(np.abs(got - a64 @ b64) <= bound), np.max(np.abs(got - a64 @ b64) / bound)


def test_gemm_k_zero_and_empty(gpu):
    c = gpu.mat_mul(np.zeros((3, 0)), np.zeros((0, 4)))
    assert c.shape == (3, 4) and not c.any()
    assert gpu.mat_mul(np.zeros((0, 5)), np.zeros((5, 2))).shape == (0, 2)
    with pytest.raises(gpu.RulinalgPanic):
        gpu.mat_mul(np.zeros((2, 3)), np.zeros((2, 3)))


THREADS = os.cpu_count() or 1


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n", [1024, 2048, 4096])
def test_gemm_config2_against_oracle(gpu, dtype, n):
    """The dense GEMM sweep's sizes (N(0,1), seeded, row-major): normwise
    ||C - C_ref||_F <= n eps ||A||_F ||B||_F against the oracle's f64 product of the same
    (type-rounded) inputs, the oracle's rows split over all host threads."""
    from rulinalg_gb300.workloads import gemm_operands
    a, b = gemm_operands(n, dtype, seed=n)
    got = gpu.mat_mul(a, b).astype(np.float64)
    ref = O.gemm(a.astype(np.float64), b.astype(np.float64), threads=THREADS)
    eps = U64 if dtype == np.float64 else U32
    err, bound = fro(got - ref), n * eps * fro(a) * fro(b)
    print(f"gemm n={n} {np.dtype(dtype).name}: ||C - C_ref||_F / bound = {err / bound:.3e}")
    assert err <= bound


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gemm_config2_8192(gpu, dtype):
    """n = 8192, the sweep's largest size: the oracle's scalar i-k-j loop would be 1.1
    TFLOP of scalar work (many minutes on the host), so the reference product here is an
    FP64 product on the GPU (torch / cuBLAS DGEMM, error ~ sqrt(n) 2^-53 |A||B|, far inside
    the bound), against the same normwise bound n eps ||A||_F ||B||_F."""
    import torch
    from rulinalg_gb300.workloads import gemm_operands
    n = 8192
    a, b = gemm_operands(n, dtype, seed=n)
    got = gpu.mat_mul(a, b).astype(np.float64)
    dev = torch.device("cuda:0")
    ref = (torch.from_numpy(a.astype(np.float64)).to(dev) @ torch.from_numpy(b.astype(np.float64)).to(dev)).cpu().numpy()
    eps = U64 if dtype == np.float64 else U32
    err, bound = fro(got - ref), n * eps * fro(a) * fro(b)
    print(f"gemm n={n} {np.dtype(dtype).name}: ||C - C_ref||_F / bound = {err / bound:.3e}")
    assert err <= bound


def test_gemm_large_linearity(gpu):
    """n = 4096: size-independent check A (B x) == (A B) x within the normwise bound."""
    n = 4096
    rng = np.random.default_rng(11)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal((n, n))
    x = rng.standard_normal(n)
    c = gpu.mat_mul(a, b)
    lhs = c @ x
    rhs = a @ (b @ x)
    bound = n * U64 * fro(a) * fro(b) * np.linalg.norm(x) * 4
    assert np.linalg.norm(lhs - rhs) <= bound


# ------------------------------------------------------------------------- LU --
def reconstruct_lu(lu, perm):
    n = lu.shape[0]
    l = np.tril(lu, -1) + np.eye(n)
    return (l @ np.triu(lu))[perm.astype(np.int64)]


def test_lu_exact_3x3(gpu, golden):
    c = golden["lu_exact_3x3"]
    lup = gpu.PartialPivLu.decompose(A(c["a"])).unpack()
    assert_matrix_float_eq(lup.l, A(c["l"]))
    assert_matrix_float_eq(lup.u, A(c["u"]))
    assert np.array_equal(lup.p.perm, perm_from_matrix(c["p"]))


@pytest.mark.parametrize("name", ["lu_reconstruct_5x5", "lu_reconstruct_9x9", "lu_reconstruct_4x4_d",
                                  "lu_reconstruct_4x4_x"])
def test_lu_reconstruction(gpu, golden, name):
    a = A(golden[name]["a"])
    lu = gpu.PartialPivLu.decompose(a)
    assert_matrix_float_eq(reconstruct_lu(lu.lu, lu.p.perm), a)
    olu, operm, _ = O.lu_decompose(a)
    assert np.array_equal(lu.p.perm, operm)


def test_lu_inverse_det_solve(gpu, golden):
    c = golden["lu_inverse_4x4"]
    assert_matrix_float_eq(gpu.PartialPivLu.decompose(A(c["a"])).inverse(), A(c["inv"]))
    c = golden["lu_det_4x4"]
    assert float_eq(gpu.PartialPivLu.decompose(A(c["a"])).det(), c["det"])
    c = golden["lu_solve_4x4"]
    assert_ulp_eq(gpu.PartialPivLu.decompose(A(c["a"])).solve(np.array(c["b"])), c["x"], c["ulp_tol"])
    c = golden["solve_poisson_9x9"]
    assert_abs_eq(gpu.PartialPivLu.decompose(A(c["a"])).solve(np.array(c["b"])), c["x"], c["abs_tol"])
    assert gpu.PartialPivLu.decompose(np.eye(3)).det() == 1.0
    assert_matrix_float_eq(gpu.PartialPivLu.decompose(np.eye(3)).inverse(), np.eye(3))


def test_lu_singular(gpu, golden):
    with pytest.raises(gpu.RulinalgError) as e:
        gpu.PartialPivLu.decompose(A(golden["lu_singular_4x4"]["a"]))
    assert e.value.kind == "DivByZero"
    with pytest.raises(gpu.RulinalgPanic):
        gpu.PartialPivLu.decompose(np.ones((2, 3)))


def test_lu_empty(gpu):
    lu = gpu.PartialPivLu.decompose(np.zeros((0, 0)))
    assert lu.det() == 1.0
    assert lu.inverse().shape == (0, 0)


def unique_pivot_input(n, rng, margin=1e-6):
    """U(-1,1) + I inputs whose oracle pivot choice is unique by `margin` at every step."""
    for _ in range(20):
        a = rng.uniform(-1.0, 1.0, (n, n)) + np.eye(n)
        _, _, st, gap = O.lu_decompose(a, gaps=True)
        if st == O.OK and (n < 2 or gap[:-1].min() > margin):
            return a
    raise RuntimeError("no input with unique pivots")


@pytest.mark.parametrize("n", [1, 2, 5, 16, 31, 32, 33, 64, 65, 100, 255, 256, 257, 511, 512, 513, 600, 777])
def test_lu_parity_random(gpu, n):
    rng = np.random.default_rng(n)
    a = unique_pivot_input(n, rng)
    b = rng.uniform(-1, 1, n)
    olu, operm, _ = O.lu_decompose(a)
    lu = gpu.PartialPivLu.decompose(a)
    assert np.array_equal(lu.p.perm, operm), "pivots differ from the oracle"
    lref, uref = np.tril(olu, -1), np.triu(olu)
    assert fro(np.tril(lu.lu, -1) - lref) <= 1e-11 * max(fro(lref), 1)
    assert fro(np.triu(lu.lu) - uref) <= 1e-11 * fro(uref)
    x = lu.solve(b)
    assert backward_error(a, x, b) <= n * U64 * 10
    xo, _ = O.lu_solve(olu, operm, b)
    assert np.max(np.abs(x - xo)) <= 1e-9 * max(np.max(np.abs(xo)), 1)


def unique_max_by_construction(n, rng, dtype):
    """A = P^T L U with L unit lower triangular, |l_ij| <= 1/(2 sqrt(n)), and a random
    row permutation P: at every elimination step the candidates of the pivot column are
    u_kk l_ik, so partial pivoting must take the row holding l_kk = 1, by a margin of
    about |u_kk| (1 - 1/(2 sqrt(n))). The off-diagonal scale keeps ||L - I||_2 below 1/2
    (L and U well conditioned), so FP32 rounding of A cannot move a multiplier far
    enough to close that margin. The tests check the oracle's gaps."""
    c = 0.5 / np.sqrt(max(n, 1))
    l = np.tril(rng.uniform(-c, c, (n, n)), -1) + np.eye(n)
    u = np.triu(rng.uniform(-2 * c, 2 * c, (n, n)), 1) + np.diag(rng.uniform(1.0, 2.0, n) * rng.choice([-1, 1], n))
    p = rng.permutation(n)
    a = np.empty((n, n))
    a[p] = l @ u  # row i of L U lands at row p[i]
    return a.astype(dtype)


def test_lu_f32_parity(gpu):
    """FP32 PartialPivLu: pivots bit-identical to the oracle's on inputs with a unique
    column maximum at every step (asserted for every size), factors and solves checked."""
    rng = np.random.default_rng(3)
    for n in (9, 100, 300, 700, 1500):
        a = unique_max_by_construction(n, rng, np.float32)
        olu, operm, st, gap = O.lu_decompose(a, gaps=True)
        assert st == O.OK and (n < 2 or gap[:-1].min() > 0.3)
        lu = gpu.PartialPivLu.decompose(a)
        assert lu.lu.dtype == np.float32
        assert np.array_equal(lu.p.perm, operm), n
        assert fro(np.triu(lu.lu) - np.triu(olu)) <= 10 * n * U32 * fro(np.triu(olu))
        b = rng.uniform(-1, 1, n).astype(np.float32)
        x = lu.solve(b)
        assert backward_error(a, x, b) <= n * U32 * 10


def test_config1_lu_1024(gpu):
    """PartialPivLu decompose + solve in f64 on the 1024 x 1024 seed-0 system: the
    permutation bit-identical, L/U normwise errors and the backward error reported."""
    from rulinalg_gb300.workloads import config1_lu
    a, x_true, b = config1_lu(1024, 0)
    olu, operm, st, gap = O.lu_decompose(a, gaps=True)
    assert st == O.OK
    lu = gpu.PartialPivLu.decompose(a)
    min_gap = float(gap[:-1].min())
    if min_gap > 1e-8:
        assert np.array_equal(lu.p.perm, operm)
    lref, uref = np.tril(olu, -1), np.triu(olu)
    el = fro(np.tril(lu.lu, -1) - lref) / fro(lref)
    eu = fro(np.triu(lu.lu) - uref) / fro(uref)
    x = lu.solve(b)
    be = backward_error(a, x, b)
    print(f"config1: min pivot gap {min_gap:.3e} L err {el:.3e} U err {eu:.3e} backward err {be:.3e}")
    assert el < 1e-11 and eu < 1e-11
    assert be <= 1024 * U64 * 10


def test_lu_multi_rhs_and_inverse_large(gpu):
    rng = np.random.default_rng(8)
    n = 700
    a = rng.uniform(-1, 1, (n, n)) + n ** 0.5 * np.eye(n)
    lu = gpu.PartialPivLu.decompose(a)
    bb = rng.standard_normal((n, 5))
    xx = lu.solve(bb)
    for j in range(5):
        assert backward_error(a, xx[:, j], bb[:, j]) <= n * U64 * 10
    inv = lu.inverse()
    assert np.max(np.abs(inv @ a - np.eye(n))) < 1e-10


# -------------------------------------------------------------------- Matrix::* --
def test_matrix_det_solve_inverse(gpu, golden):
    c = golden["matrix_det"]
    for key, want in zip(["a2", "c3", "e5", "g4"], c["dets"]):
        assert float_eq(gpu.det(A(c[key])), want), key
    assert gpu.det(np.diag([1.0, 2.0, 3.0, 4.0, 5.0])) == 120.0
    for name in ("matrix_solve_2x2", "matrix_solve_doc"):
        c = golden[name]
        assert np.array_equal(gpu.solve(A(c["a"]), np.array(c["y"])), np.array(c["x"]))
    a = np.array([[2.0, 3.0], [1.0, 2.0]])
    assert_matrix_float_eq(a @ gpu.inverse(a), np.eye(2))


# ------------------------------------------------------------------- Cholesky --
def test_cholesky_golden(gpu, golden):
    c = golden["cholesky_unpack_1x1_2x2"]
    for a, l in ((c["a1"], c["l1"]), (c["a2"], c["l2"])):
        assert_matrix_float_eq(gpu.Cholesky.decompose(A(a)).unpack(), A(l))
    assert gpu.Cholesky.decompose(np.zeros((0, 0))).det() == 1.0
    c = golden["cholesky_fails"]
    for k in ("a1", "a2", "a3", "a4"):
        with pytest.raises(gpu.RulinalgError) as e:
            gpu.Cholesky.decompose(A(c[k]))
        assert e.value.kind == "DecompFailure"
    c = golden["cholesky_det"]
    for k, want in zip(("a1", "a2"), c["dets"]):
        assert float_eq(gpu.Cholesky.decompose(A(c[k])).det(), want)
    c = golden["cholesky_solve"]
    for a, b, x in ((c["a1"], c["b1"], c["x1"]), (c["a2"], c["b2"], c["x2"])):
        assert_matrix_float_eq(gpu.Cholesky.decompose(A(a)).solve(np.array(b)), np.array(x))
    c = golden["cholesky_inverse"]
    for a, inv in ((c["a1"], c["inv1"]), (c["a2"], c["inv2"]), (c["a3"], c["inv3"])):
        assert_matrix_float_eq(gpu.Cholesky.decompose(A(a)).inverse(), A(inv), eps=1e-14)
    c = golden["cholesky_doc"]
    ch = gpu.Cholesky.decompose(A(c["a"]))
    assert_matrix_float_eq(ch.unpack(), A(c["l"]))
    for b, x in ((c["b1"], c["x1"]), (c["b2"], c["x2"])):
        assert_matrix_float_eq(ch.solve(np.array(b)), np.array(x), eps=1e-12)
    c = golden["cholesky_legacy_3x3"]
    assert np.array_equal(gpu.Cholesky.decompose(A(c["a"])).unpack().reshape(-1), np.array(c["l_flat"]))
    for n in range(0, 31, 5):  # property: Cholesky of the identity is the identity
        assert_matrix_float_eq(gpu.Cholesky.decompose(np.eye(n)).unpack(), np.eye(n))


@pytest.mark.parametrize("n", [1, 3, 16, 33, 64, 100, 257, 512, 513, 700, 1500, 2500])
def test_cholesky_parity_random(gpu, n):
    rng = np.random.default_rng(100 + n)
    g = rng.standard_normal((n, n))
    a = g @ g.T + n * np.eye(n)
    a_upper_garbage = a.copy()
    a_upper_garbage[np.triu_indices(n, 1)] = np.nan  # the strict upper triangle is never read
    ol, st = O.chol_decompose(a)
    ch = gpu.Cholesky.decompose(a_upper_garbage)
    assert np.isnan(ch.l[np.triu_indices(n, 1)]).all()  # ... nor written
    l = ch.unpack()
    assert fro(l - np.tril(ol)) <= 1e-12 * fro(np.tril(ol))
    b = rng.standard_normal(n)
    x = ch.solve(b)
    assert backward_error(a, x, b) <= n * U64 * 10
    assert ch.det() == pytest.approx(O.chol_det(ol), rel=1e-10)


@pytest.mark.parametrize("n", [513, 1100, 2500])
def test_cholesky_f32_blocked_against_f64_oracle(gpu, n):
    """Matrix<f32> Cholesky above one CTA's size: 256-column outer blocks whose L21 and
    SYRK run on the tensor cores (3xTF32). Against the f64 oracle's factor of the same
    (f32-rounded) matrix: reconstruction and factor within 10 n u32 (A = G G^T / n + I,
    condition number below 10), strict upper triangle untouched."""
    rng = np.random.default_rng(300 + n)
    g = rng.standard_normal((n, n))
    a32 = (g @ g.T / n + np.eye(n)).astype(np.float32)
    given = a32.copy()
    given[np.triu_indices(n, 1)] = np.nan
    ch = gpu.Cholesky.decompose(given)
    assert np.isnan(ch.l[np.triu_indices(n, 1)]).all()
    l = np.tril(ch.l).astype(np.float64)
    a = a32.astype(np.float64)
    ol, st = O.chol_decompose(a)
    assert st == O.OK
    u32 = 2.0 ** -24
    assert fro(l @ l.T - a) <= 10 * n * u32 * fro(a)
    assert fro(l - np.tril(ol)) <= 10 * n * u32 * fro(np.tril(ol))


# ---------------------------------------------------------------- Householder --
def test_qr_golden(gpu, golden):
    for mat in golden["qr_reconstruct_shapes"]["mats"]:
        a = A(mat)
        m, n = a.shape
        h = gpu.HouseholderQr.decompose(a)
        qr = h.unpack()
        assert_matrix_float_eq(qr.q @ qr.r, a, eps=4 * U64 * 2, ulp=100)
        assert_matrix_float_eq(qr.q.T @ qr.q, np.eye(m), eps=4 * U64 * 2, ulp=100)
        thin = h.unpack_thin()
        assert_matrix_float_eq(thin.q1 @ thin.r1, a, eps=4 * U64 * 2, ulp=100)
    c = golden["qr_legacy_3x3"]
    qr = gpu.HouseholderQr.decompose(A(c["a"])).unpack()
    assert_abs_eq(qr.q, A(c["q"]), c["abs_tol"])
    assert_abs_eq(qr.r, A(c["r"]), c["abs_tol"])


def test_householder_first_k_columns_golden(gpu, golden):
    c = golden["householder_first_k_columns"]
    h = gpu.HouseholderQr(A(c["storage"]), np.array(c["tau"]))
    q = A(c["q"])
    for k in (1, 2, 3):
        assert_matrix_float_eq(h.first_k_columns(k), q[:, :k])
    assert h.first_k_columns(0).shape == (3, 0)


@pytest.mark.parametrize("m,n", [(5, 3), (3, 5), (64, 64), (130, 70), (200, 200), (600, 300), (300, 600),
                                 (1100, 520)])
def test_qr_parity_random(gpu, m, n):
    rng = np.random.default_rng(m * 13 + n)
    a = rng.standard_normal((m, n))
    oqr, otau = O.qr_decompose(a)
    h = gpu.HouseholderQr.decompose(a)
    p = min(m, n)
    assert np.max(np.abs(h.tau - otau)) <= 1e-12
    assert fro(np.triu(h.qr) - np.triu(oqr)) <= 1e-12 * fro(a)
    assert fro(np.tril(h.qr, -1) - np.tril(oqr, -1)) <= 1e-11 * max(fro(np.tril(oqr, -1)), 1)
    q = h.first_k_columns(m)
    oq = O.qr_first_k_columns(oqr, otau, m)
    assert fro(q - oq) <= 1e-12 * m
    assert fro(q @ np.triu(h.qr) - a) <= 10 * max(m, n) * U64 * fro(a)
    assert p == len(h.tau)


@pytest.mark.parametrize("m,n", [(12, 5), (200, 100), (1024, 512), (2000, 600)])
def test_least_squares(gpu, m, n):
    rng = np.random.default_rng(m + n)
    a = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    x = gpu.least_squares(a, b)
    xo, st = O.qr_lstsq(a, b)
    assert st == O.OK
    assert np.max(np.abs(x - xo)) <= 1e-10 * max(np.max(np.abs(xo)), 1)
    # optimality: A^T (A x - b) ~ 0
    assert np.linalg.norm(a.T @ (a @ x - b)) <= 1e-10 * np.linalg.norm(a) ** 2 * np.linalg.norm(x)


@pytest.mark.parametrize("m,n", [(600, 300), (2100, 700)])
def test_qr_f32_against_f64_oracle(gpu, m, n):
    """The FP32 Householder QR (the mixed least-squares factor) agrees with the f64
    oracle to FP32 accuracy; tall panels run on one thread-block cluster."""
    rng = np.random.default_rng(m + 7 * n)
    a = rng.standard_normal((m, n))
    oqr, otau = O.qr_decompose(a)
    h = gpu.HouseholderQr.decompose(a.astype(np.float32))
    assert h.qr.dtype == np.float32
    eps32 = 2.0 ** -24
    assert np.max(np.abs(h.tau.astype(np.float64) - otau)) <= 50 * n * eps32
    r32 = np.triu(h.qr.astype(np.float64))[:n]
    assert fro(r32 - np.triu(oqr)[:n]) <= 10 * n * eps32 * fro(a)


# ---------------------------------------------- cooperative-grid panels (tunable) --
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_lu_and_qr_cooperative_panels(gpu, dtype):
    """RL_TUNE_PANEL_CLUSTER_MAX = 0 sends every blocked LU / QR panel to the
    cooperative-grid kernels (lu_panel_kernel, qr_panel_kernel), which otherwise run only
    for panels too tall for a 16-CTA cluster (FP64 m > ~6,300): pivots bit-identical to
    the oracle on unique-maximum inputs, factors and solves checked, then the default
    restored and the cluster path checked to give the same pivots."""
    from rulinalg_gb300 import _lib as L
    rng = np.random.default_rng(77)
    n = 1100
    a = unique_max_by_construction(n, rng, dtype) if dtype == np.float32 else unique_pivot_input(n, rng)
    b = rng.uniform(-1, 1, n).astype(dtype)
    olu, operm, st = O.lu_decompose(a, threads=THREADS)
    m_qr, n_qr = 1300, 600
    aq = rng.standard_normal((m_qr, n_qr)).astype(dtype)
    oqr, otau = O.qr_decompose(aq.astype(np.float64))
    eps = U64 if dtype == np.float64 else U32
    gpu.tune_set(L.TUNE_PANEL_CLUSTER_MAX, 0)
    try:
        lu = gpu.PartialPivLu.decompose(a)
        x = lu.solve(b)
        h = gpu.HouseholderQr.decompose(aq)
    finally:
        gpu.tune_set(L.TUNE_PANEL_CLUSTER_MAX, 16)
    assert np.array_equal(lu.p.perm, operm)
    assert fro(np.triu(lu.lu) - np.triu(olu)) <= 10 * n * eps * fro(np.triu(olu))
    assert backward_error(a, x, b) <= n * eps * 10
    assert np.max(np.abs(h.tau.astype(np.float64) - otau)) <= 50 * n_qr * eps
    assert fro(np.triu(h.qr.astype(np.float64))[:n_qr] - np.triu(oqr)[:n_qr]) <= 10 * n_qr * eps * fro(aq)
    lu2 = gpu.PartialPivLu.decompose(a)  # default: cluster panels
    assert np.array_equal(lu2.p.perm, operm)


@pytest.mark.parametrize("dtype,n", [(np.float64, 700), (np.float64, 2000), (np.float64, 7000), (np.float32, 1500),
                                     (np.float32, 4096)])
def test_lu_panel_lookahead_bit_identical(gpu, dtype, n):
    """RL_TUNE_PANEL_LOOKAHEAD = 1 overlaps the rest of column j's elimination with column
    j + 1's pivot search and push (cluster panels); every element gets the same
    fma(-l, u, a), so the factors and the permutation are bit-identical to the plain
    panel's (n = 7000 f64: the first panels are too tall for a cluster and run on the
    cooperative kernel, the later ones on the cluster). A mixed-precision solve with it
    stays f64-accurate."""
    from rulinalg_gb300 import _lib as L
    rng = np.random.default_rng(n)
    a = (rng.uniform(-1, 1, (n, n)) + np.eye(n)).astype(dtype)
    saved = gpu.tune_get(L.TUNE_PANEL_LOOKAHEAD)
    try:
        gpu.tune_set(L.TUNE_PANEL_LOOKAHEAD, 0)
        plain = gpu.PartialPivLu.decompose(a)
        gpu.tune_set(L.TUNE_PANEL_LOOKAHEAD, 1)
        la = gpu.PartialPivLu.decompose(a)
        if dtype == np.float64 and n <= 2000:
            b = rng.standard_normal(n)
            x, info = gpu.solve_mixed(a, b, "lu")
            assert backward_error(a, x, b) <= n * U64 * 10, info
    finally:
        gpu.tune_set(L.TUNE_PANEL_LOOKAHEAD, saved)
    assert np.array_equal(la.p.perm, plain.p.perm)
    assert np.array_equal(la.lu.view(np.uint8), plain.lu.view(np.uint8))
