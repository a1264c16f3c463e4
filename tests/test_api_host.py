"""Host-side behaviour of the Python mirror of rulinalg's types that needs no GPU: the
reference's assert!-panics on misuse (raised before any library call, with the
reference's messages) and `PartialPivLu::unpack` (lu.rs:138-149) on a compact LU from
the oracle, checked against the reference's exact 3x3 known answer
(tests/mat/mod.rs:104-125)."""
import numpy as np
import pytest

import oracle as O
from comparators import assert_matrix_float_eq, perm_from_matrix


def A(x):
    return np.array(x, dtype=np.float64)


def test_mat_mul_dimension_panic(rl):
    with pytest.raises(rl.RulinalgPanic, match="Matrix dimensions do not agree"):  # mat_mul.rs:21
        rl.mat_mul(np.zeros((2, 3)), np.zeros((2, 3)))


def test_lu_panics(rl):
    with pytest.raises(rl.RulinalgPanic, match="square for LU"):  # lu.rs:165
        rl.PartialPivLu.decompose(np.zeros((3, 4)))
    lu = rl.PartialPivLu(np.eye(3), np.arange(3, dtype=np.uint64))
    with pytest.raises(rl.RulinalgPanic, match="compatible size"):  # lu.rs:232
        lu.solve(np.ones(4))


def test_cholesky_panics(rl):
    with pytest.raises(rl.RulinalgPanic, match="square for Cholesky"):  # cholesky.rs:117
        rl.Cholesky.decompose(np.zeros((2, 3)))
    with pytest.raises(rl.RulinalgPanic, match="dimensionally compatible"):  # cholesky.rs:195
        rl.Cholesky(np.eye(3)).solve(np.ones(2))


def test_lstsq_mixed_panics(rl):
    with pytest.raises(rl.RulinalgPanic):
        rl.lstsq_mixed(np.zeros(5), np.zeros(5))
    with pytest.raises(rl.RulinalgPanic):
        rl.lstsq_mixed(np.zeros((6, 3)), np.zeros(5))


def test_lu_unpack_matches_reference_3x3(rl, golden):
    c = golden["lu_exact_3x3"]
    lu, perm, st = O.lu_decompose(A(c["a"]))
    assert st == O.OK
    lup = rl.PartialPivLu(lu, perm).unpack()
    assert_matrix_float_eq(lup.l, A(c["l"]))
    assert_matrix_float_eq(lup.u, A(c["u"]))
    assert np.array_equal(lup.p.perm, perm_from_matrix(c["p"]))
    # unit lower / upper structure
    assert np.array_equal(np.diag(lup.l), np.ones(3)) and not np.triu(lup.l, 1).any()
    assert not np.tril(lup.u, -1).any()


def test_autotune_key_follows_the_size_histogram(rl):
    """The autotuner's cache key: the same for batches with the same per-octave size
    histogram, different when the histogram, the precision or the GPU changes."""
    from rulinalg_gb300.autotune import batch_key
    n1 = [8, 9, 100, 300, 300]
    k1 = [0, 0, 1, 1, 0]
    assert batch_key(n1, k1, 1, "GB300") == batch_key([15, 8, 127, 511, 256], k1, 1, "GB300")
    assert batch_key(n1, k1, 1, "GB300") != batch_key(n1, [1, 0, 1, 1, 0], 1, "GB300")
    assert batch_key(n1, k1, 1, "GB300") != batch_key(n1, k1, 0, "GB300")
    assert batch_key(n1, k1, 1, "GB300") != batch_key(n1, k1, 1, "other")


def test_bench_profile_traffic_line(tmp_path):
    """bench.py scales the committed batched-kernel traffic line `T @ M` by matrix bytes."""
    import bench
    p = tmp_path / "prof.md"
    p.write_text("x\ntraffic_per_launch_bytes: 99200000000 @ 10012700000\n")
    assert abs(bench.profile_traffic(10012700000, p) - 99.2e9) < 1
    assert abs(bench.profile_traffic(5006350000, p) - 49.6e9) < 1
    p.write_text("traffic_per_launch_bytes: 99200000000\n")
    assert bench.profile_traffic(1.0, p) is None
    assert bench.profile_traffic(1.0) is not None  # the committed profile carries the line


def test_bench_cpulist_parse():
    """bench.py's sysfs local_cpulist parser (used to keep the end-to-end leg's pinned
    buffers on the GPU's own host memory)."""
    import bench
    assert bench.parse_cpulist("0-3,8,10-11\n") == {0, 1, 2, 3, 8, 10, 11}
    assert bench.parse_cpulist("72-143") == set(range(72, 144))
