"""Parity of the batched solver (one launch sequence for many n <= 512 systems) with the
oracle, through the C ABI: FP64 plan, mixed-precision plan (FP32 factor + FP64
refinement) and the f32 plan. Every f64-accurate solve must have a normwise backward
error <= n 2^-53 10; results are also compared with the oracle's solution."""
import os

import numpy as np
import pytest

import oracle as O
from comparators import backward_error

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53
U32 = 2.0 ** -24


def make_batch(rng, sizes, kinds):
    mats, rhs = [], []
    for n, k in zip(sizes, kinds):
        if k:
            g = rng.standard_normal((n, n))
            mats.append(g @ g.T + n * np.eye(n))
        else:
            mats.append(rng.uniform(-1, 1, (n, n)) + n * np.eye(n))
        rhs.append(rng.standard_normal(n))
    return mats, rhs


def oracle_solve(m, r, kind):
    if kind:
        l, st = O.chol_decompose(m)
        x, st2 = O.chol_solve(l, r) if st == O.OK else (None, st)
        return x, st or st2
    lu, perm, st = O.lu_decompose(m)
    if st != O.OK:
        return None, st
    return O.lu_solve(lu, perm, r)


EDGE_SIZES = [1, 2, 3, 8, 15, 16, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 200, 255, 256, 257, 300, 400,
              511, 512]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_edge_sizes(gpu, precision):
    rng = np.random.default_rng(7)
    sizes = EDGE_SIZES * 2
    kinds = [0] * len(EDGE_SIZES) + [1] * len(EDGE_SIZES)
    mats, rhs = make_batch(rng, sizes, kinds)
    prec = gpu.PREC_FP64 if precision == "fp64" else gpu.PREC_MIXED
    plan = gpu.BatchPlan(sizes, kinds, prec)
    a, b = plan.pack(mats, rhs)
    x, info, iters, berr = plan.solve(a, b)
    assert (info == 0).all(), info
    xs = plan.unpack(x)
    for i, (m, r, k) in enumerate(zip(mats, rhs, kinds)):
        n = sizes[i]
        be = backward_error(m, xs[i], r)
        assert be <= n * U64 * 10, (n, k, be)
        assert berr[i] <= n * U64 * 10
        xo, st = oracle_solve(m, r, k)
        assert st == O.OK
        assert np.max(np.abs(xs[i] - xo)) <= 1e-12 * max(np.max(np.abs(xo)), 1e-300) * n
        if precision == "mixed":
            assert iters[i] >= 1, "a refinement step always follows the FP32 solve"
    plan.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_warp_tail_boundary(gpu, precision):
    """The small tail of a largest-first batch (cost n^3, x2 for LU, at most 32^3) runs
    one system per warp; systems just above the boundary (LU 26..32, Cholesky 33..40)
    sort in between and stay on the one-CTA path. All agree with the oracle."""
    rng = np.random.default_rng(11)
    sizes = [32, 40, 26, 25, 32, 33, 24, 31, 2, 1, 17, 25, 26, 32, 40, 5]
    kinds = [0, 1, 0, 0, 1, 1, 1, 0, 0, 1, 1, 1, 0, 1, 1, 0]
    mats, rhs = make_batch(rng, sizes, kinds)
    prec = gpu.PREC_FP64 if precision == "fp64" else gpu.PREC_MIXED
    plan = gpu.BatchPlan(sizes, kinds, prec)
    a, b = plan.pack(mats, rhs)
    x, info, iters, berr = plan.solve(a, b)
    assert (info == 0).all(), info
    xs = plan.unpack(x)
    for i, (m, r, k) in enumerate(zip(mats, rhs, kinds)):
        n = sizes[i]
        assert backward_error(m, xs[i], r) <= n * U64 * 10, (n, k)
        assert 0 <= berr[i] <= n * U64 * 10
        xo, st = oracle_solve(m, r, k)
        assert np.max(np.abs(xs[i] - xo)) <= 1e-12 * max(np.max(np.abs(xo)), 1e-300) * n, (n, k)
        if precision == "mixed":
            assert iters[i] >= 1
    plan.close()


def test_batch_f32(gpu):
    rng = np.random.default_rng(9)
    sizes = EDGE_SIZES
    kinds = [i % 2 for i in range(len(sizes))]
    mats, rhs = make_batch(rng, sizes, kinds)
    plan = gpu.BatchPlan(sizes, kinds, gpu.PREC_FP32)
    a, b = plan.pack(mats, rhs)
    x, info, iters, berr = plan.solve(a, b)
    assert (info == 0).all()
    xs = plan.unpack(x)
    for i, (m, r) in enumerate(zip(mats, rhs)):
        n = sizes[i]
        m32, r32 = m.astype(np.float32), r.astype(np.float32)
        assert xs[i].dtype == np.float32
        assert backward_error(m32, xs[i], r32) <= n * U32 * 10


def test_batch_failures_and_fallback(gpu):
    """Singular / indefinite systems report the reference's errors; an ill-conditioned
    SPD system (Hilbert 12, kappa ~ 1e16) cannot be refined from an FP32 factor and is
    solved by the FP64 fallback pass (iters = -1) with the same result as the FP64 plan."""
    rng = np.random.default_rng(4)
    sing = rng.uniform(-1, 1, (6, 6))
    sing[:, 2] = 0.0
    indef = np.diag([1.0, -2.0, 3.0])
    hilb = 1.0 / (np.arange(12)[:, None] + np.arange(12)[None, :] + 1.0)
    good = rng.uniform(-1, 1, (10, 10)) + 10 * np.eye(10)
    mats = [sing, indef, hilb, good]
    kinds = [0, 1, 1, 0]
    sizes = [m.shape[0] for m in mats]
    rhs = [rng.standard_normal(n) for n in sizes]
    res = {}
    for name, prec in (("fp64", gpu.PREC_FP64), ("mixed", gpu.PREC_MIXED)):
        plan = gpu.BatchPlan(sizes, kinds, prec)
        a, b = plan.pack(mats, rhs)
        x, info, iters, berr = plan.solve(a, b)
        assert info[0] == 4, "DivByZero (lu.rs:179-183)"
        assert info[1] == 2, "DecompFailure (cholesky.rs:155-158)"
        assert info[2] == 0 and info[3] == 0
        if name == "mixed":
            assert iters[2] == -1, "the FP32 factor cannot refine kappa ~ 1e16: FP64 fallback"
            assert iters[3] >= 1
        res[name] = plan.unpack(x)
    assert np.array_equal(res["fp64"][2], res["mixed"][2])
    assert backward_error(hilb, res["mixed"][2], rhs[2]) <= 12 * U64 * 10


def test_batch_empty_and_zero_size(gpu):
    plan = gpu.BatchPlan([0, 3], [0, 1], gpu.PREC_MIXED)
    a, b = plan.pack([np.zeros((0, 0)), 4 * np.eye(3)], [np.zeros(0), np.ones(3)])
    x, info, _, _ = plan.solve(a, b)
    assert (info == 0).all() and np.allclose(plan.unpack(x)[1], 0.25)
    empty = gpu.BatchPlan([], [], gpu.PREC_FP64)
    x, info, _, _ = empty.solve(np.zeros(0), np.zeros(0))
    assert len(info) == 0
    with pytest.raises(gpu.RulinalgError):
        gpu.BatchPlan([513], [0], gpu.PREC_FP64)  # one CTA holds n <= 512


def test_batch_deterministic_and_device_api(gpu):
    """Two launches give bitwise identical results; the device-pointer entry point agrees
    with the host one."""
    import torch
    rng = np.random.default_rng(12)
    sizes = list(rng.integers(1, 300, 200))
    kinds = list(rng.integers(0, 2, 200))
    mats, rhs = make_batch(rng, sizes, kinds)
    plan = gpu.BatchPlan(sizes, kinds, gpu.PREC_MIXED)
    a, b = plan.pack(mats, rhs)
    x1, info1, it1, be1 = plan.solve(a, b)
    x2, info2, it2, be2 = plan.solve(a, b)
    assert np.array_equal(x1, x2) and np.array_equal(it1, it2)
    dev = torch.device("cuda:0")
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    tx = torch.zeros_like(tb)
    ti = torch.zeros(len(sizes), dtype=torch.int32, device=dev)
    plan.solve_dev(ta.data_ptr(), tb.data_ptr(), tx.data_ptr(), ti.data_ptr(),
                   stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(tx.cpu().numpy(), x1)
    assert (ti.cpu().numpy() == 0).all()


def _by_size(n, a_h, b_h, x, idx_filter=None):
    """Per size group: (indices, A blocks k x n x n, b k x n, x k x n) of a packed batch."""
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
    sel = np.arange(len(n)) if idx_filter is None else idx_filter
    for size in np.unique(n[sel]):
        idx = sel[n[sel] == size]
        k = int(size)
        ab = np.stack([a_h[a_off[i]:a_off[i + 1]] for i in idx]).reshape(len(idx), k, k)
        bb = np.stack([b_h[b_off[i]:b_off[i + 1]] for i in idx])
        xb = np.stack([x[b_off[i]:b_off[i + 1]] for i in idx])
        yield idx, ab, bb, xb


def host_berr(ab, bb, xb):
    """||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf) per system, in FP64 on the host."""
    r = bb - np.einsum("kij,kj->ki", ab, xb)
    an = np.max(np.sum(np.abs(ab), 2), 1)
    return np.max(np.abs(r), 1) / (an * np.max(np.abs(xb), 1) + np.max(np.abs(bb), 1))


def kappa_inf(ab):
    """||A||_inf ||A^-1||_inf of each matrix of a k x n x n stack."""
    an = np.max(np.sum(np.abs(ab), 2), 1)
    return an * np.max(np.sum(np.abs(np.linalg.inv(ab)), 2), 1)


def test_config4_full_size(gpu):
    """The full batched mix (20,000 SPD + 20,000 general, n log-uniform in [8, 512]),
    every system compared with the oracle: the oracle (PartialPivLu / Cholesky decompose
    + solve restated from lu.rs:163-244 and cholesky.rs:116-202) solves all 40,000 on all
    host threads; every backward error is recomputed on the host in FP64; every
    solution's forward error against the oracle's is within the bound that the two
    backward errors give, 2 kappa_inf (eta_gpu + eta_oracle) / (1 - kappa_inf eta), with
    each system's kappa_inf = ||A||_inf ||A^-1||_inf from a batched inverse on the host
    (up to ~130 for the SPD systems, ~3 for the general ones)."""
    import torch
    from rulinalg_gb300.workloads import mixed_batch
    dev = torch.device("cuda:0")
    n, kind, a, b = mixed_batch(20000, 20000, seed=0, device=dev)
    count = len(n)
    out = {}
    for name, prec in (("mixed", gpu.PREC_MIXED), ("fp64", gpu.PREC_FP64)):
        plan = gpu.BatchPlan(n, kind, prec)
        x = torch.zeros_like(b)
        info = torch.zeros(count, dtype=torch.int32, device=dev)
        iters = torch.zeros(count, dtype=torch.int32, device=dev)
        berr = torch.zeros(count, dtype=torch.float64, device=dev)
        plan.solve_dev(a.data_ptr(), b.data_ptr(), x.data_ptr(), info.data_ptr(), iters.data_ptr(),
                       berr.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        out[name] = (x.cpu().numpy(), info.cpu().numpy(), iters.cpu().numpy(), berr.cpu().numpy())
        plan.close()
    xm, im, itm, bm = out["mixed"]
    xf, if_, _, bf = out["fp64"]
    assert (im == 0).all() and (if_ == 0).all()
    limit = n.astype(np.float64) * U64 * 10
    assert (bm <= limit).all(), float(np.max(bm / limit))
    assert (bf <= limit).all()
    print(f"mixed: max berr {bm.max():.3e}, iters hist {np.bincount(itm + 1)}; fp64 max berr {bf.max():.3e}")
    # the oracle on every system (a and b consumed: copies)
    a_h = a.cpu().numpy()
    b_h = b.cpu().numpy()
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
    xo = b_h.copy()
    oinfo = O.batch_solve(n, kind, a_off[:-1], a_h.copy(), b_off[:-1], xo, threads=os.cpu_count() or 1)
    assert (oinfo == O.OK).all()
    worst_fe, worst_ratio, worst_host = 0.0, 0.0, 0.0
    for idx, ab, bb, xb in _by_size(n, a_h, b_h, xm):
        hb = host_berr(ab, bb, xb)
        k = int(n[idx[0]])
        assert np.all(hb <= k * U64 * 10), (k, hb.max())
        # device-reported backward errors are the solutions' own (two FP64 evaluations of
        # a residual at the rounding floor differ by up to ~sqrt(n) u relative)
        slack = 4 * np.sqrt(k) * U64
        assert np.all(bm[idx] <= 10 * hb + slack) and np.all(hb <= 10 * bm[idx] + slack)
        xob = np.stack([xo[b_off[i]:b_off[i + 1]] for i in idx])
        ho = host_berr(ab, bb, xob)
        fe = np.max(np.abs(xb - xob), 1) / np.max(np.abs(xob), 1)
        bound = 2 * kappa_inf(ab) * (hb + ho)
        worst_fe = max(worst_fe, float(fe.max()))
        worst_ratio = max(worst_ratio, float(np.max(fe / bound)))
        worst_host = max(worst_host, float(np.max(hb / (k * U64 * 10))))
        assert np.all(fe <= bound), (k, np.max(fe / bound))
    print(f"all {count} systems vs the oracle: max forward error {worst_fe:.3e}, max fe / bound {worst_ratio:.3f}, "
          f"max host berr / limit {worst_host:.3f}")
    assert np.max(np.abs(xm - xf)) <= 1e-10 * np.max(np.abs(xf))


def test_config4_spd_f32(gpu):
    """The f32 half of the SPD set: the 20,000 Cholesky systems as Matrix<f32> through
    an RL_PREC_FP32 plan: every system's host-computed backward error within
    n 2^-24 10 and its solution within the FP32 forward-error bound of the f64 oracle's
    solution of the same f32 system."""
    from rulinalg_gb300.workloads import mixed_batch
    n, kind, a, b = mixed_batch(20000, 0, seed=0, dtype=np.float32)
    plan = gpu.BatchPlan(n, kind, gpu.PREC_FP32)
    x, info, iters, berr = plan.solve(a, b)
    plan.close()
    assert (info == 0).all()
    a64, b64 = a.astype(np.float64), b.astype(np.float64)
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
    xo = b64.copy()
    oinfo = O.batch_solve(n, kind, a_off[:-1], a64.copy(), b_off[:-1], xo, threads=os.cpu_count() or 1)
    assert (oinfo == O.OK).all()
    worst = 0.0
    for idx, ab, bb, xb in _by_size(n, a64, b64, x.astype(np.float64)):
        k = int(n[idx[0]])
        hb = host_berr(ab, bb, xb)
        assert np.all(hb <= k * U32 * 10), (k, hb.max())
        xob = np.stack([xo[b_off[i]:b_off[i + 1]] for i in idx])
        fe = np.max(np.abs(xb - xob), 1) / np.max(np.abs(xob), 1)
        assert np.all(fe <= 2 * kappa_inf(ab) * (hb + host_berr(ab, bb, xob)))
        worst = max(worst, float(fe.max()))
    print(f"f32 SPD half: max berr {berr.max():.3e}, max forward error vs f64 oracle {worst:.3e}")


def test_autotune_no_slower_than_defaults_and_cached(gpu, tmp_path):
    """The autotuner times candidate launch shapes / size classes and keeps one no slower
    than the defaults; a second call on a batch of the same shape comes from the cache;
    the tuned plan still solves every system f64-accurately."""
    import torch
    from rulinalg_gb300 import autotune
    from rulinalg_gb300.workloads import mixed_batch
    from rulinalg_gb300 import _lib as L
    saved = {k: gpu.tune_get(k) for k in (L.TUNE_BATCH_CTAS_PER_SM, L.TUNE_BATCH_WARP_COST, L.TUNE_UPLOAD_CHUNKS)}
    dev = torch.device("cuda:0")
    n, kind, a, b = mixed_batch(1500, 1500, seed=3, device=dev)
    try:
        r = autotune.tune(n, kind, gpu.PREC_MIXED, a, b, reps=2, cache=tmp_path / "tune.json")
        assert not r["cached"] and r["ms"] <= r["default_ms"] and len(r["trials"]) >= 5
        print(f"autotune: {r['choice']} {r['ms']:.2f} ms (defaults {r['default_ms']:.2f} ms)")
        r2 = autotune.tune(n, kind, gpu.PREC_MIXED, a, b, cache=tmp_path / "tune.json")
        assert r2["cached"] and r2["choice"] == r["choice"]
        plan = gpu.BatchPlan(n, kind, gpu.PREC_MIXED)
        x = torch.zeros_like(b)
        info = torch.zeros(len(n), dtype=torch.int32, device=dev)
        berr = torch.zeros(len(n), dtype=torch.float64, device=dev)
        plan.solve_dev(a.data_ptr(), b.data_ptr(), x.data_ptr(), info.data_ptr(), 0, berr.data_ptr(),
                       torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        plan.close()
        assert bool((info == 0).all())
        assert bool((berr.cpu() <= torch.from_numpy(n.astype(np.float64) * U64 * 10)).all())
    finally:
        for k, v in saved.items():
            gpu.tune_set(k, v)
