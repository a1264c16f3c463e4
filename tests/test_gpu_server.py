"""The serving loop: continuous batching, resident factors, admission by device-memory
footprint, Poisson replay. Each result must be the same alone and in the mix (the
batched kernel treats every system independently and deterministically, so the check is
bitwise) and f64-accurate (normwise backward error <= n 2^-53 10)."""
import numpy as np
import pytest

import oracle as O
from comparators import backward_error

pytestmark = pytest.mark.gpu
U64 = 2.0 ** -53


def system(rng, kind, n, m=None):
    if kind == 1:
        g = rng.standard_normal((n, n))
        return g @ g.T + n * np.eye(n), rng.standard_normal(n)
    if kind == 2:
        return rng.standard_normal((m, n)), rng.standard_normal(m)
    return rng.uniform(-1, 1, (n, n)) + n * np.eye(n), rng.standard_normal(n)


@pytest.fixture(scope="module")
def server(gpu):
    s = gpu.Server(workers=4)
    yield s
    s.close()


def test_same_alone_and_in_the_mix(gpu, server):
    rng = np.random.default_rng(1)
    probes = [(0, *system(rng, 0, 37)), (1, *system(rng, 1, 200)), (0, *system(rng, 0, 700)),
              (1, *system(rng, 1, 640)), (2, *system(rng, 2, 40, 80))]
    alone = []
    for kind, a, b in probes:
        t, _ = server.submit(kind, a, b)
        alone.append(server.wait(t))
    # the same requests again, in the middle of a burst of 300 others
    tickets = []
    for i in range(300):
        kind = int(rng.integers(0, 2))
        a, b = system(rng, kind, int(rng.integers(8, 300)))
        tickets.append(server.submit(kind, a, b)[0])
        if i % 60 == 30:
            for p_i, (kind2, a2, b2) in enumerate(probes):
                tickets.append((p_i, server.submit(kind2, a2, b2)[0]))
    mixed = {}
    for t in tickets:
        if isinstance(t, tuple):
            mixed.setdefault(t[0], []).append(server.wait(t[1]))
        else:
            assert server.wait(t)["status"] == 0
    for p_i, (kind, a, b) in enumerate(probes):
        base = alone[p_i]
        assert base["status"] == 0
        for r in mixed[p_i]:
            assert r["status"] == 0
            assert np.array_equal(r["x"], base["x"]), (p_i, np.max(np.abs(r["x"] - base["x"])))
        if kind in (0, 1):
            assert backward_error(a, base["x"], b) <= a.shape[0] * U64 * 10
        else:
            want = np.linalg.lstsq(a, b, rcond=None)[0]
            assert np.max(np.abs(base["x"] - want)) <= 1e-10 * np.max(np.abs(want))
    st = server.stats()
    assert st["batches"] >= 1 and st["batched_requests"] > st["batches"], st  # continuous batching happened


def test_resident_factor_resolves(gpu, server):
    rng = np.random.default_rng(2)
    a, b = system(rng, 0, 600)
    t, _ = server.submit(0, a, b, retain=True)
    r = server.wait(t)
    assert r["status"] == 0 and r["factor"] > 0
    h = r["factor"]
    lu, perm, _ = O.lu_decompose(a)
    for _ in range(3):
        b2 = rng.standard_normal(600)
        t2, _ = server.submit(3, b=b2, factor=h)
        r2 = server.wait(t2)
        assert r2["status"] == 0
        assert backward_error(a, r2["x"], b2) <= 600 * U64 * 10
        xo, _ = O.lu_solve(lu, perm, b2)
        assert np.max(np.abs(r2["x"] - xo)) <= 1e-12 * np.max(np.abs(xo)) * 600
    assert server.stats()["resident_factors"] >= 1
    server.release_factor(h)
    with pytest.raises(gpu.RulinalgError):
        server.submit(3, b=rng.standard_normal(600), factor=h)


def test_release_while_resolves_are_queued(gpu, server):
    """A factor released while re-solves against it are queued or running: every
    re-solve either completes (f64-accurate) or reports InvalidArg (the factor was gone
    by the time a worker held it); none runs on freed device memory."""
    rng = np.random.default_rng(21)
    n = 900
    a, b = system(rng, 0, n)
    t, _ = server.submit(0, a, b, retain=True)
    h = server.wait(t)["factor"]
    rhs = [rng.standard_normal(n) for _ in range(40)]
    tickets = [server.submit(3, b=r, factor=h)[0] for r in rhs]
    server.release_factor(h)
    done = failed = 0
    for tk, r in zip(tickets, rhs):
        try:
            res = server.wait(tk)
        except gpu.RulinalgError as e:
            assert e.kind == "InvalidArg"
            failed += 1
            continue
        if res["status"] == 0:
            assert backward_error(a, res["x"], r) <= n * U64 * 10
            done += 1
        else:
            assert res["status"] == 1, res  # RL_ERR_INVALID_ARG
            failed += 1
    assert done + failed == len(rhs)
    print(f"re-solves completed before the release: {done}, refused after it: {failed}")
    # the server is still healthy
    t, _ = server.submit(0, a, b)
    assert backward_error(a, server.wait(t)["x"], b) <= n * U64 * 10


def test_admission_by_footprint(gpu):
    n = 1500  # ~27 MB of footprint each
    srv = gpu.Server(hbm_budget_bytes=64 << 20, workers=4)
    try:
        rng = np.random.default_rng(3)
        sysm = [system(rng, 0, n) for _ in range(6)]
        tickets = [srv.submit(0, a, b)[0] for a, b in sysm]
        for (a, b), t in zip(sysm, tickets):
            r = srv.wait(t)
            assert r["status"] == 0
            assert backward_error(a, r["x"], b) <= n * U64 * 10
        st = srv.stats()
        assert st["bytes_peak"] <= st["bytes_budget"] == 64 << 20
        big = rng.standard_normal((3000, 3000))
        with pytest.raises(gpu.DeviceError):  # can never fit: rejected at submit
            srv.submit(0, big, np.ones(3000))
    finally:
        srv.close()


def test_poisson_replay(gpu, server):
    rng = np.random.default_rng(4)
    count, lam = 400, 4000.0
    arrivals = np.cumsum(rng.exponential(1.0 / lam, count))
    reqs, systems = [], []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(16), np.log(257))))
        kind = int(rng.choice([0, 1, 2], p=[0.5, 0.3, 0.2]))
        if kind == 2:
            a, b = system(rng, 2, n, 2 * n)
        else:
            a, b = system(rng, kind, n)
        systems.append((kind, a, b))
        reqs.append((kind, a, b, 0))
    server.reset_stats()
    res = server.replay(arrivals, reqs)
    for (kind, a, b), r in zip(systems, res):
        assert r["status"] == 0
        if kind != 2:
            assert backward_error(a, r["x"], b) <= a.shape[0] * U64 * 10
    st = server.stats()
    assert st["completed"] == count and st["p99_us"] >= st["p50_us"] > 0
    print(f"replay: {st}")


def test_backpressure_replay_arrays(gpu):
    """max_pending = 4: a burst of 200 requests arriving at once through the array replay
    (the form the served-stream benchmark uses) is partly refused with RL_ERR_BUSY; the
    refusals are counted in the statistics, and every accepted request completes
    f64-accurate into its own output buffer."""
    from rulinalg_gb300._lib import REQUEST_DTYPE
    rng = np.random.default_rng(7)
    srv = gpu.Server(workers=2, max_pending=4)
    try:
        count = 200
        systems = [system(rng, 0, int(rng.integers(300, 700))) for _ in range(count)]
        xs = [np.zeros(len(b)) for _, b in systems]
        req = np.zeros(count, dtype=REQUEST_DTYPE)
        req["kind"] = gpu.REQ_LU
        for i, (a, b) in enumerate(systems):
            req[i]["m"] = req[i]["n"] = len(b)
            req[i]["a"], req[i]["b"], req[i]["x"] = a.ctypes.data, b.ctypes.data, xs[i].ctypes.data
        res = srv.replay_arrays(np.zeros(count), req)
        busy = res["status"] == 37
        ok = res["status"] == 0
        assert busy.any() and ok.sum() >= 4 and (busy | ok).all()
        assert srv.stats()["rejected"] == busy.sum()
        for i in np.nonzero(ok)[0]:
            a, b = systems[i]
            assert backward_error(a, xs[i], b) <= len(b) * U64 * 10
            assert res["berr"][i] <= len(b) * U64 * 10
        for i in np.nonzero(busy)[0]:
            assert not xs[i].any()
    finally:
        srv.close()
