"""Seeded synthetic inputs with the shapes and value distributions of the benchmark
configurations. numpy's PCG64 (default_rng) is the generator, so the same seed gives
the same inputs on every machine."""
from __future__ import annotations

import numpy as np


def config1_lu(n: int = 1024, seed: int = 0):
    """PartialPivLu decompose + solve, f64: A_ij ~ U(-1,1) plus 1 on the diagonal,
    x_true ~ U(-1,1), b = A x_true."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1.0, 1.0, (n, n)) + np.eye(n)
    x = rng.uniform(-1.0, 1.0, n)
    return a, x, a @ x


def gemm_operands(n: int, dtype=np.float64, seed: int = 0):
    """Square GEMM operands with N(0,1) entries."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, n)).astype(dtype), rng.standard_normal((n, n)).astype(dtype)


def log_uniform_sizes(count: int, lo: int, hi: int, rng) -> np.ndarray:
    """n log-uniform in [lo, hi] (integer)."""
    n = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count))).astype(np.int64)
    return np.clip(n, lo, hi).astype(np.int32)


def mixed_batch(count_spd: int, count_lu: int, seed: int = 0, lo: int = 8, hi: int = 512, device=None,
                dtype=np.float64):
    """The batched uneven-solve mix: count_spd SPD systems A = G G^T + n I (G ~ N(0,1),
    Cholesky) followed by count_lu general systems A = U(-1,1) + n I (PartialPivLu),
    sizes log-uniform in [lo, hi], one N(0,1) right-hand side each.

    Returns (n int32, kind uint8, a packed row-major, b packed), the packing being
    consecutive n_i x n_i blocks in system order (the rl_batch_plan layout). When
    `device` is a torch CUDA device the G G^T products run there in FP64 and the arrays
    are returned as torch tensors on that device."""
    rng = np.random.default_rng(seed)
    n = np.concatenate([log_uniform_sizes(count_spd, lo, hi, rng), log_uniform_sizes(count_lu, lo, hi, rng)])
    kind = np.concatenate([np.ones(count_spd, np.uint8), np.zeros(count_lu, np.uint8)])
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
    total = int(a_off[-1])
    b = rng.standard_normal(int(b_off[-1]))
    if device is None:
        a = np.empty(total, dtype=np.float64)
    else:
        import torch
        a = torch.empty(total, dtype=torch.float64, device=device)
    for size in np.unique(n):
        size = int(size)
        for k in (1, 0):
            idx = np.nonzero((n == size) & (kind == k))[0]
            if len(idx) == 0:
                continue
            if k == 1:
                g = rng.standard_normal((len(idx), size, size))
                if device is None:
                    blk = g @ np.transpose(g, (0, 2, 1)) + size * np.eye(size)
                else:
                    gt = torch.from_numpy(g).to(device)
                    blk = torch.bmm(gt, gt.transpose(1, 2)) + size * torch.eye(size, dtype=torch.float64, device=device)
            else:
                u = rng.uniform(-1.0, 1.0, (len(idx), size, size)) + size * np.eye(size)
                blk = u if device is None else torch.from_numpy(u).to(device)
            flat = blk.reshape(len(idx), -1)
            for j, i in enumerate(idx):
                a[a_off[i]:a_off[i + 1]] = flat[j]
    if device is not None:
        b = torch.from_numpy(b).to(device)
        if dtype == np.float32:
            a, b = a.float(), b.float()
    elif dtype == np.float32:
        a, b = a.astype(np.float32), b.astype(np.float32)
    return n, kind, a, b


def haar_orthogonal(n: int, rng):
    """A Haar-distributed orthogonal matrix: QR of a Gaussian matrix with the signs of R's
    diagonal folded into Q (Mezzadri 2007)."""
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))


def conditioned_system(n: int, kappa: float, nrhs: int = 1, seed: int = 0, device=None):
    """A = U diag(sigma) V^T with U, V Haar-random orthogonal and sigma geometric from 1
    down to 1/kappa; B with nrhs N(0,1) columns. With a torch CUDA `device` the orthogonal
    factors and the product are formed there in FP64 (the n = 16384 case would take
    minutes on the host) and torch tensors are returned."""
    sigma = kappa ** (-np.arange(n) / max(n - 1, 1))
    if device is None:
        rng = np.random.default_rng(seed)
        u = haar_orthogonal(n, rng)
        v = haar_orthogonal(n, rng)
        a = (u * sigma) @ v.T
        b = rng.standard_normal((n, nrhs))
        return np.ascontiguousarray(a), np.ascontiguousarray(b)
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)

    def haar():
        q, r = torch.linalg.qr(torch.randn(n, n, dtype=torch.float64, device=device, generator=g))
        return q * torch.sign(torch.diagonal(r))
    u, v = haar(), haar()
    a = (u * torch.from_numpy(sigma).to(device)) @ v.T
    b = torch.randn(n, nrhs, dtype=torch.float64, device=device, generator=g)
    return a.contiguous(), b.contiguous()
