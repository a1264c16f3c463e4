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
