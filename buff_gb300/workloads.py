"""Seeded synthetic columns with the shapes and value distributions of the
benchmark configurations (none of them is a public dataset).

- ``gaussian_walk``: x0 = 1.0, steps N(0, 0.01), rounded to 4 decimals
  (1,000,000 values, scale 10^4).
- ``bounded_walk``: steps U(-0.5, 0.5) reflected into [-500, 500], rounded to
  4 decimals (268,435,456 values, scale 10^4 -> 25-bit codes, 3 slices + 1 bit).
- ``outlier_column``: 99% N(100, 5) at 6 decimals, 1% U(-1e6, 1e6) at seeded
  random positions (67,108,864 values, scale 10^6).

- ``column_set``: many random-walk columns with log-uniform lengths, each with
  its own decimals (2-6), step size and start (the batched and serving
  configurations: 4,096 columns of 1K-4M rows, 2,048 columns of 64K-16M rows).

The numpy forms are for host-sized cases; the torch forms build large columns
directly in device memory.
"""
from __future__ import annotations

import numpy as np


def gaussian_walk(n: int, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = 1.0 + np.cumsum(rng.normal(0.0, 0.01, n))
    return np.round(x, 4)


def _fold(x, lo=-500.0, hi=500.0):
    """Reflects a free walk into [lo, hi] (triangle-wave fold)."""
    span = hi - lo
    y = np.mod(x - lo, 2 * span)
    return lo + np.where(y > span, 2 * span - y, y)


def bounded_walk(n: int, seed: int = 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = np.cumsum(rng.uniform(-0.5, 0.5, n))
    return np.round(_fold(x), 4)


def outlier_column(n: int, seed: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = np.round(rng.normal(100.0, 5.0, n), 6)
    m = max(1, n // 100)
    pos = rng.choice(n, size=m, replace=False)
    x[pos] = np.round(rng.uniform(-1e6, 1e6, m), 6)
    return x


def outlier_column_torch(n: int, seed: int = 3, device="cuda"):
    """outlier_column generated on the device (float64)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    x = torch.randn(n, generator=g, device=device, dtype=torch.float64) * 5.0 + 100.0
    m = max(1, n // 100)
    pos = torch.randperm(n, generator=g, device=device)[:m]
    x[pos] = (torch.rand(m, generator=g, device=device, dtype=torch.float64) * 2 - 1) * 1e6
    return torch.round(x * 1e6) / 1e6


def high_outlier_column_torch(n: int, seed: int = 6, device="cuda"):
    """99% N(100, 5) and 1% U(1e5, 1e6) at seeded random positions, 6
    decimals, generated on the device (float64): the outliers sit above the
    bulk, so the leading code byte is zero on 99% of the rows."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    x = torch.randn(n, generator=g, device=device, dtype=torch.float64) * 5.0 + 100.0
    m = max(1, n // 100)
    pos = torch.randperm(n, generator=g, device=device)[:m]
    x[pos] = 1e5 + torch.rand(m, generator=g, device=device, dtype=torch.float64) * 9e5
    return torch.round(x * 1e6) / 1e6


def bounded_walk_torch(n: int, seed: int = 2, device="cuda"):
    """bounded_walk generated on the device (float64)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    steps = torch.rand(n, generator=g, device=device, dtype=torch.float64) - 0.5
    x = torch.cumsum(steps, 0)
    lo, span = -500.0, 1000.0
    y = torch.remainder(x - lo, 2 * span)
    y = lo + torch.where(y > span, 2 * span - y, y)
    return torch.round(y * 1e4) / 1e4


def quantile_preds(x: np.ndarray, selectivities=(0.001, 0.01, 0.1, 0.5)):
    """Predicates p with P(x > p) ~= selectivity."""
    return [float(np.quantile(x, 1.0 - s)) for s in selectivities]


def column_set(ncols: int, lo: int, hi: int, seed: int):
    """Lengths (log-uniform in [lo, hi]), decimals U{2..6}, step sizes and
    starts of a seeded set of random-walk columns."""
    rng = np.random.default_rng(seed)
    lens = np.exp(rng.uniform(np.log(lo), np.log(hi), ncols)).astype(np.int64)
    dec = rng.integers(2, 7, ncols)
    sigma = 10.0 ** rng.uniform(-2, 1, ncols)
    start = rng.uniform(-1e3, 1e3, ncols)
    return lens, dec, sigma, start


def fill_walk_torch(out, n: int, dec: int, sigma: float, start: float, seed: int):
    """Writes a random walk of n rows rounded to `dec` decimals into `out[:n]`."""
    import torch

    g = torch.Generator(device=out.device)
    g.manual_seed(seed)
    v = out[:n]
    torch.randn(n, generator=g, device=out.device, dtype=torch.float64, out=v)
    v.mul_(sigma)
    v.cumsum_(0)
    v.add_(start)
    s = 10.0 ** dec
    v.mul_(s).round_().div_(s)
    return v


def outlier_u8_torch(n: int, ratio: float = 0.9, seed: int = 8, device="cuda"):
    """outlier_exp's input on the device (float64): byte values, 69 with
    probability `ratio`, otherwise uniform in [0, 256); one 0 and one 255."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    u = torch.rand(n, generator=g, device=device, dtype=torch.float64)
    v = torch.randint(0, 256, (n,), generator=g, device=device).to(torch.float64)
    x = torch.where(u < ratio, torch.full_like(u, 69.0), v)
    x[n // 3] = 0.0
    x[2 * n // 3] = 255.0
    return x
