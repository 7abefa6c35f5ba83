"""Seeded synthetic workloads of the benchmark configurations (device tensors).

headline(): the single large distribution's three shapes -- uniform(0,1] on a 2^-24 grid,
    Zipf-like (i+1)^-1.1 randomly permuted, log-normal(0, 2).
precision(): log-normal(0, 3) with 1% forced to 0 and 0.01% scaled by 1e6.
batched(): 4096 distributions, N_d = floor(exp(U(ln 64, ln 2^20))), each uniform(0,1] or
    Zipf s=1.1 (permuted) by a seeded coin, S_d proportional to N_d with a fixed total.
served(): a request stream -- Poisson arrivals, N log-uniform in [256, 2^22] log-normal
    (sigma = 1.5) weights, S log-uniform in [1, 65536], a share of requests reusing the table
    of a recent request by id.  Weights are slices of one device pool of i.i.d. log-normal
    weights (the same slice for the same table id), so no request payload is generated
    inside a timed region.
"""
from __future__ import annotations

import numpy as np


def _pad(x, a=32):
    return (x + a - 1) // a * a


HEADLINE_SEEDS = (2, 3, 4)   # uniform, Zipf-like, log-normal
PRECISION_SEED = 5


def headline(dist: int, n: int, seed: int, dev):
    """Weights of shape `dist` (0 uniform(0,1]: ((x >> 40) + 1) * 2^-24, 1 Zipf-like permuted,
    2 log-normal(0, 2)), generated on the device with PyTorch's Philox generator."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    if dist == 0:
        x = torch.randint(0, 1 << 24, (n,), generator=g, device=dev, dtype=torch.int64)
        return ((x + 1).to(torch.float64) * 2.0 ** -24).to(torch.float32)
    if dist == 1:
        w = torch.arange(1, n + 1, device=dev, dtype=torch.float64).pow(-1.1).to(torch.float32)
        return w[torch.randperm(n, generator=g, device=dev)]
    z = torch.randn(n, generator=g, device=dev, dtype=torch.float32)
    return torch.exp(2.0 * z)


def precision(n: int, dev, seed: int = PRECISION_SEED):
    """log-normal(0, 3) weights with 1% forced to 0 and 0.01% scaled by 1e6 (device)."""
    import torch
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    w = torch.exp(3.0 * torch.randn(n, generator=g, device=dev, dtype=torch.float32))
    w[torch.rand(n, generator=g, device=dev) < 0.01] = 0.0
    big = torch.rand(n, generator=g, device=dev) < 1e-4
    w[big] = (w[big].double() * 1e6).float()
    return w


def batched(dev, n_dists: int = 4096, log2_s: int = 30, seed: int = 6,
            n_min: int = 64, n_max: int = 1 << 20) -> dict:
    import torch
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(float(n_min)), np.log(float(n_max)), n_dists)))
    sizes = sizes.astype(np.int64)
    zipf = rng.random(n_dists) < 0.5
    total_s = 1 << log2_s
    counts = np.floor(sizes * (total_s / sizes.sum())).astype(np.int64)
    counts[np.argmax(sizes)] += total_s - counts.sum()
    w_off = np.concatenate([[0], np.cumsum(_pad(sizes))])
    s_off = np.concatenate([[0], np.cumsum(_pad(counts))])
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    w = torch.empty(int(w_off[-1]), dtype=torch.float32, device=dev)
    x = torch.randint(0, 1 << 24, (int(w_off[-1]),), generator=g, device=dev, dtype=torch.int64)
    w.copy_(((x + 1).to(torch.float64) * 2.0 ** -24).to(torch.float32))
    del x
    for d in np.nonzero(zipf)[0]:
        n = int(sizes[d])
        z = torch.arange(1, n + 1, device=dev, dtype=torch.float64).pow(-1.1).to(torch.float32)
        w[int(w_off[d]):int(w_off[d]) + n] = z[torch.randperm(n, generator=g, device=dev)]
    return {"sizes": sizes, "counts": counts, "zipf": zipf, "w_off": w_off, "s_off": s_off,
            "w": w}


def served(dev, n_requests: int = 200_000, rate: float = 50_000.0, seed: int = 7,
           n_min: int = 256, n_max: int = 1 << 22, s_max: int = 65536, reuse: float = 0.3,
           recent: int = 2048, pool_log2: int = 28, sigma: float = 1.5) -> dict:
    """Request i: table id, n, s, seed, arrival time, and the pool offset of its weights."""
    import torch
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    arrivals -= arrivals[0]
    n_new = np.floor(np.exp(rng.uniform(np.log(float(n_min)), np.log(float(n_max) + 1.0),
                                        n_requests))).astype(np.int64)
    n_new = np.minimum(n_new, n_max)
    s = np.floor(np.exp(rng.uniform(0.0, np.log(float(s_max) + 1.0), n_requests))).astype(np.int64)
    s = np.clip(s, 1, s_max)
    reuse_draw = rng.random(n_requests) < reuse
    back = rng.integers(1, recent + 1, n_requests)
    table_id = np.arange(n_requests, dtype=np.int64)
    for i in range(n_requests):
        if reuse_draw[i] and i > 0:
            table_id[i] = table_id[max(0, i - int(back[i]))]
    n = n_new[table_id]
    pool = 1 << pool_log2
    off = (rng.integers(0, pool - n_max, n_requests) // 32 * 32)[table_id]
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    w = torch.exp(sigma * torch.randn(pool, generator=g, device=dev, dtype=torch.float32))
    s_off = np.concatenate([[0], np.cumsum(_pad(s))])
    return {"arrivals": arrivals, "table_id": table_id, "n": n, "s": s, "w_off": off,
            "s_off": s_off, "w": w, "seeds": np.arange(n_requests, dtype=np.int64) + 1000}
