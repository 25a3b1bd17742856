"""Seeded synthetic Gaussian-mixture workloads with the shapes of the benchmark configurations.

The reference's own test matrices (SIFT 898790x128, HOG 796160x324, read from files that are
not shipped) are replaced by these generators. Each returns float32 points, the generating
component of every point, and the component means.

Configurations (points x dims, centers):
  c1  100,000 x 32,   K=64     isotropic sigma=1, equal weights, means U[-10,10]^D
  c2  4,000,000 x 128, K=1024  diagonal std log-U[0.3,3] per component, means U[-20,20]^D
  c3  200,000,000 x 96, K=4096 sigma=1.5, means U[-15,15]^D
  c4  16,000,000 x 256, K=65536 Zipf(1.1) sizes, sigma=1, means N(0, 25 I)
"""
from __future__ import annotations

import numpy as np

CONFIGS = {
    "c1": dict(n=100_000, d=32, k=64, iters=20, mean_lo=-10.0, mean_hi=10.0, std=(1.0, 1.0)),
    "c2": dict(n=4_000_000, d=128, k=1024, iters=30, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0)),
    "c3": dict(n=200_000_000, d=96, k=4096, iters=10, mean_lo=-15.0, mean_hi=15.0, std=(1.5, 1.5)),
}


def mixture_numpy(n: int, d: int, k: int, seed: int = 0, mean_lo: float = -10.0,
                  mean_hi: float = 10.0, std=(1.0, 1.0), zipf: float = 0.0):
    """Host (numpy) generator; `std` = (lo, hi): per-component, per-dimension std drawn
    log-uniform in [lo, hi] (lo == hi: isotropic)."""
    rng = np.random.default_rng(seed)
    means = rng.uniform(mean_lo, mean_hi, size=(k, d)).astype(np.float32)
    if std[0] == std[1]:
        stds = np.full((k, d), std[0], dtype=np.float32)
    else:
        stds = np.exp(rng.uniform(np.log(std[0]), np.log(std[1]), size=(k, d))).astype(np.float32)
    if zipf > 0:
        w = 1.0 / np.arange(1, k + 1) ** zipf
        comp = rng.choice(k, size=n, p=w / w.sum()).astype(np.int32)
    else:
        comp = rng.integers(0, k, size=n, dtype=np.int32)
    X = rng.standard_normal((n, d), dtype=np.float32)
    X *= stds[comp]
    X += means[comp]
    return X, comp, means


def mixture_torch(n: int, d: int, k: int, seed: int = 0, mean_lo: float = -10.0,
                  mean_hi: float = 10.0, std=(1.0, 1.0), device="cuda", chunk: int = 1 << 22):
    """Device (torch) generator for the large configurations; deterministic for a seed on a
    given GPU type."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    means = torch.empty((k, d), device=device).uniform_(mean_lo, mean_hi, generator=g)
    if std[0] == std[1]:
        stds = torch.full((k, d), float(std[0]), device=device)
    else:
        lo, hi = float(np.log(std[0])), float(np.log(std[1]))
        stds = torch.empty((k, d), device=device).uniform_(lo, hi, generator=g).exp_()
    X = torch.empty((n, d), device=device, dtype=torch.float32)
    comp = torch.empty(n, device=device, dtype=torch.int32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        c = torch.randint(0, k, (e - s,), device=device, generator=g)
        z = torch.randn((e - s, d), device=device, generator=g)
        X[s:e] = z * stds[c] + means[c]
        comp[s:e] = c.to(torch.int32)
    return X, comp, means


def zipf_blobs_numpy(n: int, d: int, k: int, seed: int = 0, s: float = 1.1, sigma: float = 1.0,
                     mean_std: float = 5.0, bf16: bool = True):
    """The c4 shape at any size: k isotropic Gaussians (sigma) with Zipf(s) sizes around means
    drawn from N(0, mean_std^2 I); values rounded to BF16 numbers when bf16 is set."""
    rng = np.random.default_rng(seed)
    w = 1.0 / np.arange(1, k + 1) ** s
    comp = rng.choice(k, size=n, p=w / w.sum()).astype(np.int32)
    means = (rng.standard_normal((k, d)) * mean_std).astype(np.float32)
    X = rng.standard_normal((n, d), dtype=np.float32) * np.float32(sigma)
    X += means[comp]
    if bf16:  # round to nearest even BF16 through the bit pattern
        b = X.view(np.uint32)
        b += np.uint32(0x7FFF) + ((b >> 16) & np.uint32(1))
        b &= np.uint32(0xFFFF0000)
    return X, comp, means


def sample_init(n: int, k: int, seed: int = 1) -> np.ndarray:
    """k distinct row indices chosen uniformly by seed (initial centers = those rows)."""
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=k, replace=False)).astype(np.int64)
