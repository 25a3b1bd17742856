"""Sharded Lloyd: the rows partitioned over ranks (one GPU per rank), one exchange per iteration.

The reference runs on one GPU (main/cpp/kmeans.cpp:1185-1247). Its iteration shards by rows:
the assignment of a row needs only the centers, and the update and compactness
(kmeans.cpp:1018-1104) need only per-cluster sums. Every rank therefore

  1. assigns its rows to the current centers and forms the canonical FP64 sums of its rows per
     cluster -- S (k x d), counts (k), Q (k, sums of ||x||^2) -- (kmgb_shard_partials),
  2. all-gathers every rank's partials and adds them in rank order in FP64
     (0 + P_0 + P_1 + ...; a gather, not an all-reduce, so the order of the additions is fixed),
  3. turns the totals into the new centers and the SSE (kmgb_shard_update), the same on every
     rank, and evaluates the reference's stop rule (relErr = |SSE - SSE_old| / |SSE|) on the same
     numbers, so all ranks stop together.

The result is the single-GPU run whose rows are streamed in tiles equal to the shards (the
library's host-streamed path adds tile sums to its totals in the same order), bit for bit for
labels and centers. Exchanged bytes per iteration and rank: (k d + 2 k) x 8.

A shard backend has partials() -> (S, counts, Q) and update(S, counts, Q) -> SSE; LibraryShard
is the GPU one. The communication goes through torch.distributed (NCCL between GPUs, gloo on
CPUs) when a process group is given.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np


class LibraryShard:
    """One shard of rows in a resident handle of the library (the rank's GPU)."""

    def __init__(self, X, k: int, init: np.ndarray, assign_tier: int = 0, empty_policy: int = 0):
        import kmeans_gb300 as km
        n, d = X.shape
        self.k, self.d = k, d
        self.h = km.Handle(n, d, k, assign_tier=assign_tier, empty_policy=empty_policy,
                           max_iters=1)
        self.h.set_data(X, not isinstance(X, np.ndarray))
        self.h.set_centers(np.ascontiguousarray(init, dtype=np.float32), False)

    def partials(self):
        return self.h.shard_partials()

    def update(self, S, counts, Q) -> float:
        return self.h.shard_update(S, counts, Q)

    def centers(self) -> np.ndarray:
        return self.h.centers()

    def labels(self) -> np.ndarray:
        return self.h.labels()

    def close(self):
        self.h.close()


def gather_sum(vec: np.ndarray, dist=None) -> np.ndarray:
    """Every rank's vector (same length), summed in rank order starting from zero, on every rank."""
    total = np.zeros_like(vec, dtype=np.float64)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        total += vec
        return total
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.from_numpy(np.ascontiguousarray(vec, dtype=np.float64)).to(device)
    parts = [torch.empty_like(t) for _ in range(dist.get_world_size())]
    dist.all_gather(parts, t)
    for p in parts:
        total += p.cpu().numpy()
    return total


@dataclass
class ShardedResult:
    status: int
    iterations: int
    sse: np.ndarray
    exchanged_bytes_per_iteration: int


def lloyd_sharded(shards: Sequence, k: int, d: int, max_iters: int, criterion: float = -1.0,
                  dist=None) -> ShardedResult:
    """Lloyd iterations over this rank's shards (usually one; several are summed in list order
    before the exchange, as consecutive ranks would be) and the other ranks' through `dist`.
    Returns the status (0, or 13 = KMEANS_NONCONVERGENCE when relErr > criterion at exit), the
    iterations run and the SSE of every iteration."""
    sse_hist: List[float] = []
    sse_old, rel, it = 0.0, 1.0, 0
    kd = k * d
    while it < max_iters and rel > criterion:
        local = np.zeros(kd + 2 * k, np.float64)
        for sh in shards:
            S, n, Q = sh.partials()
            local += np.concatenate([np.asarray(S, np.float64).ravel(),
                                     np.asarray(n, np.float64), np.asarray(Q, np.float64)])
        tot = gather_sum(local, dist)
        S_t = np.ascontiguousarray(tot[:kd])
        n_t = np.ascontiguousarray(tot[kd:kd + k].astype(np.int32))
        Q_t = np.ascontiguousarray(tot[kd + k:])
        sse = None
        for sh in shards:  # every shard of every rank computes the same centers and SSE
            sse = sh.update(S_t, n_t, Q_t)
        rel = abs(sse - sse_old) / abs(sse) if sse != 0 else float("nan")
        sse_old = sse
        sse_hist.append(sse)
        it += 1
    status = 0 if rel <= criterion else 13
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    return ShardedResult(status, it, np.array(sse_hist), world * (kd + 2 * k) * 8)


def lloyd_sharded_device(shard: "LibraryShard", k: int, d: int, max_iters: int,
                         criterion: float = -1.0, dist=None) -> ShardedResult:
    """lloyd_sharded for one LibraryShard per rank with the exchange on the GPU: the partials are
    written into a device buffer, all-gathered (NCCL) and added in rank order by FP64 element-wise
    additions on the device (the same numbers as the host path), so no partial crosses the host
    link."""
    import torch
    kd = k * d
    world = dist.get_world_size() if dist is not None and dist.is_initialized() else 1
    buf = torch.empty(kd + 2 * k, dtype=torch.float64, device="cuda")
    S, Q = buf[:kd], buf[kd + k:]
    cnt = torch.empty(k, dtype=torch.int32, device="cuda")
    parts = [torch.empty_like(buf) for _ in range(world)] if world > 1 else None
    tot = torch.empty_like(buf)
    sse_hist: List[float] = []
    sse_old, rel, it = 0.0, 1.0, 0
    while it < max_iters and rel > criterion:
        shard.h.shard_partials(S, cnt, Q)  # returns once its stream is done
        buf[kd:kd + k] = cnt.double()
        tot.zero_()
        if parts is not None:
            dist.all_gather(parts, buf)
            for p in parts:
                tot += p
        else:
            tot += buf
        n_t = tot[kd:kd + k].to(torch.int32)
        torch.cuda.current_stream().synchronize()  # the handle's stream reads these next
        sse = shard.h.shard_update(tot[:kd], n_t, tot[kd + k:])
        rel = abs(sse - sse_old) / abs(sse) if sse != 0 else float("nan")
        sse_old = sse
        sse_hist.append(sse)
        it += 1
    status = 0 if rel <= criterion else 13
    return ShardedResult(status, it, np.array(sse_hist), world * (kd + 2 * k) * 8)
