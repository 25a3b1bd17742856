"""The sharded Lloyd driver (kmeans_gb300/shard.py) with CPU processes as ranks (gloo on
127.0.0.1): every rank holds a contiguous range of the rows and an oracle shard (the CPU
restatement's assignment and canonical FP64 per-cluster sums, test infrastructure), the ranks
exchange their partials once per iteration and add them in rank order. The result must equal the
oracle's single-process loop with the host-streamed tiles' update order and tiles equal to the
shards: labels and centers bit for bit, the SSE to FP64 rounding (identity form here, direct form
there), iterations and status equal -- whatever the number of ranks."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class OracleShard:
    """Test stand-in for kmeans_gb300.shard.LibraryShard on the CPU."""

    def __init__(self, X, k, init, empty_policy=0):
        import oracle
        self.orc = oracle
        self.X, self.k, self.d = X, k, X.shape[1]
        self.C = np.array(init, dtype=np.float32)
        self.empty_policy = empty_policy
        self.lab = None

    def partials(self):
        self.lab = self.orc.assign(self.X, self.C)
        _, cnt, sums = self.orc.update(self.X, self.lab, self.k)
        x64 = self.X.astype(np.float64)
        Q = np.bincount(self.lab, weights=(x64 * x64).sum(1), minlength=self.k)
        return sums.ravel(), cnt, Q

    def update(self, S, n, Q):
        S = np.asarray(S, np.float64).reshape(self.k, self.d)
        n = np.asarray(n)
        mu = np.empty_like(self.C)
        for j in range(self.k):
            if n[j] > 0:
                mu[j] = (S[j] / float(n[j])).astype(np.float32)
            elif self.empty_policy == 1:
                mu[j] = self.C[j]
            else:
                mu[j] = np.nan
        self.C = mu
        used = n > 0
        m64 = mu.astype(np.float64)
        return float(np.sum(Q[used] - 2.0 * (m64[used] * S[used]).sum(1)
                            + n[used] * (m64[used] * m64[used]).sum(1)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, X, init, k, iters, criterion, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from kmeans_gb300.shard import lloyd_sharded
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rows = np.array_split(np.arange(len(X)), world)[rank]
    sh = OracleShard(X[rows], k, init)
    res = lloyd_sharded([sh], k, X.shape[1], iters, criterion, dist)
    out.put((rank, res.status, res.iterations, res.sse, sh.C, sh.lab,
             res.exchanged_bytes_per_iteration))
    dist.barrier()
    dist.destroy_process_group()


def run_ranks(world, X, init, k, iters, criterion=-1.0):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, X, init, k, iters, criterion, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_lloyd_equals_tiled_oracle(world):
    sys.path.insert(0, ROOT)
    import oracle
    from kmeans_gb300.synthetic import mixture_numpy, sample_init
    n, d, k, iters = 6000 * world, 12, 24, 6
    X, _, _ = mixture_numpy(n, d, k, seed=40 + world)
    init = X[sample_init(n, k, seed=41)].copy()
    res = run_ranks(world, X, init, k, iters)
    st, cen, lab, sse, it = oracle.lloyd_tiled(X, init, iters, tile_rows=n // world)
    for rank, status, iterations, ssev, C, L, nbytes in res:
        assert iterations == it and status == st
        assert np.array_equal(C, cen)                       # every rank: the same centers
        assert np.allclose(ssev, sse, rtol=1e-10, atol=0)
        assert nbytes == world * (k * d + 2 * k) * 8
    labels = np.concatenate([r[5] for r in res])              # rank order = row order
    assert np.array_equal(labels, lab)


def test_sharded_stop_rule_fires_on_every_rank_together():
    sys.path.insert(0, ROOT)
    import oracle
    from kmeans_gb300.synthetic import mixture_numpy, sample_init
    n, d, k = 8000, 6, 10
    X, _, _ = mixture_numpy(n, d, k, seed=9)
    init = X[sample_init(n, k, seed=10)].copy()
    res = run_ranks(2, X, init, k, 50, criterion=1e-6)
    st, cen, lab, sse, it = oracle.lloyd_tiled(X, init, 50, tile_rows=n // 2, criterion=1e-6)
    assert it < 50
    for rank, status, iterations, ssev, C, L, _ in res:
        assert iterations == it and status == st == 0
        assert np.array_equal(C, cen)
