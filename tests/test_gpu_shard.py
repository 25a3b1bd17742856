"""The sharded Lloyd through the C-ABI (kmgb_shard_partials / kmgb_shard_update) on one GPU: two
shards of the rows in two handles of one process, their partials added in shard order (what the
ranks of a multi-GPU run exchange), against the oracle's loop with the host-streamed tiles'
update order and tiles equal to the shards: labels and centers bit for bit, SSE to 1e-10, in the
FP32 and split BF16 tiers; and against the library's own streamed handle."""
import numpy as np
import pytest

from kmeans_gb300.shard import LibraryShard, lloyd_sharded, lloyd_sharded_device
from kmeans_gb300.synthetic import mixture_numpy, sample_init

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tier_name", ["fp32", "bf16x3"])
def test_two_shards_equal_tiled_oracle(km, orc, torch_cuda, tier_name):
    tier = {"fp32": km.ASSIGN_FP32, "bf16x3": km.ASSIGN_BF16X3}[tier_name]
    n, d, k, iters = 60_000, 40, 96, 6
    X, _, _ = mixture_numpy(n, d, k, seed=51)
    init = X[sample_init(n, k, seed=52)].copy()
    half = n // 2
    shards = [LibraryShard(X[:half], k, init, tier), LibraryShard(X[half:], k, init, tier)]
    res = lloyd_sharded(shards, k, d, iters)
    st, cen, lab, sse, it = orc.lloyd_tiled(X, init, iters, tile_rows=half)
    assert res.iterations == it and res.status == st
    for sh in shards:  # an empty cluster is 0/0 = NaN in both
        assert np.array_equal(sh.centers(), cen, equal_nan=True)
        assert np.array_equal(np.isnan(sh.centers()), np.isnan(cen))
    labels = np.concatenate([sh.labels() for sh in shards])
    assert np.array_equal(labels, lab)
    assert np.allclose(res.sse, sse, rtol=1e-10, atol=0)
    # the library's own host-streamed run with the same tiles gives the same centers
    one = km.lloyd(X, k, init=init, max_iters=iters, assign_tier=tier, stream_tile_rows=half)
    assert np.array_equal(one.centers, cen, equal_nan=True) and np.array_equal(one.labels, lab)
    for sh in shards:
        sh.close()


def test_shard_partials_device_buffers(km, torch_cuda):
    """Partials written straight into device tensors (what a NCCL exchange uses) equal the host
    copies."""
    torch = torch_cuda
    n, d, k = 20_000, 16, 32
    X, _, _ = mixture_numpy(n, d, k, seed=53)
    init = X[sample_init(n, k, seed=54)].copy()
    sh = LibraryShard(X, k, init)
    S, c, Q = sh.h.shard_partials()
    Sd = torch.empty(k * d, dtype=torch.float64, device="cuda")
    cd = torch.empty(k, dtype=torch.int32, device="cuda")
    Qd = torch.empty(k, dtype=torch.float64, device="cuda")
    sh.h.shard_partials(Sd, cd, Qd)
    assert np.array_equal(Sd.cpu().numpy(), S) and np.array_equal(cd.cpu().numpy(), c)
    assert np.array_equal(Qd.cpu().numpy(), Q)
    assert c.sum() == n
    sh.close()


def test_device_exchange_path_equals_host_path(km, torch_cuda):
    """The exchange kept on the device (what the bench's multi-GPU run uses) gives the host path's
    centers and SSE bit for bit."""
    n, d, k, iters = 30_000, 24, 48, 5
    X, _, _ = mixture_numpy(n, d, k, seed=55)
    init = X[sample_init(n, k, seed=56)].copy()
    a = LibraryShard(X, k, init)
    b = LibraryShard(X, k, init)
    ra = lloyd_sharded([a], k, d, iters)
    rb = lloyd_sharded_device(b, k, d, iters)
    assert np.array_equal(ra.sse, rb.sse)
    assert np.array_equal(a.centers(), b.centers(), equal_nan=True)
    assert np.array_equal(a.labels(), b.labels())
    a.close()
    b.close()
