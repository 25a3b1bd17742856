"""The allocation-free ClusterCentersF variant (ClusterCentersF_noalloc) against the allocating
entry point, through the C-ABI.

Some callers cannot let a library allocate device memory: they reserve all of it up front and
forbid allocation afterwards, or their memory pool owns the whole GPU. For them the variant takes
its working memory from a static 8 MiB device array. This file runs last (pytest collects it
last), so a failure here leaves every other result in place. It must pass alone in a fresh process
and after the other tests; it calls the variant twice in a row, so the second call also shows that
the array's leftover contents from the first call do not leak into the result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(km, torch, fn, X, lab, k, tiles):
    m, d = X.shape
    Xt = torch.from_numpy(X).cuda()
    lt = torch.from_numpy(lab).cuda()
    big = torch.zeros(k * d * 2, dtype=torch.float32, device="cuda")
    cnt_big = torch.zeros(k, dtype=torch.int32, device="cuda")
    cen = torch.zeros((k, d), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(k, dtype=torch.int32, device="cuda")
    bounds = np.linspace(0, m, tiles + 1).astype(int)
    for t in range(tiles):
        a, b = int(bounds[t]), int(bounds[t + 1])
        rc = fn(a, b - a, d, k, t == tiles - 1, Xt[a:b], lt, big, cnt_big, cen, cnt)
        assert rc == 0, km.last_error()
    torch.cuda.synchronize()
    return cen.cpu().numpy(), cnt.cpu().numpy()


def test_noalloc_cluster_centers_matches_allocating_entry(km, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(12)
    cases = [(40_000, 64, 100, 1), (25_000, 40, 37, 3)]  # second call: other sizes, 3 tiles
    for m, d, k, tiles in cases:
        X = (rng.standard_normal((m, d)) * 7).astype(np.float32)
        lab = rng.integers(0, k - 1, size=m).astype(np.int32)  # cluster k-1 stays empty (NaN)
        want_c, want_n = run(km, torch, km.ClusterCentersF, X, lab, k, tiles)
        got_c, got_n = run(km, torch, km.ClusterCentersF_noalloc, X, lab, k, tiles)
        assert np.array_equal(got_c, want_c, equal_nan=True)  # same kernels, same sum order
        assert np.array_equal(got_n, want_n)
        assert np.isnan(got_c[k - 1]).all() and got_n[k - 1] == 0


def test_noalloc_rejects_sizes_beyond_its_array(km, torch_cuda):
    torch = torch_cuda
    m, d, k = 2_500_000, 8, 64  # the sorted ids alone need 10 MB > 8 MiB
    lab = torch.zeros(m, dtype=torch.int32, device="cuda")
    X = torch.zeros((m, d), dtype=torch.float32, device="cuda")  # full size: valid even if read
    big = torch.zeros(k * d * 2, dtype=torch.float32, device="cuda")
    cnt_big = torch.zeros(k, dtype=torch.int32, device="cuda")
    cen = torch.zeros((k, d), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(k, dtype=torch.int32, device="cuda")
    rc = km.ClusterCentersF_noalloc(0, m, d, k, True, X, lab, big, cnt_big, cen, cnt)
    assert rc == 4  # ERROR_CLUSTERCENTERS
    assert "8 MiB" in km.last_error()


def test_noalloc_finalize_only_call_at_any_size(km, torch_cuda):
    """A finalize-only call (no rows, lastTile) uses no working memory: it is accepted whatever
    k and n, as ClusterCentersF accepts it, and gives the same means from the same totals."""
    torch = torch_cuda
    rng = np.random.default_rng(3)
    k, d = 4096, 300  # (k + 1) * d * 8 bytes of sums alone exceed the 8 MiB array
    sums = torch.from_numpy(rng.standard_normal(k * d) * 50).cuda()  # FP64 running sums
    counts = torch.from_numpy(rng.integers(0, 9, size=k).astype(np.int32)).cuda()
    outs = []
    for fn in (km.ClusterCentersF, km.ClusterCentersF_noalloc):
        big = sums.clone().view(torch.float32)
        cnt_big = counts.clone()
        cen = torch.zeros((k, d), dtype=torch.float32, device="cuda")
        cnt = torch.zeros(k, dtype=torch.int32, device="cuda")
        dummy = torch.zeros(1, dtype=torch.float32, device="cuda")
        lab = torch.zeros(1, dtype=torch.int32, device="cuda")
        rc = fn(0, 0, d, k, True, dummy, lab, big, cnt_big, cen, cnt)
        assert rc == 0, km.last_error()
        torch.cuda.synchronize()
        outs.append((cen.cpu().numpy(), cnt.cpu().numpy()))
    assert np.array_equal(outs[0][0], outs[1][0], equal_nan=True)
    assert np.array_equal(outs[0][1], outs[1][1])
