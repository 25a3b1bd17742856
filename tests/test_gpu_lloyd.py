"""GPU parity of the Lloyd loop (assignment + update + SSE + stop rule + mini-batch) against the
FP64 oracle: labels bit-exact, centers bit-exact (canonical FP64 sums rounded once), SSE within
1e-10 relative (the GPU evaluates each cluster's SSE as Q - 2 mu.S + n|mu|^2 in FP64, the
oracle sums the direct form), iteration count and status equal."""
import os

import numpy as np
import pytest

from kmeans_gb300.synthetic import mixture_numpy, sample_init

pytestmark = pytest.mark.gpu
SSE_RTOL = 1e-10
TIERS = [0, 1, 2]  # plain FP32 fused kernel, tcgen05 BF16, tcgen05 split BF16 (x3)


def check_same(res, ref, sse_rtol=SSE_RTOL):
    st, c, lab, sse, it = ref
    assert res.iterations == it
    assert res.status == st
    assert np.array_equal(res.labels, lab)
    assert np.array_equal(res.centers, c, equal_nan=True)
    np.testing.assert_allclose(res.sse, sse, rtol=sse_rtol)


@pytest.mark.parametrize("tier", TIERS)
def test_c1_config(km, orc, torch_cuda, tier):
    X, _, _ = mixture_numpy(100_000, 32, 64, seed=101, mean_lo=-10, mean_hi=10)
    init = X[sample_init(len(X), 64, seed=102)]
    res = km.lloyd(X, 64, init=init, max_iters=20, assign_tier=tier)
    check_same(res, orc.lloyd(X, init, 20))
    assert res.status == 13


# D = 196 and 300: rows of 2 and 3 128-dimension chunks, the last one partial, in the piece sums
@pytest.mark.parametrize("n,d,k", [(1, 1, 1), (130, 3, 7), (1000, 129, 200), (4097, 64, 129),
                                   (20000, 128, 256), (3001, 17, 1), (2000, 256, 300),
                                   (5000, 196, 37), (2500, 300, 50)])
@pytest.mark.parametrize("tier", TIERS)
def test_odd_shapes(km, orc, torch_cuda, n, d, k, tier):
    if (tier == 1 and d > 512) or (tier == 2 and d > 320):
        pytest.skip("the BF16 tier covers D <= 512, the split tier D <= 320")
    X, _, _ = mixture_numpy(n, d, max(k, 1), seed=n + d + k)
    init = X[sample_init(n, k, seed=3)]
    res = km.lloyd(X, k, init=init, max_iters=6, assign_tier=tier)
    check_same(res, orc.lloyd(X, init, 6))


@pytest.mark.parametrize("n,d,k", [(20000, 128, 256), (3001, 17, 40), (50000, 256, 300)])
def test_bf16_valued_data_two_product_mode(km, orc, torch_cuda, n, d, k):
    # every x a BF16 number: the split tier drops the x_lo product (its residual plane is zero)
    # and certifies with the exact-x bound; labels and centers stay those of the oracle
    X, _, _ = mixture_numpy(n, d, k, seed=n + d)
    X = torch_cuda.from_numpy(X).to(torch_cuda.bfloat16).float().numpy()
    init = X[sample_init(n, k, seed=4)]
    for tier in (1, 2):
        res = km.lloyd(X, k, init=init, max_iters=5, assign_tier=tier)
        check_same(res, orc.lloyd(X, init, 5))


@pytest.mark.parametrize("tier", TIERS)
def test_near_ties_are_resolved_exactly(km, orc, torch_cuda, tier):
    # points placed on (or within a few ulps of) the bisector of two centers
    rng = np.random.default_rng(17)
    d, k = 48, 20
    Cn = rng.uniform(-5, 5, size=(k, d)).astype(np.float32)
    a, b = rng.integers(0, k, 4000), rng.integers(0, k, 4000)
    t = 0.5 + rng.integers(-3, 4, 4000) * 1e-7
    X = (Cn[a] * t[:, None] + Cn[b] * (1 - t[:, None])).astype(np.float32)
    X = np.concatenate([X, Cn, Cn[:5]])  # exact duplicates of centers too
    res = km.lloyd(X, k, init=Cn, max_iters=1, assign_tier=tier)
    check_same(res, orc.lloyd(X, Cn, 1))
    assert res.reranked > 0
    if tier != 0:
        # nearly every point is flagged: more than the candidate pass's compact buffer holds
        # (1024 rows at this size), the excess takes the full rescan
        assert res.reranked > 2100 and res.reranked_fp64 > 0


@pytest.mark.parametrize("tier", TIERS)
def test_duplicate_centers_take_the_lowest_index(km, orc, torch_cuda, tier):
    # identical centers give identical FP64 distances: the label is the lowest index. Center 2
    # has one copy (the candidate resolver's exact path), center 5 has 100 copies (more than a
    # column slice of the BF16 epilogue records: 16 in the split tier, 8 in the plain one, so
    # those points take the full rescan).
    rng = np.random.default_rng(23)
    d, k = 40, 200
    Cn = rng.uniform(-4, 4, size=(k, d)).astype(np.float32)
    Cn[9] = Cn[2]
    Cn[20:120] = Cn[5]
    X = np.concatenate([Cn[rng.integers(0, k, 3000)] +
                        rng.normal(0, 0.3, size=(3000, d)).astype(np.float32),
                        Cn[[2, 5, 9, 125]]]).astype(np.float32)
    res = km.lloyd(X, k, init=Cn, max_iters=1, assign_tier=tier)
    ref = orc.lloyd(X, Cn, 1)
    check_same(res, ref)
    assert not np.isin(res.labels, [9] + list(range(20, 120))).any()
    if tier != 0:
        assert res.reranked_fp64 > 0  # the 100-copy points took the full rescan


def test_reference_init_compute_kmeans_f(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(50_000, 24, 40, seed=7)
    m, n, k = X.shape[0], X.shape[1], 40
    result = np.zeros(n * k, np.float32)
    rc = km.computeKmeansF(X, m, n, k, -1.0, 12, 1, 0, 0, 0, result, 1.0)
    assert rc == 13
    st, c, lab, sse, it = orc.lloyd(X, orc.reference_init(X, k), 12)
    assert np.array_equal(result.reshape(n, k), c.T, equal_nan=True)  # D x K, K fastest
    # doFullSGEMM / matrixFormat map to the same implementation; numRetries is ignored with
    # the reference initialisation (initAlgorithm 0)
    r2 = np.zeros_like(result)
    assert km.computeKmeansF(X, m, n, k, -1.0, 12, 3, 0, 1, 1, r2, 1.0) == 13
    assert np.array_equal(r2, result, equal_nan=True)


def test_convergence_criterion(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(30_000, 8, 12, seed=8)
    m, n, k = X.shape[0], X.shape[1], 12
    ref = orc.lloyd(X, orc.reference_init(X, k), 200, criterion=1e-6)
    assert ref[0] == 0 and ref[4] < 200
    result = np.zeros(n * k, np.float32)
    rc = km.computeKmeansF(X, m, n, k, 1e-6, 200, 1, 0, 0, 0, result, 1.0)
    assert rc == 0
    assert np.array_equal(result.reshape(n, k), ref[1].T, equal_nan=True)
    res = km.lloyd(X, k, init=None, max_iters=200, criterion=1e-6)
    check_same(res, ref)


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("policy", [0, 1])
def test_empty_cluster_policy(km, orc, torch_cuda, policy, tier):
    X, _, _ = mixture_numpy(8000, 10, 6, seed=9)
    init = np.concatenate([X[:6], np.full((2, 10), 1e4, np.float32)])  # two far centers
    res = km.lloyd(X, 8, init=init, max_iters=5, empty_policy=policy, assign_tier=tier)
    ref = orc.lloyd(X, init, 5, empty_policy=policy)
    check_same(res, ref)
    assert res.empty_clusters == 2
    if policy == 0:
        assert np.isnan(res.centers[6:]).all()
    else:
        assert np.array_equal(res.centers[6:], init[6:])


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("frac", [0.25, 0.3333, 0.9])
def test_minibatch_windows(km, orc, torch_cuda, frac, tier):
    X, _, _ = mixture_numpy(20_000, 16, 10, seed=10)
    init = X[sample_init(len(X), 10, seed=4)]
    res = km.lloyd(X, 10, init=init, max_iters=9, mini_batch_fraction=frac, assign_tier=tier)
    check_same(res, orc.lloyd(X, init, 9, mb_fraction=frac))


def test_minibatch_compute_kmeans_f(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(20_000, 16, 10, seed=12)
    m, n, k = X.shape[0], X.shape[1], 10
    result = np.zeros(n * k, np.float32)
    assert km.computeKmeansF(X, m, n, k, -1.0, 7, 1, 0, 0, 0, result, 0.2) == 13
    ref = orc.lloyd(X, orc.reference_init(X, k), 7, mb_fraction=0.2)
    assert np.array_equal(result.reshape(n, k), ref[1].T, equal_nan=True)


def test_device_input_and_handle_resume(km, orc, torch_cuda):
    torch = torch_cuda
    X, _, _ = mixture_numpy(60_000, 40, 50, seed=13)
    init = X[sample_init(len(X), 50, seed=5)]
    Xd = torch.from_numpy(X).cuda()
    res = km.lloyd(Xd, 50, init=init, max_iters=5)
    check_same(res, orc.lloyd(X, init, 5))
    h = km.Handle(len(X), 40, 50, max_iters=8)
    h.set_data(Xd, True)
    h.set_centers(init, False)
    h.run(3)
    h.run(2)  # resumes from the current centers
    h.synchronize()
    ref = orc.lloyd(X, init, 5)
    assert np.array_equal(h.centers(), ref[1], equal_nan=True)
    assert np.array_equal(h.labels(), ref[2])
    h.close()


def test_compute_kmeans_d(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(12_000, 9, 15, seed=14)
    X = X.astype(np.float64) * 1.0000001
    m, n, k = X.shape[0], X.shape[1], 15
    result = np.zeros(n * k, np.float64)
    assert km.computeKmeansD(X, m, n, k, -1.0, 6, 1, 0, 1, 0, result, 1.0) == 13
    perm = orc.shuffle_perm(m)
    init = X[perm[orc.init_picks(m, k)]]
    st, c, lab, sse, it = orc.lloyd_d(X, init, 6)
    assert np.array_equal(result.reshape(n, k), c.T, equal_nan=True)


@pytest.mark.parametrize("tier", TIERS)
def test_c2_scale_properties(km, orc, torch_cuda, tier):
    """Full c2 size (4M x 128, K=1024): sampled labels equal the oracle's FP64 arg-min with the
    centers that produced them, centers equal FP64 means of their members, SSE equals an
    independent FP64 evaluation."""
    torch = torch_cuda
    from kmeans_gb300.synthetic import mixture_torch
    n, d, k = 4_000_000, 128, 1024
    X, _, _ = mixture_torch(n, d, k, seed=20, mean_lo=-20, mean_hi=20, std=(0.3, 3.0))
    idx = torch.from_numpy(sample_init(n, k, seed=21)).cuda()
    init = X[idx].cpu().numpy()
    h = km.Handle(n, d, k, max_iters=4, assign_tier=tier)
    h.set_data(X, True)
    h.set_centers(init, False)
    h.run(2)
    h.synchronize()
    c_prev = h.centers()
    h.run(1)
    h.synchronize()
    lab = h.labels()
    c_new = h.centers()
    sse = h.sse(1)[0]
    rng = np.random.default_rng(0)
    s = rng.choice(n, 3000, replace=False)
    Xs = X[torch.from_numpy(s).cuda()].cpu().numpy()
    assert np.array_equal(lab[s], orc.assign(Xs, c_prev))
    Xg = X.double()
    lt = torch.from_numpy(lab).cuda().long()
    sums = torch.zeros((k, d), dtype=torch.float64, device="cuda").index_add_(0, lt, Xg)
    cnt = torch.bincount(lt, minlength=k).double()
    means = (sums / cnt[:, None]).float().cpu().numpy()
    ok = cnt.cpu().numpy() > 0
    np.testing.assert_allclose(c_new[ok], means[ok], rtol=2e-7, atol=1e-6)
    ref_sse = ((Xg - torch.from_numpy(c_new).cuda().double()[lt]) ** 2).sum().item()
    assert abs(sse - ref_sse) <= 1e-9 * ref_sse
    h.close()


def test_zero_sse_stops_like_the_reference(km, orc, torch_cuda):
    """relErr = |0 - 0| / |0| is NaN: the reference loop ends (NaN > criterion is false) even for
    criterion < 0 (kmeans.cpp:1194, 1237)."""
    X = np.array([[1.5, -2.0]], np.float32)
    res = km.lloyd(X, 1, init=X.copy(), max_iters=6)
    assert res.iterations == 1 and res.status == 13 and res.sse[0] == 0.0


@pytest.mark.parametrize("tier", [1, 2])
def test_bf16_tiers_certify_well_separated_points(km, orc, torch_cuda, tier):
    """On well separated clusters almost every point is certified by the tensor-core pass."""
    X, comp, means = mixture_numpy(200_000, 64, 100, seed=31, mean_lo=-50, mean_hi=50)
    res = km.lloyd(X, 100, init=means, max_iters=2, assign_tier=tier)
    check_same(res, orc.lloyd(X, means, 2))
    assert res.reranked < 0.01 * 2 * len(X)


def test_split_tier_certifies_more_than_plain_bf16(km, orc, torch_cuda):
    """Overlapping clusters: the split operand (x_hi.c_hi + x_hi.c_lo + x_lo.c_hi) leaves far fewer
    points to the exact re-rank than plain BF16, with identical labels."""
    X, _, _ = mixture_numpy(100_000, 128, 256, seed=33, mean_lo=-20, mean_hi=20, std=(0.3, 3.0))
    init = X[sample_init(len(X), 256, seed=34)]
    ref = orc.lloyd(X, init, 2)
    r1 = km.lloyd(X, 256, init=init, max_iters=2, assign_tier=1)
    r2 = km.lloyd(X, 256, init=init, max_iters=2, assign_tier=2)
    check_same(r1, ref)
    check_same(r2, ref)
    assert r2.reranked * 5 < r1.reranked


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("tile", [997, 4096, 12000])
def test_host_streamed_tiles(km, orc, torch_cuda, tier, tile):
    # the reference's out-of-memory path: X stays in host memory and passes through the GPU in
    # tiles every iteration; centers follow the tiled canonical order (per-tile sums, tiles in
    # order), labels are the FP64 arg-min
    X, _, _ = mixture_numpy(20000, 48, 40, seed=61)
    init = X[sample_init(len(X), 40, seed=62)]
    res = km.lloyd(X, 40, init=init, max_iters=5, assign_tier=tier, stream_tile_rows=tile)
    check_same(res, orc.lloyd_tiled(X, init, 5, tile_rows=tile))


def test_host_streamed_tiles_stop_rule_and_odd_width(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(9000, 37, 20, seed=63)  # width not a multiple of 4: padded rows
    init = X[sample_init(len(X), 20, seed=64)]
    res = km.lloyd(X, 20, init=init, max_iters=50, criterion=1e-4, assign_tier=km.ASSIGN_BF16,
                   stream_tile_rows=2500)
    ref = orc.lloyd_tiled(X, init, 50, tile_rows=2500, criterion=1e-4)
    check_same(res, ref)
    assert res.iterations < 50


def test_host_streamed_tiles_reject_device_data_and_mini_batch(km, torch_cuda):
    X, _, _ = mixture_numpy(5000, 16, 8, seed=65)
    init = X[sample_init(len(X), 8, seed=66)]
    with pytest.raises(km.KmeansError):
        km.lloyd(torch_cuda.from_numpy(X).cuda(), 8, init=init, max_iters=2, stream_tile_rows=1000)
    with pytest.raises(km.KmeansError):
        km.lloyd(X, 8, init=init, max_iters=2, stream_tile_rows=1000, mini_batch_fraction=0.5)


def test_memory_pool_reuses_and_releases_handle_memory(km, torch_cuda):
    """A destroyed handle's device memory stays in the library's pool, the next handle of the
    same size takes it again without growing the pool, and release_cached_memory gives it back.
    The second run's results equal the first's (reused memory carries nothing over)."""
    torch = torch_cuda
    n, d, k = 1_000_000, 128, 256
    gen = torch.Generator(device="cuda").manual_seed(3)
    X = torch.randn(n, d, device="cuda", generator=gen)
    init = X[:k].cpu().numpy()
    torch.cuda.synchronize()
    km.release_cached_memory()
    free0 = torch.cuda.mem_get_info()[0]

    def one_run():
        h = km.Handle(n, d, k, assign_tier=km.ASSIGN_BF16X3)
        h.set_data(X, True)
        h.set_centers(init)
        h.run(2)
        out = (h.centers(), h.labels(), h.sse(2))
        h.close()
        torch.cuda.synchronize()
        return out

    a = one_run()
    free1 = torch.cuda.mem_get_info()[0]
    b = one_run()
    free2 = torch.cuda.mem_get_info()[0]
    mib = 1 << 20
    # X alone is 512 MB in the handle; its BF16 planes another 512 MB
    assert free0 - free1 > 1000 * mib, (free0, free1)
    assert abs(free1 - free2) < 64 * mib, (free1, free2)
    km.release_cached_memory()
    free3 = torch.cuda.mem_get_info()[0]
    assert abs(free3 - free0) < 64 * mib, (free0, free3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[2], b[2])


# The reference's own test configurations: test/cpp/KmeansTests.cpp:52-60 (mat-sift, 898,790 x
# 128, K=256, 50 iterations, rtol 1e-5, custom kernels, full batch), test/python/kmeansSIFT.py:2-3
# (K=1024) and kmeansHOG.py:2-3 (mat-hog, 796,160 x 324, K=1024), each run with useCUBLAS 0 and 1.
# The SIFT/HOG matrices are not shipped; seeded stand-ins with their shapes and value ranges
# replace them: SIFT descriptors are integers in [0, 255] (so every x is a BF16 number and the
# split tier runs its two-product mode), HOG features FP32 in [0, 1].
REFERENCE_TEST_CONFIGS = [
    ("sift", 898_790, 128, 256, 50),
    ("sift", 898_790, 128, 1024, 50),
    ("hog", 796_160, 324, 1024, 50),
]


def reference_test_data(kind, m, n):
    if kind == "sift":
        X, _, _ = mixture_numpy(m, n, 300, seed=11, mean_lo=0.0, mean_hi=120.0, std=(2.0, 25.0))
        return np.clip(np.rint(X), 0, 255).astype(np.float32)
    X, _, _ = mixture_numpy(m, n, 300, seed=12, mean_lo=0.0, mean_hi=0.5, std=(0.01, 0.1))
    return np.clip(X, 0.0, 1.0).astype(np.float32)


@pytest.mark.parametrize("kind,m,n,k,iters", REFERENCE_TEST_CONFIGS)
def test_reference_test_configurations(km, orc, torch_cuda, kind, m, n, k, iters):
    """computeKmeansF with the reference test's arguments returns the centers of the certified
    loop; its last iteration is pinned to the oracle: labels from the centers one iteration
    earlier on a row sample, the canonical update of all rows bit for bit, the SSE."""
    X = reference_test_data(kind, m, n)
    rtol = 1e-5
    result = np.zeros(n * k, np.float32)
    rc = km.computeKmeansF(X, m, n, k, rtol, iters, 1, 0, 0, 0, result, 1.0)
    assert rc in (0, 13), km.kmeansGetErrorString(rc)
    result_cublas = np.zeros_like(result)
    assert km.computeKmeansF(X, m, n, k, rtol, iters, 1, 0, 1, 0, result_cublas, 1.0) == rc
    assert np.array_equal(result_cublas, result, equal_nan=True)

    # computeKmeansF runs the split BF16 tier where D <= 320, FP32 above; the labels (and so the
    # centers) are the certified FP64 arg-min's in either
    tier = km.ASSIGN_BF16X3 if n <= 320 else km.ASSIGN_FP32
    full = km.lloyd(X, k, max_iters=iters, criterion=rtol, assign_tier=tier)
    t = full.iterations
    assert full.status == rc
    assert np.array_equal(result.reshape(n, k), full.centers.T, equal_nan=True)  # D x K
    assert t >= 2
    prev = km.lloyd(X, k, max_iters=t - 1, criterion=rtol, assign_tier=tier)
    assert prev.iterations == t - 1
    rows = np.random.default_rng(5).choice(m, 16384, replace=False)
    assert np.array_equal(orc.assign(X[rows], prev.centers), full.labels[rows])
    newc, _, _ = orc.update(X, full.labels, k)
    assert np.array_equal(newc, full.centers, equal_nan=True)
    s = orc.sse(X, full.labels, full.centers)
    assert abs(full.sse[-1] - s) <= 1e-10 * s
    print(f"{kind} {m}x{n} K={k}: {t} iterations (rc {rc}), SSE {s:.6e}, "
          f"re-ranked {full.reranked} points")


def test_memory_pool_off_returns_memory_at_destroy(km, torch_cuda):
    """KMGB_POOL=0 (read once per process, so in a child process): a destroyed handle's memory
    goes back to the device without kmgb_release_cached_memory."""
    import subprocess
    import sys
    code = (
        "import torch, numpy as np, kmeans_gb300 as km\n"
        "X = torch.randn(1_000_000, 128, device='cuda')\n"
        "init = X[:256].cpu().numpy()\n"
        "torch.cuda.synchronize()\n"
        "f0 = torch.cuda.mem_get_info()[0]\n"
        "h = km.Handle(1_000_000, 128, 256, assign_tier=km.ASSIGN_BF16X3)\n"
        "h.set_data(X, True); h.set_centers(init); h.run(1)\n"
        "f1 = torch.cuda.mem_get_info()[0]\n"
        "h.close(); torch.cuda.synchronize()\n"
        "f2 = torch.cuda.mem_get_info()[0]\n"
        "assert f0 - f1 > 1000 * 2**20, (f0, f1)\n"
        "assert abs(f2 - f0) < 64 * 2**20, (f0, f2)\n"
        "print('pool off ok')\n")
    env = dict(os.environ, KMGB_POOL="0")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env["PYTHONPATH"] = root + os.pathsep + env.get("PYTHONPATH", "")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and "pool off ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("tier", [1, 2])
@pytest.mark.parametrize("bf16_values", [False, True])
def test_upload_with_first_iteration_matches_resident(km, orc, torch_cuda, tier, bf16_values):
    """A one-shot call on host data sends the data set along with the first iteration (chunks
    assigned as they land, three-product bound until every x is known to be a BF16 number); the
    run from device data uploads first. Labels, centers, SSE and status are the same, and equal
    the oracle's."""
    X, _, _ = mixture_numpy(70_001, 40, 48, seed=21, mean_lo=-8, mean_hi=8)
    if bf16_values:
        X = torch_cuda.from_numpy(X).to(torch_cuda.bfloat16).float().numpy()
    init = X[sample_init(len(X), 48, seed=22)]
    host = km.lloyd(X, 48, init=init, max_iters=7, assign_tier=tier)
    dev = km.lloyd(torch_cuda.from_numpy(X).cuda(), 48, init=init, max_iters=7, assign_tier=tier)
    assert host.status == dev.status and host.iterations == dev.iterations == 7
    assert np.array_equal(host.labels, dev.labels)
    assert np.array_equal(host.centers, dev.centers, equal_nan=True)
    assert np.array_equal(host.sse, dev.sse)
    check_same(host, orc.lloyd(X, init, 7))


def test_compute_kmeans_d_tensor_path(km, orc, torch_cuda):
    """computeKmeansD with D <= 256 runs the split BF16 tier on FP32 roundings of the FP64 data
    and centers, with the bound widened by that rounding, and the exact FP64 scan for the points
    it cannot certify: the result equals the FP64 oracle's. The data carry FP64 precision (an
    FP32 rounding of x loses information)."""
    X, _, _ = mixture_numpy(150_001, 64, 96, seed=31, mean_lo=-5, mean_hi=5)
    rng = np.random.default_rng(32)
    X = X.astype(np.float64) + rng.uniform(-1e-6, 1e-6, X.shape)
    m, n, k = X.shape[0], X.shape[1], 96
    result = np.zeros(n * k, np.float64)
    assert km.computeKmeansD(X, m, n, k, -1.0, 5, 1, 0, 0, 0, result, 1.0) == 13
    perm = orc.shuffle_perm(m)
    init = X[perm[orc.init_picks(m, k)]]
    st, c, lab, sse, it = orc.lloyd_d(X, init, 5)
    assert np.array_equal(result.reshape(n, k), c.T, equal_nan=True)


def test_compute_kmeans_d_fp64_near_ties(km, orc, torch_cuda):
    """Near-ties only FP64 resolves, and exact FP64 duplicates, planted where the reference
    initialisation picks its centers: centers 11 and 12 differ by ~1e-11 (identical after FP32
    rounding), center 7 duplicates center 3, and 200 points sit within 1e-13 of the bisector of
    11 and 12. The tensor pass cannot certify them; the FP64 scan decides (lowest index on
    exact ties), as the oracle does."""
    rng = np.random.default_rng(33)
    m, d, k = 40_600, 16, 40
    X, _, _ = mixture_numpy(m, d, k, seed=34, mean_lo=-4, mean_hi=4)
    X = X.astype(np.float64)
    rows = orc.shuffle_perm(m)[orc.init_picks(m, k)]  # data rows that become the centers
    X[rows[12]] = X[rows[11]] + 1e-11 * rng.standard_normal(d)
    X[rows[7]] = X[rows[3]]
    free = np.setdiff1d(np.arange(m), rows)
    mid = 0.5 * (X[rows[11]] + X[rows[12]])
    X[free[:200]] = mid + 1e-13 * rng.standard_normal((200, d))
    X[free[200:400]] = X[rows[3]] + 1e-3 * rng.standard_normal((200, d))
    # the planted structure is what the oracle's first iteration sees
    _, _, lab1, _, _ = orc.lloyd_d(X, X[rows], 1)
    assert set(lab1[free[:200]].tolist()) == {11, 12}
    assert (lab1[free[200:400]] == 3).all()
    res = np.zeros(d * k, np.float64)
    assert km.computeKmeansD(X, m, d, k, -1.0, 3, 1, 0, 0, 0, res, 1.0) == 13
    _, c, _, _, _ = orc.lloyd_d(X, X[rows], 3)
    assert np.array_equal(res.reshape(d, k), c.T, equal_nan=True)
