"""GPU parity of batched Lloyd (kmgb_lloyd_batched_f32): every problem of a batch equals the
oracle's single-problem loop -- labels and centers bit-exact, SSE within 1e-10 relative,
iteration count and status equal -- for mixed dimensions, sizes, inits, stop rules and empty
clusters."""
import numpy as np
import pytest

from kmeans_gb300.synthetic import mixture_numpy, sample_init

pytestmark = pytest.mark.gpu
SSE_RTOL = 1e-10


def check(res, ref):
    st, c, lab, sse, it = ref
    assert res.iterations == it
    assert res.status == st
    assert np.array_equal(res.labels, lab)
    assert np.array_equal(res.centers, c, equal_nan=True)
    np.testing.assert_allclose(res.sse, sse, rtol=SSE_RTOL)


def make_batch(count, seed, dims=(3, 16, 32, 64, 128, 130), nmax=20_000, kmax=316):
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        d = int(rng.choice(dims))
        n = int(np.exp(rng.uniform(np.log(1), np.log(nmax))))
        k = int(max(1, min(n, kmax, round(np.sqrt(max(n, 1) / 2)) + int(rng.integers(0, 3)))))
        X, _, _ = mixture_numpy(n, d, max(1, k), seed=seed * 1000 + i)
        init = None
        if i % 3 == 1:  # explicit, point-sampled init
            init = X[sample_init(n, k, seed=i)]
        probs.append((X, k, init))
    return probs


TIERS = [0, 1, 2]  # FP32 grouped kernel, tcgen05 BF16, tcgen05 split BF16 (pair units)


@pytest.mark.parametrize("tier", TIERS)
def test_mixed_batch_matches_oracle(km, orc, torch_cuda, tier):
    probs = make_batch(40, 5)
    res, st = km.lloyd_batched(probs, max_iters=6, assign_tier=tier)
    for (X, k, init), r in zip(probs, res):
        ini = orc.reference_init(X, k) if init is None else init
        check(r, orc.lloyd(X, ini, 6))
    assert st.iterations == 6
    # the label audit ran in every group iteration (sampled rows that fall in padding or in a
    # stopped problem are skipped) and found nothing
    audited, violations = st.reserved[7] >> 24, st.reserved[7] & 0xFFFFFF
    assert audited > 0 and violations == 0


@pytest.mark.parametrize("tier", TIERS)
def test_per_problem_stop_rule(km, orc, torch_cuda, tier):
    probs = make_batch(24, 9, dims=(8, 32), nmax=5000, kmax=20)
    res, st = km.lloyd_batched(probs, max_iters=60, criterion=1e-4, assign_tier=tier)
    iters = set()
    for (X, k, init), r in zip(probs, res):
        ini = orc.reference_init(X, k) if init is None else init
        ref = orc.lloyd(X, ini, 60, criterion=1e-4)
        check(r, ref)
        iters.add(r.iterations)
    assert len(iters) > 1  # the problems stopped at different iterations


@pytest.mark.parametrize("tier", TIERS)
@pytest.mark.parametrize("policy", [0, 1])
def test_empty_clusters(km, orc, torch_cuda, policy, tier):
    probs = []
    for i, d in enumerate((4, 33)):
        X, _, _ = mixture_numpy(3000, d, 6, seed=40 + i)
        init = X[sample_init(len(X), 9, seed=i)].copy()
        init[5] = init[2]  # duplicate centers: one of each pair stays empty
        init[7] = 1e6      # far away: empty
        probs.append((X, 9, init))
    res, _ = km.lloyd_batched(probs, max_iters=4, empty_policy=policy, assign_tier=tier)
    for (X, k, init), r in zip(probs, res):
        check(r, orc.lloyd(X, init, 4, empty_policy=policy))


def test_matches_single_problem_calls(km, orc, torch_cuda):
    probs = make_batch(6, 13, dims=(24,), nmax=30_000, kmax=64)
    res, _ = km.lloyd_batched(probs, max_iters=5)
    for (X, k, init), r in zip(probs, res):
        one = km.lloyd(X, k, init=init, max_iters=5)
        assert np.array_equal(one.labels, r.labels)
        assert np.array_equal(one.centers, r.centers, equal_nan=True)


@pytest.mark.parametrize("tier", [0, 2])
def test_many_small_problems(km, orc, torch_cuda, tier):
    probs = make_batch(2000, 21, dims=(16, 32, 64, 128), nmax=3000, kmax=40)
    res, st = km.lloyd_batched(probs, max_iters=3, assign_tier=tier)
    rng = np.random.default_rng(0)
    for i in rng.choice(len(probs), 60, replace=False):
        X, k, init = probs[i]
        ini = orc.reference_init(X, k) if init is None else init
        check(res[i], orc.lloyd(X, ini, 3))


@pytest.mark.parametrize("tier", [0, 2])
def test_device_and_host_problems_mixed(km, orc, torch_cuda, tier):
    probs = make_batch(12, 31, dims=(5, 32), nmax=8000, kmax=30)
    mixed = [((torch_cuda.from_numpy(X).cuda() if i % 2 else X), k, init)
             for i, (X, k, init) in enumerate(probs)]
    res, _ = km.lloyd_batched(mixed, max_iters=4, assign_tier=tier)
    for (X, k, init), r in zip(probs, res):
        ini = orc.reference_init(X, k) if init is None else init
        check(r, orc.lloyd(X, ini, 4))


def test_rejections(km, torch_cuda):
    X, _, _ = mixture_numpy(500, 8, 4, seed=3)
    with pytest.raises(km.KmeansError):
        km.lloyd_batched([(X, 501)])  # reference init needs k <= n
    Xw, _, _ = mixture_numpy(300, 330, 4, seed=4)
    with pytest.raises(km.KmeansError):  # the split tier keeps two planes up to D = 320
        km.lloyd_batched([(Xw, 4)], assign_tier=km.ASSIGN_BF16X3)
    Xw, _, _ = mixture_numpy(300, 600, 4, seed=4)
    with pytest.raises(km.KmeansError):  # the plain BF16 tier one plane up to D = 512
        km.lloyd_batched([(Xw, 4)], assign_tier=km.ASSIGN_BF16)
    with pytest.raises(km.KmeansError):  # the FP8 tier runs single problems
        km.lloyd_batched([(X, 4)], assign_tier=km.ASSIGN_FP8)
    arr = (km.kmgb_problem * 1)()
    arr[0].X, arr[0].n, arr[0].d, arr[0].k = X.ctypes.data, 500, 8, 4
    for kw in ({"mini_batch_fraction": 0.5}, {"init_algorithm": km.INIT_KMEANSPP}):
        opt = km.default_options(**kw)
        assert km.lib().kmgb_lloyd_batched_f32(arr, 1, km.C.byref(opt), None) == 1


def test_auto_tier_and_graph_replay_equal_oracle(km, orc, torch_cuda):
    """KMGB_ASSIGN_AUTO (one tier per dimension from the tuned cost table) and the per-iteration
    CUDA graph give every problem the oracle's result; the graph path equals the kernel-by-kernel
    path."""
    import os
    rng = np.random.default_rng(71)
    probs = []
    for i in range(24):
        d = int(rng.choice([16, 32, 64, 128]))
        k = int(rng.choice([5, 20, 60, 150, 300]))
        n = int(max(k, rng.integers(300, 6000)))
        X, _, _ = mixture_numpy(n, d, k, seed=500 + i)
        probs.append((X, k, X[sample_init(n, k, seed=600 + i)].copy()))
    res, st = km.lloyd_batched(probs, max_iters=4, assign_tier=km.ASSIGN_AUTO)
    assert st.reserved[5] > 0 and st.reserved[6] >= 4  # graph launches, groups (4 dimensions)
    for (X, k, init), r in zip(probs, res):
        stt, c, lab, sse, it = orc.lloyd(X, init, 4)
        assert np.array_equal(r.labels, lab) and np.array_equal(r.centers, c, equal_nan=True)
        np.testing.assert_allclose(r.sse, sse, rtol=1e-10)
    old = os.environ.get("KMGB_GRAPHS")
    os.environ["KMGB_GRAPHS"] = "0"
    try:
        res2, st2 = km.lloyd_batched(probs, max_iters=4, assign_tier=km.ASSIGN_AUTO)
    finally:
        if old is None:
            os.environ.pop("KMGB_GRAPHS")
        else:
            os.environ["KMGB_GRAPHS"] = old
    assert st2.reserved[5] == 0
    for a, b in zip(res, res2):
        assert np.array_equal(a.labels, b.labels)
        assert np.array_equal(a.centers, b.centers, equal_nan=True)
