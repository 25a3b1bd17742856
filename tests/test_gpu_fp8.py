"""The FP8 E4M3 tier (tcgen05 kind::f8f6f4, per-row power-of-two scales) and the BF16 tiers past
D = 256, against the FP64 oracle: labels and centers bit for bit, SSE to 1e-10. E4M3 keeps 3
mantissa bits, so most points of clustered data still certify by their margin; the rest take
the candidate pass (a second FP8 scan recording every center within the bound) and the exact
settlement, so labels are the FP64 arg-min as in every tier."""
import numpy as np
import pytest

from kmeans_gb300.synthetic import mixture_numpy, sample_init

pytestmark = pytest.mark.gpu


def check_same(res, ref):
    st, c, lab, sse, it = ref
    assert res.iterations == it and res.status == st
    assert np.array_equal(res.labels, lab)
    assert np.array_equal(res.centers, c, equal_nan=True)
    np.testing.assert_allclose(res.sse, sse, rtol=1e-10)


@pytest.mark.parametrize("n,d,k", [(1, 1, 1), (130, 3, 7), (1000, 129, 200), (4097, 64, 129),
                                   (20000, 128, 256), (3001, 17, 1), (2000, 300, 300),
                                   (1500, 512, 64)])
def test_fp8_odd_shapes(km, orc, torch_cuda, n, d, k):
    X, _, _ = mixture_numpy(n, d, max(k, 1), seed=n + d + k)
    init = X[sample_init(n, k, seed=3)]
    res = km.lloyd(X, k, init=init, max_iters=6, assign_tier=km.ASSIGN_FP8)
    check_same(res, orc.lloyd(X, init, 6))


def test_fp8_c1_config(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(100_000, 32, 64, seed=101, mean_lo=-10, mean_hi=10)
    init = X[sample_init(len(X), 64, seed=102)]
    res = km.lloyd(X, 64, init=init, max_iters=20, assign_tier=km.ASSIGN_FP8)
    check_same(res, orc.lloyd(X, init, 20))
    assert res.reranked > 0  # E4M3's band leaves points to the exact settlement


def test_fp8_rows_of_many_magnitudes_and_duplicates(km, orc, torch_cuda):
    """Rows scaled over six decades (each row has its own scale; components far below a row's
    largest become E4M3 subnormals) and duplicate centers (exact ties: lowest index)."""
    rng = np.random.default_rng(11)
    n, d, k = 6000, 48, 80
    X, _, _ = mixture_numpy(n, d, k, seed=12)
    X *= (10.0 ** rng.uniform(-3, 3, (n, 1))).astype(np.float32)
    X[:500, : d // 2] *= 1e-4
    init = X[sample_init(n, k, seed=13)].copy()
    init[5] = init[4]  # duplicate center
    res = km.lloyd(X, k, init=init, max_iters=4, assign_tier=km.ASSIGN_FP8)
    check_same(res, orc.lloyd(X, init, 4))


@pytest.mark.parametrize("tier,d", [(1, 324), (1, 512), (2, 300), (2, 320)])
def test_bf16_tiers_past_256_dims(km, orc, torch_cuda, tier, d):
    """The plain BF16 tier keeps one point plane in shared memory up to D = 512 (the reference's
    own HOG test width, 324, included), the split tier its two planes up to 320."""
    n, k = 5000, 96
    X, _, _ = mixture_numpy(n, d, k, seed=d)
    init = X[sample_init(n, k, seed=5)]
    res = km.lloyd(X, k, init=init, max_iters=4, assign_tier=tier)
    check_same(res, orc.lloyd(X, init, 4))


def test_fp8_rejected_where_unsupported(km, torch_cuda):
    X = np.zeros((1000, 600), np.float32)
    with pytest.raises(km.KmeansError):
        km.lloyd(X, 4, init=X[:4], max_iters=1, assign_tier=km.ASSIGN_FP8)
    X = np.random.default_rng(0).standard_normal((1000, 16)).astype(np.float32)
    with pytest.raises(km.KmeansError):
        km.lloyd(X, 4, init=X[:4], max_iters=1, assign_tier=km.ASSIGN_FP8,
                 mini_batch_fraction=0.5)
