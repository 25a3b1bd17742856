"""GPU parity of the k-means++ initialisation (kmgb_kmeanspp_f32/_f64, kmgb_init_kmeanspp,
init_algorithm/num_retries of kmgb_lloyd_f32 and computeKmeansF/D) against the oracle's
restatement of the draw rule: the picked rows are bit-exact (D^2 is evaluated with the same
FP32/FP64 operation order, the weights and their sums are integers)."""
import numpy as np
import pytest

from kmeans_gb300.synthetic import mixture_numpy

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,d,k", [(1, 1, 1), (1000, 3, 17), (1025, 33, 64), (5000, 40, 64),
                                   (3000, 130, 100), (50, 6, 50), (20000, 256, 32)])
def test_picks_match_oracle(km, orc, torch_cuda, n, d, k):
    X, _, _ = mixture_numpy(n, d, max(1, min(k, 40)), seed=n + d)
    for seed in (0, 7):
        cen, picks = km.kmeanspp(X, k, seed)
        want, wcen = orc.kmeanspp(X, k, seed)
        assert np.array_equal(picks, want)
        assert np.array_equal(cen, wcen)


def test_many_weight_blocks(km, orc, torch_cuda):
    # more than 1024 blocks of 1024 points: every scan thread owns a run of several blocks
    rng = np.random.default_rng(5)
    X = (rng.standard_normal((2_100_000, 8)) * 3).astype(np.float32)
    cen, picks = km.kmeanspp(X, 6, 3)
    want, _ = orc.kmeanspp(X, 6, 3)
    assert np.array_equal(picks, want)


@pytest.mark.parametrize("d", [33, 7])
def test_unaligned_device_rows_take_the_register_kernel(km, orc, torch_cuda, d):
    # a device array whose rows are not 16-byte aligned cannot be staged with bulk copies
    X, _, _ = mixture_numpy(9000, d, 20, seed=d)
    want, wcen = orc.kmeanspp(X, 40, 12)
    cen, picks = km.kmeanspp(torch_cuda.from_numpy(X).cuda(), 40, 12)
    assert np.array_equal(picks, want)
    assert np.array_equal(cen, wcen)


def test_float64_picks_match_oracle(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(7000, 45, 30, seed=21)
    X = X.astype(np.float64) * (1 + 1e-9)
    cen, picks = km.kmeanspp(X, 30, 2)
    want, wcen = orc.kmeanspp(X, 30, 2)
    assert np.array_equal(picks, want)
    assert cen.dtype == np.float64 and np.array_equal(cen, wcen)


def test_identical_points_and_duplicates(km, orc, torch_cuda):
    X = np.ones((3000, 5), np.float32)
    X[::7] = 2.0
    for k in (1, 2, 9):
        _, picks = km.kmeanspp(X, k, 4)
        assert np.array_equal(picks, orc.kmeanspp(X, k, 4)[0])


def test_device_input_and_resident_handle(km, orc, torch_cuda):
    torch = torch_cuda
    X, _, _ = mixture_numpy(40_000, 24, 50, seed=31)
    want, wcen = orc.kmeanspp(X, 50, 9)
    Xd = torch.from_numpy(X).cuda()
    cen, picks = km.kmeanspp(Xd, 50, 9)
    assert np.array_equal(picks, want)
    h = km.Handle(len(X), 24, 50, assign_tier=0)
    h.set_data(Xd, True)
    assert np.array_equal(h.init_kmeanspp(9), want)
    assert np.array_equal(h.centers(), wcen)
    h.run(4)
    h.synchronize()
    st, c, lab, sse, it = orc.lloyd(X, wcen, 4)
    assert np.array_equal(h.centers(), c, equal_nan=True)
    assert np.array_equal(h.labels(), lab)
    h.close()


@pytest.mark.parametrize("tier", [0, 2])
def test_retries_keep_the_lowest_final_sse(km, orc, torch_cuda, tier):
    X, _, _ = mixture_numpy(30_000, 16, 24, seed=41)
    k, iters, seed0, retries = 24, 5, 100, 4
    finals = []
    for r in range(retries):
        _, init = orc.kmeanspp(X, k, seed0 + r)
        finals.append(orc.lloyd(X, init, iters))
    best = min(range(retries), key=lambda r: (finals[r][3][-1], r))
    res = km.lloyd(X, k, max_iters=iters, assign_tier=tier, init_algorithm=km.INIT_KMEANSPP,
                   num_retries=retries, seed=seed0)
    st, c, lab, sse, it = finals[best]
    assert np.array_equal(res.centers, c, equal_nan=True)
    assert np.array_equal(res.labels, lab)
    np.testing.assert_allclose(res.sse, sse, rtol=1e-10)


def test_compute_kmeans_f_init_algorithm(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(20_000, 12, 16, seed=51)
    m, n, k = X.shape[0], X.shape[1], 16
    finals = []
    for r in range(3):
        _, init = orc.kmeanspp(X, k, r)
        finals.append(orc.lloyd(X, init, 6))
    best = min(range(3), key=lambda r: (finals[r][3][-1], r))
    result = np.zeros(n * k, np.float32)
    assert km.computeKmeansF(X, m, n, k, -1.0, 6, 3, 1, 0, 0, result, 1.0) == 13
    assert np.array_equal(result.reshape(n, k), finals[best][1].T, equal_nan=True)
    # initAlgorithm 0 keeps the reference initialisation whatever numRetries says
    r0 = np.zeros_like(result)
    assert km.computeKmeansF(X, m, n, k, -1.0, 6, 5, 0, 0, 0, r0, 1.0) == 13
    ref = orc.lloyd(X, orc.reference_init(X, k), 6)
    assert np.array_equal(r0.reshape(n, k), ref[1].T, equal_nan=True)


def test_compute_kmeans_d_init_algorithm(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(8000, 10, 12, seed=61)
    X = X.astype(np.float64) * (1 + 1e-9)
    m, n, k = X.shape[0], X.shape[1], 12
    finals = []
    for r in range(2):
        _, init = orc.kmeanspp(X, k, r)
        finals.append(orc.lloyd_d(X, init, 5))
    best = min(range(2), key=lambda r: (finals[r][3][-1], r))
    result = np.zeros(n * k, np.float64)
    assert km.computeKmeansD(X, m, n, k, -1.0, 5, 2, 1, 0, 0, result, 1.0) == 13
    assert np.array_equal(result.reshape(n, k), finals[best][1].T, equal_nan=True)


def test_mini_batch_handle_restarts_at_the_first_window(km, orc, torch_cuda):
    X, _, _ = mixture_numpy(12_000, 8, 10, seed=71)
    _, init = orc.kmeanspp(X, 10, 1)
    ref = orc.lloyd(X, init, 4, mb_fraction=0.25)
    res = km.lloyd(X, 10, max_iters=4, mini_batch_fraction=0.25,
                   init_algorithm=km.INIT_KMEANSPP, seed=1)
    assert np.array_equal(res.centers, ref[1], equal_nan=True)


def test_rejections(km, torch_cuda):
    X, _, _ = mixture_numpy(2000, 8, 4, seed=81)
    with pytest.raises(km.KmeansError):
        km.kmeanspp(X, 2001, 0)
    with pytest.raises(km.KmeansError):  # host-streamed data is not resident
        km.lloyd(X, 4, max_iters=2, stream_tile_rows=500, init_algorithm=km.INIT_KMEANSPP)
