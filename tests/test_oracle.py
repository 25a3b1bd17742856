"""CPU tests of the oracle: pinned against the golden fixtures (independent restatements of
the reference's PRNG calls and its known-answer procedure) and against numpy."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_shuffle_matches_libstdcxx_restatement(orc):
    sh = json.load(open(os.path.join(GOLD, "shuffle.json")))
    for n, v in sh.items():
        p = orc.shuffle_perm(int(n))
        assert sorted(p.tolist()) == list(range(int(n)))
        if isinstance(v, list):
            assert p.tolist() == v
        else:
            assert p[:64].tolist() == v["head"] and p[-64:].tolist() == v["tail"]
            assert sum(i * x for i, x in enumerate(p.tolist())) % (1 << 61) == v["sum_i_p"]


def test_init_picks_match_glibc_rand(orc):
    pk = json.load(open(os.path.join(GOLD, "picks.json")))
    for key, v in pk.items():
        m, k = map(int, key.split("_"))
        assert orc.init_picks(m, k).tolist() == v, key
    # the reference's binary_search on an unsorted list lets duplicates through
    p = orc.init_picks(50, 40).tolist()
    assert len(set(p)) < len(p)


def test_init_rejects_k_above_m(orc):
    with pytest.raises(ValueError):
        orc.init_picks(5, 6)


def test_distance_known_answer(orc):
    z = np.load(os.path.join(GOLD, "distance.npz"))
    a, b, lab = z["a"], z["b"], z["labels"]
    # oracle FP64 arg-min of the direct distance equals the expansion arg-min (no near ties)
    got = orc.assign(a, np.ascontiguousarray(b.T))
    assert np.array_equal(got, lab)


def test_assign_ties_and_nan(orc):
    X = np.array([[0, 0], [1, 1], [2, 2]], np.float32)
    Cn = np.array([[1, 1], [1, 1], [0, 0], [np.nan, 0]], np.float32)
    lab = orc.assign(X, Cn)
    assert lab.tolist() == [2, 0, 0]  # duplicate centers -> lowest index; NaN never wins
    lab = orc.assign(X, np.full((3, 2), np.nan, np.float32))
    assert lab.tolist() == [0, 0, 0]


def test_update_matches_numpy(orc):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((5000, 7)).astype(np.float32)
    k = 9
    lab = rng.integers(0, k - 1, size=5000).astype(np.int32)  # cluster k-1 empty
    old = rng.standard_normal((k, 7)).astype(np.float32)
    c, cnt, sums = orc.update(X, lab, k, old, empty_policy=0)
    for j in range(k - 1):
        mem = X[lab == j].astype(np.float64)
        assert cnt[j] == len(mem)
        np.testing.assert_allclose(sums[j], mem.sum(0), rtol=1e-13, atol=1e-10)
        assert np.array_equal(c[j], (sums[j] / len(mem)).astype(np.float32))
    assert cnt[k - 1] == 0 and np.isnan(c[k - 1]).all()
    c2, _, _ = orc.update(X, lab, k, old, empty_policy=1)
    assert np.array_equal(c2[k - 1], old[k - 1])


def test_sse_matches_numpy(orc):
    rng = np.random.default_rng(4)
    X = rng.standard_normal((3000, 5)).astype(np.float32)
    Cn = rng.standard_normal((6, 5)).astype(np.float32)
    lab = rng.integers(0, 6, size=3000).astype(np.int32)
    want = ((X.astype(np.float64) - Cn.astype(np.float64)[lab]) ** 2).sum()
    assert abs(orc.sse(X, lab, Cn) - want) <= 1e-12 * want


def test_lloyd_matches_numpy_restatement(orc):
    z = np.load(os.path.join(GOLD, "lloyd_small.npz"))
    st, c, lab, sse, it = orc.lloyd(z["X"], z["init"], 10)
    assert st == 13 and it == 10  # criterion < 0 runs all iterations, non-convergence code
    assert np.array_equal(lab, z["labels"])
    np.testing.assert_allclose(c, z["centers"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(sse, z["sse"], rtol=1e-12)


def test_reference_init_uses_shuffled_rows(orc):
    z = np.load(os.path.join(GOLD, "lloyd_small.npz"))
    init = orc.reference_init(z["X"], z["init"].shape[0])
    assert np.array_equal(init, z["init"])


def test_lloyd_sse_monotone_and_convergence(orc):
    from kmeans_gb300.synthetic import mixture_numpy
    X, _, _ = mixture_numpy(4000, 6, 10, seed=1)
    init = X[:10].copy()
    st, c, lab, sse, it = orc.lloyd(X, init, 300, criterion=1e-7)
    assert np.all(np.diff(sse) <= 1e-9 * sse[0])
    assert st == 0 and it < 300
    rel = abs(sse[-1] - sse[-2]) / sse[-1]
    assert rel <= 1e-7


def test_minibatch_windows(orc):
    from kmeans_gb300.synthetic import mixture_numpy
    X, _, _ = mixture_numpy(1000, 4, 5, seed=2)
    init = X[:5].copy()
    frac = 0.3
    st, c, lab, sse, it = orc.lloyd(X, init, 5, mb_fraction=frac)
    m_mb = int(np.float32(frac) * np.float32(1000))
    perm = orc.shuffle_perm(1000)
    # restate the windows: iteration t uses shuffled rows [(t*m_mb) mod m, +m_mb)
    C = init.copy()
    for t in range(5):
        start = (t * m_mb) % 1000
        rows = perm[(start + np.arange(m_mb)) % 1000]
        Xw = X[rows]
        lw = orc.assign(Xw, C)
        C, _, _ = orc.update(Xw, lw, 5, C)
        assert abs(orc.sse(Xw, lw, C) - sse[t]) <= 1e-12 * sse[t]
    assert np.array_equal(C, c, equal_nan=True)
    assert (lab >= 0).sum() == m_mb


def test_port_close_to_oracle(orc):
    from kmeans_gb300.synthetic import mixture_numpy
    X, _, _ = mixture_numpy(3000, 16, 8, seed=5)
    init = X[:8].copy()
    c, lab, sse = orc.port_lloyd(X, init, 3)
    _, c2, lab2, sse2, _ = orc.lloyd(X, init, 3)
    assert (lab != lab2).mean() < 1e-3
    np.testing.assert_allclose(sse, sse2, rtol=1e-5)


def test_tiled_oracle_with_one_tile_is_the_untiled_loop(orc):
    from kmeans_gb300.synthetic import mixture_numpy, sample_init
    X, _, _ = mixture_numpy(3000, 12, 9, seed=44)
    init = X[sample_init(3000, 9, seed=45)]
    a = orc.lloyd(X, init, 4)
    b = orc.lloyd_tiled(X, init, 4, tile_rows=3000)
    assert a[0] == b[0] and a[4] == b[4]
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert np.array_equal(a[3], b[3])
    c = orc.lloyd_tiled(X, init, 4, tile_rows=700)  # same labels, centers within rounding
    assert np.array_equal(a[2], c[2])
    np.testing.assert_allclose(a[1], c[1], rtol=1e-6)
