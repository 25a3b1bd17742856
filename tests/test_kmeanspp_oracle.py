"""The k-means++ oracle (oracle.cpp orc_kmeanspp) against an independent pure-Python
restatement of the same draw rule, and the D^2 sampling law it is meant to follow.

Rule: D^2 in the data's precision from 32 lane partials (lane l: dims l, l+32, ... as an fma
chain) folded by an xor butterfly; weights q = trunc(D^2 * 2^31 / max D^2); draw r uses
u = splitmix64(splitmix64(seed) + r) >> 11 and the point whose [prefix, prefix + q) holds
(u * sum q) >> 53; draw 0 and zero-weight draws take (u * n) >> 53."""
import math

import numpy as np
import pytest

M64 = (1 << 64) - 1


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def fma32(a, b, c):
    """a*b + c rounded once to float32 (round to nearest, ties to even), from the exact value."""
    from fractions import Fraction
    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    f = np.float32(float(exact))
    cands = [f, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf))]
    return min(cands, key=lambda v: (abs(Fraction(float(v)) - exact),
                                     int(np.float32(v).view(np.uint32)) & 1))


def d2_lanes(x, c):
    d = len(x)
    lanes = []
    for l in range(32):
        s = np.float32(0)
        for t in range(l, d, 32):
            u = np.float32(x[t] - c[t])
            s = fma32(u, u, s)
        lanes.append(s)
    o = 16
    while o:
        lanes = [np.float32(lanes[i] + lanes[i ^ o]) for i in range(32)]
        o >>= 1
    return lanes[0]


def py_kmeanspp(X, k, seed):
    n = len(X)
    d2 = [None] * n
    picks = []
    s0 = splitmix64(seed)
    for r in range(k):
        total = 0
        q = [0] * n
        if r > 0:
            c = X[picks[-1]]
            for i in range(n):
                v = d2_lanes(X[i], c)
                d2[i] = v if r == 1 else np.float32(min(d2[i], v))
            M = max(d2)
            scale = np.float32(np.float32(2147483648.0) / M) if M > 0 else np.float32(0)
            for i in range(n):
                p = np.float32(d2[i] * scale)
                q[i] = int(p) if p > 0 else 0
            total = sum(q)
        u = splitmix64((s0 + r) & M64) >> 11
        chosen = (u * n) >> 53
        if total > 0:
            target = (u * total) >> 53
            ex = 0
            for i in range(n):
                if q[i] > 0 and target < ex + q[i]:
                    chosen = i
                    break
                ex += q[i]
        picks.append(chosen)
    return np.array(picks, np.int32)


@pytest.mark.parametrize("n,d,k,seed", [(40, 3, 5, 0), (70, 37, 6, 11), (33, 64, 33, 5)])
def test_oracle_matches_python_restatement(orc, n, d, k, seed):
    rng = np.random.default_rng(n * 7 + d)
    X = (rng.standard_normal((n, d)) * rng.uniform(0.1, 10, d)).astype(np.float32)
    picks, cen = orc.kmeanspp(X, k, seed)
    assert np.array_equal(picks, py_kmeanspp(X, k, seed))
    assert np.array_equal(cen, X[picks])


def test_second_draw_follows_d2(orc):
    # five points on a line; the first draw is uniform, the second proportional to D^2
    X = np.array([[0.0], [1.0], [3.0], [7.0], [15.0]], np.float32)
    n, trials = len(X), 6000
    obs = np.zeros((n, n))
    for s in range(trials):
        p, _ = orc.kmeanspp(X, 2, s)
        obs[p[0], p[1]] += 1
    exp = np.zeros((n, n))
    for a in range(n):
        w = (X[:, 0] - X[a, 0]) ** 2
        exp[a] = trials / n * w / w.sum()
    assert np.all(np.diag(obs) == 0)  # a drawn point has D^2 = 0
    mask = exp > 0
    z = (obs[mask] - exp[mask]) / np.sqrt(exp[mask])
    assert np.max(np.abs(z)) < 5.0


def test_separated_clusters_get_one_center_each(orc):
    rng = np.random.default_rng(3)
    means = np.arange(16)[:, None] * 1000.0 * np.ones((1, 8))
    X = (means[rng.integers(0, 16, 4000)] + rng.standard_normal((4000, 8))).astype(np.float32)
    for seed in range(5):
        p, cen = orc.kmeanspp(X, 16, seed)
        assert len(set(np.round(cen[:, 0] / 1000.0).astype(int).tolist())) == 16


def test_identical_points_fall_back_to_uniform_draws(orc):
    X = np.ones((50, 4), np.float32)
    p, _ = orc.kmeanspp(X, 6, 2)
    s0 = splitmix64(2)
    want = [((splitmix64((s0 + r) & M64) >> 11) * 50) >> 53 for r in range(6)]
    assert p.tolist() == want


def test_float64_rule(orc):
    rng = np.random.default_rng(9)
    X = rng.standard_normal((300, 20))
    p, cen = orc.kmeanspp(X, 12, 4)
    assert cen.dtype == np.float64 and np.array_equal(cen, X[p])
    assert len(set(p.tolist())) == 12


def test_rejects_k_above_n(orc):
    with pytest.raises(ValueError):
        orc.kmeanspp(np.zeros((3, 2), np.float32), 4, 0)
