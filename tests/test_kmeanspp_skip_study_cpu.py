"""The row-skip rule considered for the k-means++ D^2 pass, simulated on the CPU.

A draw can skip row x when the new center c cannot lower D^2(x): with a(x) the chosen center
nearest to x and D(x) = |x - c_a(x)|, |c - c_a(x)| >= 2 D(x) implies |x - c| >= D(x) (triangle
inequality). This follows the D^2-weighted draw of the library's k-means++ (in FP64 numpy,
without its integer weights) on the 4M x 128, K=1024 mixture's distribution (1024 anisotropic Gaussians, std
log-U[0.3, 3], means U[-20, 20]^128) with fewer rows, and measures the share of rows the rule
would skip per draw. The clusters are far apart relative to their spread, so a row skips exactly
when its own cluster already holds a center: the share grows with the draws as the clusters are
covered, about r / K after r draws, and averages about one half over the K draws."""
import numpy as np

from kmeans_gb300.synthetic import mixture_numpy


def skip_shares(n=8192, d=128, k=1024, seed=5):
    X, comp, _ = mixture_numpy(n, d, k, seed=seed, mean_lo=-20, mean_hi=20, std=(0.3, 3.0))
    X = X.astype(np.float64)
    xx = (X * X).sum(1)
    rng = np.random.default_rng(1)
    first = int(rng.integers(n))
    C = np.empty((k, d))
    C[0] = X[first]
    D2 = np.maximum(xx - 2.0 * X @ C[0] + C[0] @ C[0], 0.0)
    a = np.zeros(n, np.int64)
    shares, covered = [], {int(comp[first])}
    for r in range(1, k):
        cdf = np.cumsum(D2)
        i = int(np.searchsorted(cdf, rng.uniform(0.0, cdf[-1]), side="right"))
        i = min(i, n - 1)
        c = X[i]
        covered.add(int(comp[i]))
        dc = np.sqrt(((C[:r] - c) ** 2).sum(1))  # |c - c_j| for the chosen centers
        skip = dc[a] >= 2.0 * np.sqrt(D2)
        d2n = ((X - c) ** 2).sum(1)
        lower = d2n < D2
        assert not np.any(lower & skip)  # the rule is sound: a skipped row keeps its D^2
        shares.append(float(skip.mean()))
        D2 = np.where(lower, d2n, D2)
        a = np.where(lower, r, a)
        C[r] = c
    return np.array(shares), len(covered)


def test_skip_share_follows_covered_clusters():
    s, covered = skip_shares()
    k = len(s) + 1
    print(f"mean share {s.mean():.3f}; after 64/256/512/768/1023 draws "
          + " ".join(f"{s[j - 1]:.3f}" for j in (64, 256, 512, 768, 1023))
          + f"; {covered} of {k} clusters covered")
    assert 0.4 < s.mean() < 0.6
    # early draws skip little, late draws nearly everything: about r / K after r draws
    assert s[63] < 0.15 and s[-1] > 0.85
    for r in (256, 512, 768):
        assert abs(s[r - 1] - r / k) < 0.15
