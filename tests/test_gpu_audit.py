"""GPU checks of the label audit (launch_audit_labels, kmgb_stats reserved[6..7],
kmgb_debug_audit): every certified run samples rows each iteration and checks their labels
against the FP64 arg-min over all centers. The runs of every tier report no violation; the audit
kernel counts exactly the sampled rows whose label was made wrong on the host, and does not judge
ties (equal FP64 distances)."""
import numpy as np
import pytest

from kmeans_gb300.synthetic import mixture_numpy, sample_init

pytestmark = pytest.mark.gpu
MASK = (1 << 64) - 1


def sampled_rows(n, rows, seq=0):
    """The rows one audit samples: a SplitMix64 hash (Steele, Lea and Flood 2014) of the sampling
    sequence plus the sample index, modulo n."""
    out = []
    for r in range(rows):
        z = (seq + r + 0x9E3779B97F4A7C15) & MASK
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        out.append((z ^ (z >> 31)) % n)
    return np.array(out, dtype=np.int64)


def fp64_labels(X, C):
    d2 = ((X[:, None, :].astype(np.float64) - C[None, :, :].astype(np.float64)) ** 2).sum(-1)
    return d2.argmin(1).astype(np.int32)


@pytest.mark.parametrize("tier", [0, 1, 2, 3])  # FP32, BF16, split BF16, FP8
def test_every_tier_audits_without_violation(km, torch_cuda, tier):
    X, _, _ = mixture_numpy(20_000, 64, 40, seed=3)
    init = X[sample_init(len(X), 40, seed=1)].copy()
    r = km.lloyd(X, 40, init=init, max_iters=5, assign_tier=tier)
    assert r.audited == 5 * 64
    assert r.audit_violations == 0


def test_audit_rows_follow_the_environment(km, torch_cuda, monkeypatch):
    X, _, _ = mixture_numpy(4000, 16, 10, seed=4)
    init = X[:10].copy()
    monkeypatch.setenv("KMGB_AUDIT_ROWS", "0")
    assert km.lloyd(X, 10, init=init, max_iters=3).audited == 0
    monkeypatch.setenv("KMGB_AUDIT_ROWS", "7")
    assert km.lloyd(X, 10, init=init, max_iters=3).audited == 21
    # no certificate, no audit
    monkeypatch.delenv("KMGB_AUDIT_ROWS")
    assert km.lloyd(X, 10, init=init, max_iters=3, certify=False).audited == 0


def test_audit_counts_planted_wrong_labels(km, torch_cuda):
    torch = torch_cuda
    X, _, _ = mixture_numpy(5000, 32, 20, seed=5)
    C = X[sample_init(5000, 20, seed=2)].copy()
    lab = fp64_labels(X, C)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    assert km.debug_audit(dev(X), dev(C), dev(lab), rows=200) == (200, 0, 0)
    wrong = lab.copy()
    wrong[::2] = (wrong[::2] + 1) % 20  # even rows: another (strictly farther) center
    rows = sampled_rows(5000, 200)
    expect = int((rows % 2 == 0).sum())
    aud, viol, last = km.debug_audit(dev(X), dev(C), dev(wrong), rows=200)
    assert aud == 200 and viol == expect and viol > 0
    assert last > 0 and (last - 1) % 2 == 0 and (last - 1) in set(rows.tolist())


def test_audit_skips_empty_cluster_centers(km, torch_cuda):
    """An empty cluster's NaN center (the reference's 0/0) is no center: runs with empty clusters
    report no violation, and the kernel ignores NaN rows of C."""
    torch = torch_cuda
    X, _, _ = mixture_numpy(6000, 12, 5, seed=8)
    init = X[sample_init(6000, 9, seed=4)].copy()
    init[6] = 1e6  # far away: empty after the first assignment, then NaN
    r = km.lloyd(X, 9, init=init, max_iters=4, assign_tier=km.ASSIGN_BF16X3)
    assert r.empty_clusters >= 1 and r.audited == 4 * 64 and r.audit_violations == 0
    C = init.copy()
    lab = fp64_labels(X, C)
    C[6] = np.nan
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    assert km.debug_audit(dev(X), dev(C), dev(lab), rows=128)[1] == 0


def test_audit_does_not_judge_ties(km, torch_cuda):
    torch = torch_cuda
    X, _, _ = mixture_numpy(3000, 8, 6, seed=6)
    C = X[sample_init(3000, 6, seed=3)].copy()
    C[5] = C[2]  # duplicate center: equal FP64 distances
    lab = fp64_labels(X, C)  # lowest index on ties: never 5
    assert (lab == 2).any() and not (lab == 5).any()
    tied = np.where(lab == 2, 5, lab).astype(np.int32)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    assert km.debug_audit(dev(X), dev(C), dev(tied), rows=256)[1] == 0
