"""The learned router on the GPU, through the C-ABI.

The network's kernels (kmgb_router_mlp_train: FP32 SIMT forward/backward and Adam) against the
FP64 oracle (oracle/router.py, itself checked against finite differences on the CPU); the
routed Lloyd run against the full scan on Zipf-sized clustered data (the large-K configuration's
shape at test size): labels, centers and SSE must be identical, since every label the router
proposes is certified (or rescanned) to be the FP64 arg-min; and the ablation: what the trained
router saves (centers scanned per point, certification rate) next to the run without it."""
import time

import numpy as np
import pytest

from oracle import router as orr

pytestmark = pytest.mark.gpu


def net_problem(seed, B=384, d=40, hidden=256, groups=24):
    rng = np.random.default_rng(seed)
    means = rng.standard_normal((groups, d)).astype(np.float32) * 3
    y = rng.integers(0, groups, B).astype(np.int32)
    X = (means[y] + rng.standard_normal((B, d)).astype(np.float32))
    n = hidden * d + hidden + groups * hidden + groups
    p = np.concatenate([rng.standard_normal(hidden * d) * np.sqrt(2.0 / d), np.zeros(hidden),
                        rng.standard_normal(groups * hidden) * np.sqrt(1.0 / hidden),
                        np.zeros(groups)]).astype(np.float32)
    assert p.size == n
    return X, y, p, d, hidden, groups


def test_router_gradients_match_fp64_oracle(km, torch_cuda):
    for seed in (1, 2):
        X, y, p, d, h, g = net_problem(seed)
        loss, grads = km.router_mlp_train(X, y, p.copy(), h, g, batch=len(X), steps=0)
        want_loss, want = orr.loss_and_grads(p, X, y, d, h, g)
        # FP32 sums of up to 384 terms against FP64: relative to the gradient's scale
        scale = np.max(np.abs(want))
        assert abs(loss - want_loss) <= 1e-5 * max(1.0, abs(want_loss))
        assert np.max(np.abs(grads - want)) <= 2e-5 * scale, np.max(np.abs(grads - want)) / scale
        # every block of the flat vector, on its own scale (b1/b2 are small)
        o = 0
        for size in (h * d, h, g * h, g):
            blk, wb = grads[o:o + size], want[o:o + size]
            assert np.max(np.abs(blk - wb)) <= 2e-5 * max(np.max(np.abs(wb)), 1e-6)
            o += size


def test_router_adam_training_follows_the_oracle(km, torch_cuda):
    X, y, p, d, h, g = net_problem(7, B=1024)
    steps, batch, lr = 12, 256, 1e-3
    got = p.copy()
    loss, _ = km.router_mlp_train(X, y, got, h, g, batch=batch, steps=steps, lr=lr)
    want, want_loss = orr.adam_train(p, X, y, d, h, g, batch=batch, steps=steps, lr=lr)
    assert abs(loss - want_loss) <= 1e-4 * max(1.0, abs(want_loss))
    diff = np.abs(got - want)
    # Adam's first steps move each parameter by about lr * sign(gradient): a gradient that is
    # ~0 in FP64 can take the other sign in FP32, so a few parameters may differ by up to
    # 2 lr per step; the rest agree to FP32 rounding
    assert np.mean(diff > 1e-5) < 0.01, np.mean(diff > 1e-5)
    assert np.max(diff) <= 2 * lr * steps + 1e-6
    # and it learns: the loss on the whole set falls
    l0, _ = orr.loss_and_grads(p, X, y, d, h, g)
    l1, _ = orr.loss_and_grads(got, X, y, d, h, g)
    assert l1 < l0


def zipf_case(n=200_000, d=64, k=2048, seed=11):
    from kmeans_gb300.synthetic import sample_init, zipf_blobs_numpy
    X, _, _ = zipf_blobs_numpy(n, d, k, seed=seed)
    init = X[sample_init(n, k, seed=seed + 1)].copy()
    return X, init


def run(km, X, init, iters, **kw):
    k = init.shape[0]
    h = km.Handle(len(X), X.shape[1], k, assign_tier=km.ASSIGN_BF16X3, max_iters=iters, **kw)
    h.set_data(X, False)
    h.set_centers(init, False)
    t0 = time.perf_counter()
    h.run(iters)
    h.synchronize()
    wall = time.perf_counter() - t0
    out = (h.labels(), h.centers(), h.sse(iters), h.stats(), h.router_stats(), wall)
    h.close()
    return out


@pytest.mark.parametrize("shape", [(200_000, 64, 2048, 32), (120_000, 40, 700, 16)])
def test_routed_run_equals_full_scan(km, torch_cuda, shape):
    n, d, k, groups = shape
    X, init = zipf_case(n, d, k)
    iters = 8
    lab0, cen0, sse0, st0, _, _ = run(km, X, init, iters)
    lab1, cen1, sse1, st1, rs, _ = run(km, X, init, iters, router=1, router_groups=groups,
                                      router_retrain=3)
    assert np.array_equal(lab1, lab0)
    assert np.array_equal(cen1, cen0, equal_nan=True)
    assert np.array_equal(sse1, sse0)
    # trained after iterations 0, 3 and 6; iterations 1..7 routed
    assert rs.trainings == 3 and rs.routed_iterations == iters - 1
    # every point of a routed iteration is either certified or rescanned
    assert rs.certified + rs.fallback == n * rs.routed_iterations
    assert rs.certified > 0


def test_routed_run_equals_oracle(km, orc, torch_cuda):
    X, init = zipf_case(30_000, 32, 400, seed=5)
    iters = 5
    res = km.lloyd(X, 400, init=init, max_iters=iters, assign_tier=km.ASSIGN_BF16X3, router=True,
                   router_groups=8, router_retrain=2)
    st, c, lab, sse, it = orc.lloyd(X, init, iters)
    assert np.array_equal(res.labels, lab)
    assert np.array_equal(res.centers, c, equal_nan=True)
    assert np.allclose(res.sse, sse, rtol=1e-10)
    # the label audit also samples the routed iterations
    assert res.audited == 64 * iters and res.audit_violations == 0


def test_router_ablation(km, torch_cuda, capsys):
    """What the trained network gains: the same run without it scans all K centers for every
    point; with it, a certified point scans only its group. Reports the certification rate,
    the centers scanned per point and the times of both runs (labels identical)."""
    X, init = zipf_case(400_000, 128, 4096, seed=21)
    iters = 6
    lab0, _, _, _, _, t_full = run(km, X, init, iters)
    lab1, _, _, _, rs, t_routed = run(km, X, init, iters, router=1, router_groups=64,
                                      router_retrain=5)
    assert np.array_equal(lab1, lab0)
    routed_pts = rs.routed
    cert_rate = rs.certified / max(1, len(X) * rs.routed_iterations)
    with capsys.disabled():
        print(f"\nrouter ablation 400000x128 K=4096 G=64: trainings {rs.trainings} "
              f"(train {rs.train_ms:.0f} ms, grouping {rs.group_ms:.0f} ms, components "
              f"{rs.components}), routed {routed_pts}, certified {rs.certified} "
              f"({cert_rate:.3f} of the points), "
              f"fallback {rs.fallback}, last accuracy {rs.last_accuracy:.3f}; "
              f"{iters} iterations: full scan {t_full:.3f} s, routed {t_routed:.3f} s")
    # a trained router certifies most points of well-separated clustered data
    assert rs.certified >= 0.5 * len(X) * rs.routed_iterations, cert_rate
    assert rs.last_accuracy >= 0.8
