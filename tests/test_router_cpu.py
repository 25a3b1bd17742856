"""CPU checks of the router's FP64 oracle (oracle/router.py): its gradients against central
finite differences and its Adam step against the update written out by hand. The GPU kernels are
checked against this oracle in tests/test_gpu_router.py."""
import numpy as np

from oracle import router as orr


def small_problem(seed=0, B=7, d=5, hidden=6, groups=4):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((B, d))
    y = rng.integers(0, groups, B)
    n = hidden * d + hidden + groups * hidden + groups
    p = rng.standard_normal(n) * 0.7
    return X, y, p, d, hidden, groups


def test_oracle_gradients_match_finite_differences():
    X, y, p, d, h, g = small_problem()
    loss, grad = orr.loss_and_grads(p, X, y, d, h, g)
    assert np.isfinite(loss) and grad.shape == p.shape
    eps = 1e-6
    num = np.empty_like(p)
    for i in range(p.size):
        q = p.copy()
        q[i] += eps
        lp, _ = orr.loss_and_grads(q, X, y, d, h, g)
        q[i] -= 2 * eps
        lm, _ = orr.loss_and_grads(q, X, y, d, h, g)
        num[i] = (lp - lm) / (2 * eps)
    # a ReLU kink within eps of a finite-difference point would break this; the seeds avoid one
    assert np.max(np.abs(num - grad)) < 1e-7 * max(1.0, np.max(np.abs(grad)))


def test_oracle_adam_step_written_out():
    X, y, p, d, h, g = small_problem(seed=3)
    lr, b1, b2, eps = 1e-2, 0.9, 0.999, 1e-8
    p1, loss = orr.adam_train(p, X, y, d, h, g, batch=7, steps=1, lr=lr)
    l0, g0 = orr.loss_and_grads(p, X, y, d, h, g)
    m = (1 - b1) * g0
    v = (1 - b2) * g0 * g0
    want = p - lr * (m / (1 - b1)) / (np.sqrt(v / (1 - b2)) + eps)
    assert loss == l0
    assert np.allclose(p1, want, rtol=0, atol=1e-15)


def test_oracle_training_lowers_the_loss():
    rng = np.random.default_rng(5)
    means = rng.standard_normal((4, 8)) * 4
    y = rng.integers(0, 4, 512)
    X = means[y] + rng.standard_normal((512, 8))
    d, h, g = 8, 16, 4
    n = h * d + h + g * h + g
    p0 = rng.standard_normal(n) * 0.2
    l0, _ = orr.loss_and_grads(p0, X, y, d, h, g)
    p1, _ = orr.adam_train(p0, X, y, d, h, g, batch=64, steps=200, lr=1e-2)
    l1, _ = orr.loss_and_grads(p1, X, y, d, h, g)
    assert l1 < 0.2 * l0
