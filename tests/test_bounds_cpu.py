"""CPU checks of the rounding-error constants the certified assignment relies on (numpy, exact
FP64 arithmetic on BF16 operands): the operand-rounding terms of the plain and split BF16 tiers,
and the FP32 direct-form bound of the re-rank."""
import numpy as np

UB = 2.0 ** -9


def bf16(a: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even FP32 -> BF16, returned as FP32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def split(a):
    hi = bf16(a)
    lo = bf16(a - hi)  # a - hi is exact in FP32
    return hi, lo


def data(seed, n=400, d=96, k=300):
    rng = np.random.default_rng(seed)
    X = (rng.standard_normal((n, d)) * 10.0 ** rng.uniform(-2, 2, (n, 1))).astype(np.float32)
    C = (rng.standard_normal((k, d)) * 10.0 ** rng.uniform(-2, 2, (k, 1))).astype(np.float32)
    return X, C


def test_plain_bf16_operand_bound():
    for seed in range(3):
        X, C = data(seed)
        exact = X.astype(np.float64) @ C.astype(np.float64).T
        approx = bf16(X).astype(np.float64) @ bf16(C).astype(np.float64).T
        scale = np.abs(X).astype(np.float64) @ np.abs(C).astype(np.float64).T
        assert np.max(np.abs(approx - exact) / scale) <= 2 * UB + UB * UB


def test_split_bf16_operand_bound():
    worst = 0.0
    for seed in range(3):
        X, C = data(seed)
        xh, xl = split(X)
        ch, cl = split(C)
        f = lambda a: a.astype(np.float64)
        exact = f(X) @ f(C).T
        approx = f(xh) @ f(ch).T + f(xh) @ f(cl).T + f(xl) @ f(ch).T
        scale = np.abs(f(X)) @ np.abs(f(C)).T
        worst = max(worst, float(np.max(np.abs(approx - exact) / scale)))
    assert worst <= 3.03 * UB * UB, worst
    assert worst > 0.01 * UB * UB  # the bound is not vacuous


def test_direct_form_fp32_bound():
    rng = np.random.default_rng(7)
    for d in (3, 32, 128, 256):
        X = rng.standard_normal((300, d)).astype(np.float32) * 5
        C = X[rng.integers(0, 300, 50)] + rng.standard_normal((50, d)).astype(np.float32) * 1e-3
        for i in range(0, 300, 7):
            t = (X[i][None, :] - C).astype(np.float32)  # fl(x - c)
            acc = np.zeros(len(C), np.float32)
            for j in range(d):  # sequential FP32 accumulation (numpy rounds each step)
                acc = (acc + t[:, j] * t[:, j]).astype(np.float32)
            exact = ((X[i][None, :].astype(np.float64) - C.astype(np.float64)) ** 2).sum(1)
            gam = (d + 4) * 2.0 * 2.0 ** -24 * 1.01
            assert np.all(np.abs(acc - exact) <= gam * exact + 1e-30)
