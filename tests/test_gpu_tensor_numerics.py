"""Tensor-core numerics behind the certified BF16 assignment: the raw tcgen05 accumulators
(x.c - ||c||^2/2 with FP32 accumulation in TMEM) are compared with the exact sums of the same
BF16 products. The kernel's certificate assumes the accumulation error stays below
(terms/16 + 2) * 2^-21 * (|start| + sum |products|) (one rounding per 16-product MMA step plus
the start value, with margin); this test measures the worst case on the device and requires it
to be at least 4x below that model."""
import numpy as np
import pytest

from test_bounds_cpu import bf16, bound_fp8, fp8_operands, split

pytestmark = pytest.mark.gpu


def cases():
    rng = np.random.default_rng(3)
    n, d, k = 384, 128, 256
    X = (rng.standard_normal((n, d)) * 10.0 ** rng.uniform(-1, 1, (n, 1))).astype(np.float32)
    C = (rng.standard_normal((k, d)) * 10.0 ** rng.uniform(-1, 1, (k, 1))).astype(np.float32)
    yield "mixed", X, C
    # heavy cancellation: points close to centers, large common offset
    C2 = (rng.uniform(-20, 20, (k, d)) + 50).astype(np.float32)
    X2 = (C2[rng.integers(0, k, n)] + rng.standard_normal((n, d)).astype(np.float32) * 0.1)
    yield "offset", X2.astype(np.float32), C2
    X3 = rng.uniform(-1, 1, (n, 64)).astype(np.float32)
    C3 = rng.uniform(-1, 1, (k, 64)).astype(np.float32)
    yield "d64", X3, C3
    # the widest rows the tiers take (3 x 256 products per element in the split tier)
    X4 = (rng.standard_normal((n, 256)) * 3 + 20).astype(np.float32)
    C4 = (X4[rng.integers(0, n, k)] + rng.standard_normal((k, 256)).astype(np.float32))
    yield "d256", X4, C4.astype(np.float32)


@pytest.mark.parametrize("use_split", [0, 1, 2])
def test_tc_accumulation_error_model(km, torch_cuda, use_split):
    f = lambda a: a.astype(np.float64)
    for name, X, C in cases():
        d = X.shape[1]
        if use_split == 2:  # the two-product mode takes BF16-valued points
            X = bf16(X).astype(np.float32)
        acc = km.tc_accumulators(X, C, use_split).astype(np.float64)
        cn = (f(C) ** 2).sum(1).astype(np.float32)  # ||c||^2 rounded once to FP32
        start = -0.5 * f(cn)
        if use_split == 2:
            ch, cl = split(C)
            prod = f(X) @ f(ch).T + f(X) @ f(cl).T
            mag = np.abs(f(X)) @ np.abs(f(ch)).T + np.abs(f(X)) @ np.abs(f(cl)).T
            terms = 2 * d
        elif use_split:
            xh, xl = split(X)
            ch, cl = split(C)
            prod = f(xh) @ f(ch).T + f(xh) @ f(cl).T + f(xl) @ f(ch).T
            mag = np.abs(f(xh)) @ np.abs(f(ch)).T + np.abs(f(xh)) @ np.abs(f(cl)).T \
                + np.abs(f(xl)) @ np.abs(f(ch)).T
            terms = 3 * d
        else:
            xb, cb = bf16(X), bf16(C)
            prod = f(xb) @ f(cb).T
            mag = np.abs(f(xb)) @ np.abs(f(cb)).T
            terms = d
        exact = prod + start[None, :]
        scale = mag + np.abs(start)[None, :]
        err = np.max(np.abs(acc - exact) / scale)
        model = (terms // 16 + 2) * 2.0 ** -21
        print(f"{name} split={use_split}: max accumulation error {err:.3e} of scale, "
              f"model {model:.3e} (ratio {err / model:.4f})")
        assert err * 4 <= model, (name, err, model)


def test_fp8_keys_within_model_and_certificate_bound(km, torch_cuda):
    """The FP8 tier's raw keys: against the exact sums of the same E4M3 products (accumulation
    error >= 4x below the model) and against the exact x.c - |c|^2/2 (within the certificate's
    bound_fp8, which the label certificate relies on)."""
    f = lambda a: a.astype(np.float64)
    for name, X, C in cases():
        d = X.shape[1]
        keys = km.tc_accumulators(X, C, 3).astype(np.float64)
        cn = (f(C) ** 2).sum(1).astype(np.float32)
        start = -0.5 * f(cn)
        X8, sx, C8, sc = fp8_operands(X, C)
        prod = (X8 @ C8.T) * (sx[:, None] * sc)
        mag = (np.abs(X8) @ np.abs(C8).T) * (sx[:, None] * sc)
        err = np.max(np.abs(keys - (prod + start[None, :])) / (mag + np.abs(start)[None, :]))
        model = (d // 16 + 2) * 2.0 ** -21
        print(f"{name} fp8: max accumulation error {err:.3e} of scale, model {model:.3e}")
        assert err * 4 <= model, (name, err, model)
        exact = f(X) @ f(C).T - 0.5 * (f(C) ** 2).sum(1)[None, :]
        xn = np.sqrt((f(X) ** 2).sum(1))
        cm = np.sqrt((f(C) ** 2).sum(1)).max()
        eb = bound_fp8(xn[:, None], cm, d, sx[:, None], sc)
        worst = np.max(np.abs(keys - exact) / eb)
        print(f"{name} fp8: key error {worst:.3f} of the certificate bound")
        assert worst <= 1.0
