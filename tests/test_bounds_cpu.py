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


def f32_dist8_emulated(x, c):
    """rerank.cu f32_dist8<true> on one candidate, operation by operation in FP32: lane r of the
    8-lane group owns dimensions 4r..4r+3, 4r+32, ...; four FMA chains per lane, merged in two
    levels, then three butterfly levels (lane 0's view). The FMA is modelled as the exact FP64
    product plus the accumulator in FP64, rounded to FP32: that FP64 sum can itself round when
    the two differ widely in magnitude, a double rounding at most one FP32 ulp away from a true
    FMA on such steps -- far inside the bound's slack (errors reach ~11% of it here)."""
    d = len(x)
    f = np.float32
    lanes = []
    for r in range(8):
        acc = [f(0.0)] * 4
        for t in range(4 * r, d, 32):
            for comp in range(4):
                if t + comp < d:
                    u = f(x[t + comp]) - f(c[t + comp])  # FP32 subtraction, rounded
                    acc[comp] = f(np.float64(u) * np.float64(u) + np.float64(acc[comp]))
        lanes.append(f(f(acc[0] + acc[1]) + f(acc[2] + acc[3])))
    for o in (4, 2, 1):
        lanes = [f(lanes[i] + lanes[i ^ o]) for i in range(8)]
    return float(lanes[0])


def test_resolve_fp32_tier_bound():
    """The candidate resolve's first tier certifies with rel32 = 1.1 (m + 8) 2^-24, m =
    ceil(d/8): the emulated FP32 group distance stays within it of the exact distance."""
    from fractions import Fraction
    rng = np.random.default_rng(11)
    worst = 0.0
    for trial in range(60):
        d = int(rng.choice([7, 32, 96, 128, 130]))
        x = (rng.standard_normal(d) * 10.0 ** rng.uniform(-2, 3)).astype(np.float32)
        c = (x + rng.standard_normal(d).astype(np.float32) * np.float32(10.0 ** rng.uniform(-3, 1))
             ).astype(np.float32)
        if d % 4:  # the float4 path needs d % 4 == 0; the scalar path has the same bound
            continue
        exact = sum((Fraction(float(a)) - Fraction(float(b))) ** 2 for a, b in zip(x, c))
        v = f32_dist8_emulated(x, c)
        m = (d + 7) // 8
        rel32 = 1.1 * (m + 8) * 2.0 ** -24
        err = abs(Fraction(v) - exact)
        assert err <= Fraction(rel32) * exact + Fraction(2.0 ** -140), (d, float(err / exact))
        worst = max(worst, float(err / exact) / rel32)
    assert worst < 1.0


def test_ballot_peer_groups_equal_match_any():
    """update.cu/common.cuh warp_peers: one ballot per label bit gives, for every lane, the lanes
    holding the same label (-1 lanes form their own group), as __match_any_sync does."""
    rng = np.random.default_rng(3)

    def ballot(pred):
        return sum(1 << i for i, p in enumerate(pred) if p)

    for _ in range(3000):
        k = int(rng.choice([1, 2, 3, 16, 1000, 1024, 1025, 65536]))
        nbits = 0 if k <= 1 else (k - 1).bit_length()
        labels = [int(rng.choice([-1, rng.integers(k), rng.integers(min(k, 3))])) for _ in range(32)]
        valid = ballot([l >= 0 for l in labels])
        sets = [ballot([((l >> b) & 1) if l >= 0 else 1 for l in labels]) for b in range(nbits)]
        for i, l in enumerate(labels):
            m = valid if l >= 0 else ~valid & 0xFFFFFFFF
            for b in range(nbits):
                bit = ((l >> b) & 1) if l >= 0 else 1
                m &= sets[b] if bit else ~sets[b] & 0xFFFFFFFF
            assert m == ballot([x == l for x in labels])
