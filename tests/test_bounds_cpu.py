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


# ------------------------------- FP8 E4M3 tier -------------------------------
U8 = 2.0 ** -4


def e4m3(v) -> np.ndarray:
    """Round-to-nearest-even to E4M3 (3 mantissa bits, smallest normal 2^-6, subnormal spacing
    2^-9), in FP64; |v| below 448 (the scaling keeps it below 256)."""
    v = np.asarray(v, np.float64)
    a = np.abs(v)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    q = 2.0 ** (np.maximum(e, -6.0) - 3.0)
    return np.sign(v) * np.round(a / q) * q


def pow2_scale(mx):
    """The FP8 tier's power-of-two scale: 2^(e - 8) with mx = f 2^e, f in [0.5, 1) (1 for 0)."""
    mx = np.asarray(mx, np.float64)
    _, e = np.frexp(np.where(mx > 0, mx, 1.0))
    return np.where(mx > 0, np.ldexp(1.0, e - 8), 1.0)


def fp8_operands(X, C, cmax=None):
    """E4M3 copies as the FP8 tier makes them: per-row scales for X, one scale for C (from the
    bound of the largest center norm)."""
    X = np.asarray(X, np.float32)
    C = np.asarray(C, np.float32)
    sx = pow2_scale(np.abs(X).max(axis=1))
    cm = np.sqrt((C.astype(np.float64) ** 2).sum(1)).max() if cmax is None else cmax
    sc = float(pow2_scale(np.float32(cm * 1.0000001)))
    return e4m3(X / sx[:, None]), sx, e4m3(C / sc), sc


def bound_fp8(xn, cm, d, sx, sc):
    """Restatement of the kernel's bound_fp8 (FP64 here): |key - (x.c - |c|^2/2)|."""
    u = 2.0 ** -24
    ax, ac = sx * 2.0 ** -10, sc * 2.0 ** -10
    xc = xn * cm * 1.01
    slack = (1 + U8) * np.sqrt(d) * (ax * cm + ac * xn) + d * ax * ac
    op = (2 * U8 + U8 * U8) * xc + slack
    gacc = (d // 16 + 2) * 2.0 ** -21
    cc = 0.5 * cm * cm
    e = 0.5 * u * cm * cm + op + (gacc + 2.0 ** -18 + u) * (cc + 1.2 * xc + slack) \
        + (d + 2) * 1.2e-16 * (xn + cm) ** 2
    return e * 1.02


def test_e4m3_rounding_error():
    rng = np.random.default_rng(7)
    v = rng.standard_normal(200_000) * 10.0 ** rng.uniform(-4, 2.3, 200_000)
    v = v[np.abs(v) < 240]
    r = e4m3(v)
    normal = np.abs(v) >= 2.0 ** -6
    assert np.all(np.abs(r - v)[normal] <= U8 * np.abs(v[normal]))
    assert np.all(np.abs(r - v)[~normal] <= 2.0 ** -10 + 1e-300)
    # representable values are fixed points, and the grid has 8 steps per binade
    assert np.array_equal(e4m3(r), r)
    assert np.array_equal(e4m3(np.array([1.0625, 1.1875, 3.0e-3])), [1.0, 1.25, 2.0 ** -9 * 2])


def test_fp8_operand_bound_holds_exactly():
    """The operand part of bound_fp8 against exact arithmetic, with rows whose components span
    many magnitudes (subnormal E4M3 values included)."""
    rng = np.random.default_rng(8)
    for seed in range(4):
        X, C = data(seed, n=300, d=128, k=200)
        X[:50, :64] *= 1e-4  # components deep below the row's largest: subnormals after scaling
        X8, sx, C8, sc = fp8_operands(X, C)
        exact = X.astype(np.float64) @ C.astype(np.float64).T
        approx = (sx[:, None] * X8) @ (sc * C8).T
        xn = np.sqrt((X.astype(np.float64) ** 2).sum(1))
        cm = np.sqrt((C.astype(np.float64) ** 2).sum(1)).max()
        d = X.shape[1]
        ax, ac = sx * 2.0 ** -10, sc * 2.0 ** -10
        op = (2 * U8 + U8 * U8) * xn[:, None] * cm + (1 + U8) * np.sqrt(d) * (
            ax[:, None] * cm + ac * xn[:, None]) + d * ax[:, None] * ac
        assert np.all(np.abs(approx - exact) <= op)
