"""GPU parity of the reference's per-kernel C entry points against the oracle (bit-exact for
labels and the canonical FP64 sums; FP64 tolerances stated where the reduction order differs).
Device memory comes from torch; every call goes through the C-ABI library."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def closest_f(km, torch, A, B, nb, m0=0, extra=0):
    m, d = A.shape
    k = B.shape[1]
    At, Bt, nbt = dev(torch, A), dev(torch, B), dev(torch, nb)
    out = torch.full((m0 + m + extra,), -7, dtype=torch.int32, device="cuda")
    rc = km.ClosestCentersF(m0, m, d, At, k, Bt, None, None, nbt, (k + 63) // 64, None, None, out)
    torch.cuda.synchronize()
    assert rc == 0
    o = out.cpu().numpy()
    assert (o[:m0] == -7).all() and (o[m0 + m:] == -7).all()
    return o[m0:m0 + m]


def test_closest_centers_distance_known_answer(km, orc, torch_cuda):
    z = np.load(os.path.join(GOLD, "distance.npz"))
    a, b, lab = z["a"], z["b"], z["labels"]
    nb = (b.astype(np.float64) ** 2).sum(0).astype(np.float32)
    got = closest_f(km, torch_cuda, a, b, nb)
    assert np.array_equal(got, orc.closest_expansion(a, b, nb))
    assert np.array_equal(got, lab)


@pytest.mark.parametrize("m,d,k", [(1, 1, 1), (37, 3, 5), (300, 32, 64), (1000, 129, 200),
                                   (2048, 128, 1024), (513, 17, 130), (4000, 96, 300)])
def test_closest_centers_shapes(km, orc, torch_cuda, m, d, k):
    rng = np.random.default_rng(m * 7 + d * 13 + k)
    A = rng.standard_normal((m, d)).astype(np.float32)
    B = rng.standard_normal((d, k)).astype(np.float32)
    nb = (B.astype(np.float64) ** 2).sum(0).astype(np.float32)
    got = closest_f(km, torch_cuda, A, B, nb, m0=3, extra=2)
    assert np.array_equal(got, orc.closest_expansion(A, B, nb))


def test_closest_centers_ties_and_near_ties(km, orc, torch_cuda):
    rng = np.random.default_rng(11)
    d, k = 24, 40
    B = rng.standard_normal((d, k)).astype(np.float32)
    B[:, 7] = B[:, 3]     # duplicate centers: lowest index must win
    B[:, 20] = B[:, 19]
    A = np.concatenate([B.T[[3, 19, 5]], rng.standard_normal((500, d)).astype(np.float32)])
    A[3:100] = B.T[rng.integers(0, k, 97)] + 1e-4 * rng.standard_normal((97, d)).astype(np.float32)
    nb = (B.astype(np.float64) ** 2).sum(0).astype(np.float32)
    got = closest_f(km, torch_cuda, A, B, nb)
    want = orc.closest_expansion(A, B, nb)
    assert np.array_equal(got, want)
    assert got[0] == 3 and got[1] == 19


def test_closest_centers_d(km, orc, torch_cuda):
    rng = np.random.default_rng(5)
    m, d, k = 700, 33, 90
    A = rng.standard_normal((m, d))
    B = rng.standard_normal((d, k))
    nb = (B ** 2).sum(0)
    out = torch_cuda.zeros(m, dtype=torch_cuda.int32, device="cuda")
    rc = km.ClosestCentersD(0, m, d, dev(torch_cuda, A), k, dev(torch_cuda, B), None, None,
                            dev(torch_cuda, nb), 2, None, None, out)
    torch_cuda.cuda.synchronize()
    assert rc == 0
    assert np.array_equal(out.cpu().numpy(), orc.closest_expansion(A, B, nb))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_row_transform_minimum(km, orc, torch_cuda, dtype):
    rng = np.random.default_rng(9)
    m, n = 333, 257
    G = rng.standard_normal((m, n)).astype(dtype)
    G[:, 100] = G[:, 50]  # exact ties -> lowest index
    na = rng.random(m).astype(dtype)
    nbv = rng.random(n).astype(dtype)
    nbv[100] = nbv[50]
    m0 = 5
    out = torch_cuda.full((m0 + m,), -3, dtype=torch_cuda.int32, device="cuda")
    fn = km.rowTransformMinimumF if dtype == np.float32 else km.rowTransformMinimumD
    assert fn(m0, m, n, dev(torch_cuda, na), dev(torch_cuda, nbv), dev(torch_cuda, G), out) == 0
    torch_cuda.cuda.synchronize()
    ref = (orc.row_transform_min_f if dtype == np.float32 else orc.row_transform_min_d)(
        m0, na, nbv, G, m0 + m)
    got = out.cpu().numpy()
    assert np.array_equal(got[m0:], ref[m0:]) and (got[:m0] == -3).all()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_cluster_centers_tiles(km, orc, torch_cuda, dtype):
    torch = torch_cuda
    rng = np.random.default_rng(21)
    m, d, k = 5000, 19, 37
    X = rng.standard_normal((m, d)).astype(dtype)
    lab = rng.integers(0, k - 1, size=m).astype(np.int32)  # cluster k-1 stays empty
    Xt, lt = dev(torch, X), dev(torch, lab)
    big = torch.zeros(k * d * 2, dtype=torch.float32 if dtype == np.float32 else torch.float64,
                      device="cuda")
    cnt_big = torch.zeros(k, dtype=torch.int32, device="cuda")
    cen = torch.zeros((k, d), dtype=big.dtype, device="cuda")
    cnt = torch.zeros(k, dtype=torch.int32, device="cuda")
    fn = km.ClusterCentersF if dtype == np.float32 else km.ClusterCentersD
    # two tiles: rows [0, 3000) and [3000, 5000); indices are global (m0 offset)
    assert fn(0, 3000, d, k, False, Xt[:3000], lt, big, cnt_big, cen, cnt) == 0
    assert fn(3000, 2000, d, k, True, Xt[3000:], lt, big, cnt_big, cen, cnt) == 0
    torch.cuda.synchronize()
    c = cen.cpu().numpy()
    got_cnt = cnt.cpu().numpy()
    for j in range(k - 1):
        mem = X[lab == j].astype(np.float64)
        assert got_cnt[j] == len(mem)
        np.testing.assert_allclose(c[j], mem.sum(0) / len(mem), rtol=2e-7 if dtype == np.float32 else 1e-14,
                                   atol=1e-7 if dtype == np.float32 else 1e-15)
    assert got_cnt[k - 1] == 0 and np.isnan(c[k - 1]).all()


def test_cluster_centers_single_tile_bit_exact(km, orc, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(22)
    m, d, k = 20000, 24, 50
    X = (rng.standard_normal((m, d)) * 100).astype(np.float32)
    lab = rng.integers(0, k, size=m).astype(np.int32)
    big = torch.zeros(k * d * 2, dtype=torch.float32, device="cuda")
    cnt_big = torch.zeros(k, dtype=torch.int32, device="cuda")
    cen = torch.zeros((k, d), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(k, dtype=torch.int32, device="cuda")
    assert km.ClusterCentersF(0, m, d, k, True, dev(torch, X), dev(torch, lab), big, cnt_big, cen,
                              cnt) == 0
    torch.cuda.synchronize()
    want, wcnt, _ = orc.update(X, lab, k)
    assert np.array_equal(cen.cpu().numpy(), want)
    assert np.array_equal(cnt.cpu().numpy(), wcnt.astype(np.int32))


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_compactness(km, orc, torch_cuda, dtype):
    torch = torch_cuda
    rng = np.random.default_rng(31)
    m, d, k = 6000, 40, 25
    X = rng.standard_normal((m, d)).astype(dtype)
    Cn = rng.standard_normal((k, d)).astype(dtype)
    lab = rng.integers(0, k, size=m).astype(np.int32)
    buf = torch.zeros(8, dtype=torch.float32 if dtype == np.float32 else torch.float64,
                      device="cuda")
    fn = km.CompactnessF if dtype == np.float32 else km.CompactnessD
    Xt, lt, ct = dev(torch, X), dev(torch, lab), dev(torch, Cn)
    assert fn(0, 2500, False, d, k, Xt[:2500], lt, ct, buf) == 0
    assert fn(2500, 3500, True, d, k, Xt[2500:], lt, ct, buf) == 0
    torch.cuda.synchronize()
    want = ((X.astype(np.float64) - Cn.astype(np.float64)[lab]) ** 2).sum()
    got = float(buf[0].item())
    assert abs(got - want) <= (1e-6 if dtype == np.float32 else 1e-12) * want


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_row_col_normalize(km, torch_cuda, dtype):
    torch = torch_cuda
    rng = np.random.default_rng(41)
    m, n = 1234, 77
    A = rng.standard_normal((m, n)).astype(dtype)
    out = torch.zeros(m + 4, dtype=torch.float32 if dtype == np.float32 else torch.float64,
                      device="cuda")
    f = km.rowNormalizeF if dtype == np.float32 else km.rowNormalizeD
    assert f(4, m, n, dev(torch, A), out) == 0
    cout = torch.zeros(n, dtype=out.dtype, device="cuda")
    g = km.colNormalizeF if dtype == np.float32 else km.colNormalizeD
    assert g(m, n, dev(torch, A), cout) == 0
    torch.cuda.synchronize()
    rt = 1e-6 if dtype == np.float32 else 1e-13
    np.testing.assert_allclose(out.cpu().numpy()[4:], (A.astype(np.float64) ** 2).sum(1), rtol=rt)
    np.testing.assert_allclose(cout.cpu().numpy(), (A.astype(np.float64) ** 2).sum(0), rtol=rt)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("ra,ca,cb", [(1, 1, 1), (130, 77, 65), (1000, 128, 1024), (64, 0, 5),
                                      (5, 300, 3)])
def test_mat_mat_mult(km, torch_cuda, dtype, ra, ca, cb):
    """MatMatMultF/D (MatMatMult.cu:70-110): C = A B, row-major. The reference's own test
    (test/cpp/MatMultTests.cpp:85-107) compares against cuBLAS; here against FP64 (exact sums
    for the FP64 entry, via math.fsum on a sample) within the FMA chain's bound."""
    torch = torch_cuda
    rng = np.random.default_rng(ra * 7 + ca * 3 + cb)
    A = rng.standard_normal((ra, ca)).astype(dtype)
    B = rng.standard_normal((ca, cb)).astype(dtype)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    C = torch.full((ra, cb), 7.0, dtype=tdt, device="cuda")
    f = km.MatMatMultF if dtype == np.float32 else km.MatMatMultD
    assert f(ra, ca, dev(torch, A) if ca else None, cb, dev(torch, B) if ca else None, C) == 0
    torch.cuda.synchronize()
    got = C.cpu().numpy().astype(np.float64)
    if ca == 0:
        assert (got == 0).all()
        return
    eps = 2.0 ** -24 if dtype == np.float32 else 2.0 ** -53
    mag = np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64))
    bound = 1.01 * (ca + 1) * eps * mag
    if dtype == np.float32:
        exact = A.astype(np.float64) @ B.astype(np.float64)  # FP64 error << the FP32 bound
        assert np.all(np.abs(got - exact) <= bound)
    else:
        import math
        rr = rng.integers(0, ra, 40)
        cc = rng.integers(0, cb, 40)
        for r, c in zip(rr, cc):
            exact = math.fsum(float(A[r, t]) * float(B[t, c]) for t in range(ca))
            # the products themselves are exact only in the FP64 sum's own rounding: one more eps
            assert abs(got[r, c] - exact) <= bound[r, c] + eps * mag[r, c]


def test_mat_mat_mult_rejects_negative_sizes(km, torch_cuda):
    out = torch_cuda.zeros(4, device="cuda")
    assert km.MatMatMultF(-1, 2, None, 2, None, out) == 1  # ERROR_MATMATMULT
    assert km.MatMatMultD(2, 2, None, -3, None, out) == 1
