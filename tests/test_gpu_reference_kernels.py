"""The oracle's assignment rule pinned against the REFERENCE's own GPU kernels.

oracle/_ref holds the reference's main/cuda/ClosestCenters.cu compiled from its sources for
sm_103a and a loader that launches it the way the reference's ClosestCentersF does
(ClosestCenters.cu:181-231, 312-315). The reference evaluates ||c||^2 - 2 x.c in FP32 with its
own summation order, the oracle the FP64 arg-min, so labels must agree wherever the FP64 margin
between the best and second-best center exceeds the FP32 evaluation error, and exact ties
(duplicate centers) must go to the lowest index in both. Also times the reference kernels on the
4M x 128, K=1024 workload next to this library's assignment.
"""
import math

import numpy as np
import pytest

import oracle
from kmeans_gb300.synthetic import mixture_numpy, sample_init

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(torch_cuda):
    L = oracle.ref_kernels()
    if L is None:
        pytest.skip("oracle/_ref (the reference's kernels) not built")
    return L


def run_ref(ref, torch, X, Cn, time_it=False):
    """Reference labels for X (n x d) against centers Cn (k x d); buffers padded the way the
    reference's kernels read them (see oracle/ref_kernels.cpp)."""
    n, d = X.shape
    k = Cn.shape[0]
    assert k % 4 == 0
    rows_padded = (n + 63) // 64 * 64
    dev = torch.device("cuda")
    A = torch.zeros((rows_padded + 1) * d + 16, dtype=torch.float32, device=dev)
    A[: n * d] = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32).ravel()).to(dev)
    B = torch.zeros((d + 16) * k, dtype=torch.float32, device=dev)
    B[: d * k] = torch.from_numpy(np.ascontiguousarray(Cn.T, dtype=np.float32).ravel()).to(dev)
    Ct = torch.from_numpy(np.ascontiguousarray(Cn, dtype=np.float32)).to(dev)
    normB = (Ct * Ct).sum(1).contiguous()
    ncolsc = (k + 63) // 64
    part = torch.empty(ncolsc * n, dtype=torch.float32, device=dev)
    pidx = torch.empty(ncolsc * n, dtype=torch.int32, device=dev)
    labels = torch.full((n,), -1, dtype=torch.int32, device=dev)
    args = (0, n, d, A.data_ptr(), k, B.data_ptr(), normB.data_ptr(), ncolsc, part.data_ptr(),
            pidx.data_ptr(), labels.data_ptr())
    ms = None
    if time_it:
        rc = ref.refk_closest_centers_f(*args)
        assert rc == 0, ref.refk_last_error()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        e0.record(torch.cuda.default_stream())
        for _ in range(reps):
            rc = ref.refk_closest_centers_f(*args)
        e1.record(torch.cuda.default_stream())
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
    rc = ref.refk_closest_centers_f(*args)
    assert rc == 0, ref.refk_last_error()
    torch.cuda.synchronize()
    return labels.cpu().numpy(), ms


def fp64_top2(X, Cn):
    x = X.astype(np.float64)
    c = Cn.astype(np.float64)
    d2 = (x * x).sum(1)[:, None] - 2.0 * x @ c.T + (c * c).sum(1)[None, :]
    part = np.partition(d2, 1, axis=1)
    return part[:, 0], part[:, 1], (x * x).sum(1), (c * c).sum(1).max()


@pytest.mark.parametrize("n,d,k", [(20000, 32, 64), (20000, 128, 256), (8000, 7, 128),
                                   (8000, 40, 1024), (5000, 129, 64)])
def test_reference_kernels_agree_with_the_oracle(ref, torch_cuda, n, d, k):
    X, _, _ = mixture_numpy(n, d, k, seed=n + d + k)
    Cn = X[sample_init(n, k, seed=4)].astype(np.float32)
    lab_ref, _ = run_ref(ref, torch_cuda, X, Cn)
    lab_orc = oracle.assign(X, Cn)
    assert lab_ref.min() >= 0 and lab_ref.max() < k
    b1, b2, xx, cc = fp64_top2(X, Cn)
    # the reference's FP32 value ||c||^2 - 2 x.c is within ~(d+2) 2^-24 (||x||^2 + ||c||^2) of
    # the exact one (x3 margin); a label may differ from the FP64 arg-min only inside that band
    band = 3.0 * (d + 2) * 2.0 ** -24 * (xx + cc)
    differ = lab_ref != lab_orc
    assert np.all((b2 - b1)[differ] <= 2 * band[differ]), "a well-separated label differs"
    assert differ.mean() <= 1e-3
    print(f"n={n} d={d} k={k}: {differ.sum()} of {n} labels differ, all inside the FP32 band")


def test_reference_kernels_break_exact_ties_by_lowest_index(ref, torch_cuda):
    rng = np.random.default_rng(8)
    d, k = 24, 64
    Cn = rng.uniform(-3, 3, size=(k, d)).astype(np.float32)
    Cn[17] = Cn[5]
    Cn[40:44] = Cn[33]
    X = np.concatenate([Cn[[5, 17, 33, 41]] + rng.normal(0, 0.05, size=(4, d)).astype(np.float32),
                        Cn[rng.integers(0, k, 2000)]]).astype(np.float32)
    lab_ref, _ = run_ref(ref, torch_cuda, X, Cn)
    lab_orc = oracle.assign(X, Cn)
    assert np.array_equal(lab_ref, lab_orc)
    assert not np.isin(lab_ref, [17, 40, 41, 42, 43]).any()


def test_reference_kernels_time_on_the_4m_workload(ref, torch_cuda, km):
    torch = torch_cuda
    n, d, k = 4_000_000, 128, 1024
    from kmeans_gb300.synthetic import mixture_torch
    Xt, _, _ = mixture_torch(n, d, k, seed=1234, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0))
    idx = torch.from_numpy(sample_init(n, k, seed=99)).cuda()
    Cn = Xt[idx].cpu().numpy()
    X = Xt.cpu().numpy()
    del Xt
    lab_ref, ms = run_ref(ref, torch, X, Cn, time_it=True)
    # sampled agreement with the FP64 oracle
    rows = np.random.default_rng(0).choice(n, 20000, replace=False)
    lab_orc = oracle.assign(X[rows], Cn)
    b1, b2, xx, cc = fp64_top2(X[rows], Cn)
    band = 3.0 * (d + 2) * 2.0 ** -24 * (xx + cc)
    differ = lab_ref[rows] != lab_orc
    assert np.all((b2 - b1)[differ] <= 2 * band[differ])
    tflops = 2.0 * n * k * d / (ms / 1000.0) / 1e12
    print(f"reference ClosestCentersF (FP32 SIMT, its own kernels) on 4M x 128, K=1024: "
          f"{ms:.2f} ms per assignment = {tflops:.1f} TFLOP/s")


# --- the reference's center and compactness kernels (ClusterCenters.cu, Compactness.cu) ---------

def ref_blocks(torch):
    """getMaxConcurrentBlocks() of the reference (KmeansCudaKernels.h:138-149): SMs x 8."""
    return torch.cuda.get_device_properties(0).multi_processor_count * 8


def run_ref_update(ref, torch, X, labels, k, centers_for_sse):
    if not getattr(ref, "has_update", False):
        pytest.skip("the reference's ClusterCenters/Compactness cubins not built")
    n, d = X.shape
    p = ref_blocks(torch)
    dev = torch.device("cuda")
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
    Ld = torch.from_numpy(np.ascontiguousarray(labels, dtype=np.int32)).to(dev)
    cl = torch.zeros(p * k * d, dtype=torch.float32, device=dev)
    nl = torch.zeros(p * k, dtype=torch.int32, device=dev)
    cen = torch.empty((k, d), dtype=torch.float32, device=dev)
    cnt = torch.empty(k, dtype=torch.int32, device=dev)
    rc = ref.refk_cluster_centers_f(n, d, k, Xd.data_ptr(), Ld.data_ptr(), cl.data_ptr(),
                                    nl.data_ptr(), cen.data_ptr(), cnt.data_ptr())
    assert rc == 0, ref.refk_last_error()
    Cs = torch.from_numpy(np.ascontiguousarray(centers_for_sse, dtype=np.float32)).to(dev)
    comp = torch.zeros(p, dtype=torch.float32, device=dev)
    rc = ref.refk_compactness_f(n, d, k, Xd.data_ptr(), Ld.data_ptr(), Cs.data_ptr(),
                                comp.data_ptr())
    assert rc == 0, ref.refk_last_error()
    torch.cuda.synchronize()
    return cen.cpu().numpy(), cnt.cpu().numpy(), float(comp[0].item()), p


def emulate_reference_centers(X, labels, k, p):
    """The reference's FP32 summation order for the centers (ClusterCenters.cu:3-23, 47-87):
    block b adds rows b, b+p, b+2p, ... into its own partial sums (one row per block per round);
    one block per center then adds the p partials in block order and divides (0/0 = NaN)."""
    n, d = X.shape
    part = np.zeros((p, k, d), dtype=np.float32)
    for r0 in range(0, n, p):
        rows = np.arange(r0, min(n, r0 + p))
        part[rows - r0, labels[rows]] += X[rows]
    total = np.zeros((k, d), dtype=np.float32)
    for b in range(p):
        total += part[b]
    counts = np.bincount(labels, minlength=k).astype(np.int32)
    with np.errstate(invalid="ignore", divide="ignore"):
        centers = total / counts[:, None].astype(np.float32)
    return centers, counts


@pytest.mark.parametrize("n,d,k", [(20000, 32, 64), (12000, 130, 16), (9000, 7, 100)])
def test_reference_center_and_compactness_kernels_agree_with_the_oracle(ref, torch_cuda, n, d,
                                                                        k):
    X, _, _ = mixture_numpy(n, d, k, seed=3 * n + d)
    X = X.astype(np.float32)
    init = X[sample_init(n, k, seed=5)].astype(np.float32)
    init[[1, k - 2]] = 1e4  # two centers no point is closest to: empty clusters
    labels = oracle.assign(X, init)
    assert not np.isin(labels, [1, k - 2]).any()
    newc, cnt_orc, sums = oracle.update(X, labels, k, old_centers=init)
    cen_ref, cnt_ref, sse_ref, p = run_ref_update(ref, torch_cuda, X, labels, k, newc)

    # the loader runs the reference's kernels in the reference's own summation order
    cen_emu, cnt_emu = emulate_reference_centers(X, labels, k, p)
    assert np.array_equal(cnt_ref, cnt_emu)
    assert np.array_equal(cen_ref, cen_emu, equal_nan=True)

    # counts are exact; empty clusters come out as 0/0 = NaN in the reference
    assert np.array_equal(cnt_ref, cnt_orc.astype(np.int32))
    empty = cnt_orc == 0
    assert empty[[1, k - 2]].all()
    assert np.isnan(cen_ref[empty]).all()

    # against the oracle's exact sums: a sequential FP32 sum of c terms is within
    # (c - 1) u sum|x| of the exact one, and the division adds u |mean| (u = 2^-24)
    u = 2.0 ** -24
    full = ~empty
    c = cnt_orc[full].astype(np.float64)[:, None]
    abs_sum = np.zeros((k, d))
    np.add.at(abs_sum, labels, np.abs(X.astype(np.float64)))
    exact = sums[full] / c
    bound = 1.01 * ((c - 1) * u * abs_sum[full] / c + u * np.abs(exact)) + 1e-30
    err = np.abs(cen_ref[full].astype(np.float64) - exact)
    assert np.all(err <= bound), float((err / bound).max())
    # the oracle's own centers are the exact means rounded once
    assert np.array_equal(newc[full], exact.astype(np.float32))

    # compactness: every term is positive, so the FP32 result is within (depth + 3) u of the
    # FP64 sum, depth = rows per thread + the two 128-way trees + partials per thread
    sse_orc = oracle.sse(X, labels, newc)
    depth = math.ceil(n / p) * math.ceil(d / 128) + 7 + math.ceil(p / 128) + 7
    assert abs(sse_ref - sse_orc) <= 1.01 * (depth + 3) * u * sse_orc, (sse_ref, sse_orc)
    print(f"n={n} d={d} k={k}: centers bit-equal to the reference's FP32 order, max "
          f"{float((err / bound).max()):.3f} of the bound from the oracle; SSE rel "
          f"{abs(sse_ref - sse_orc) / sse_orc:.2e}")
