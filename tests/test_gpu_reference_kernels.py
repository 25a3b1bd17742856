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
