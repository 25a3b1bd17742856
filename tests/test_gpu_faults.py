"""Failure paths, through the C-ABI, without faulting the GPU.

Host-side injection (kmgb_debug_fail_nth) makes one allocation, copy or kernel launch of a call
fail as the CUDA call would have failed: the call must return the kmeansErrorStatus of the phase
it was in (the reference reports failures only through these codes, kmeans.hpp:44-59), leave a
message, give back every byte it took from the library's memory pool, and leave the context usable
(the next call returns the oracle's result). A bounded device wait is made to run out by
withholding one TMA load of the FP32 assignment (kmgb_debug_withhold_stage) with a short wait
limit: every load issued before it has been consumed, so nothing is left in flight, and the kernel
reports the timeout through the device error word."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, D, K, ITERS = 5000, 24, 12, 3


@pytest.fixture()
def no_graphs():
    old = os.environ.get("KMGB_GRAPHS")
    os.environ["KMGB_GRAPHS"] = "0"  # kernel-by-kernel launches: the event order is fixed
    yield
    if old is None:
        os.environ.pop("KMGB_GRAPHS")
    else:
        os.environ["KMGB_GRAPHS"] = old


def data():
    from kmeans_gb300.synthetic import mixture_numpy, sample_init
    X, _, _ = mixture_numpy(N, D, K, seed=21)
    return X, X[sample_init(N, K, seed=22)].copy()


def call(km, X, init, tier):
    try:
        res = km.lloyd(X, K, init=init, max_iters=ITERS, assign_tier=tier)
        return 0, res
    except km.KmeansError as e:
        return e.code, None


def check_clean(km, torch, orc, X, init, tier, base_used):
    torch.cuda.synchronize()
    assert km.debug_pool_used_bytes() == base_used, "pool memory not given back"
    rc, res = call(km, X, init, tier)
    assert rc == 0
    st, c, lab, sse, it = orc.lloyd(X, init, ITERS)
    assert np.array_equal(res.labels, lab) and np.array_equal(res.centers, c)


@pytest.mark.parametrize("tier_name", ["fp32", "bf16x3"])
def test_injected_failures_return_phase_codes_and_release_memory(km, orc, torch_cuda, no_graphs,
                                                                  tier_name):
    torch = torch_cuda
    tier = {"fp32": km.ASSIGN_FP32, "bf16x3": km.ASSIGN_BF16X3}[tier_name]
    X, init = data()
    call(km, X, init, tier)  # warm: module loading, pool creation
    torch.cuda.synchronize()
    base = km.debug_pool_used_bytes()
    assert base >= 0
    valid = set(range(1, 13))
    seen = {}
    for kind in (km.FAULT_ALLOC, km.FAULT_COPY, km.FAULT_LAUNCH):
        nth = 1
        while True:
            km.debug_fail_nth(kind, nth)
            rc, res = call(km, X, init, tier)
            km.debug_fail_nth(kind, 0)
            if rc == 0:  # more events asked for than the call has: it ran untouched
                break
            assert rc in valid, (kind, nth, rc)
            assert km.last_error(), (kind, nth)
            seen[(kind, nth)] = rc
            check_clean(km, torch, orc, X, init, tier, base)
            nth += 1
            assert nth < 200
    # the first allocation is the handle's arena (KMEANS_ERROR_BUILDDATA); the second copy
    # uploads the initial centers (KMEANS_ERROR_INITIALIZE)
    assert seen[(km.FAULT_ALLOC, 1)] == km.KMEANS_ERROR_BUILDDATA
    assert seen[(km.FAULT_COPY, 2)] == km.KMEANS_ERROR_INITIALIZE
    codes = set(seen.values())
    # every phase of an iteration was reached by some launch failure: center preparation
    # (reset), assignment / re-rank (closest centers) and the update (cluster centers)
    assert {km.KMEANS_ERROR_RESET, km.KMEANS_ERROR_CLOSEST_CENTERS, km.KMEANS_ERROR_CLUSTER_CENTERS} <= {seen[k] for k in seen if k[0] == km.FAULT_LAUNCH}, seen
    assert codes <= valid


def test_withheld_tma_load_times_out_and_reports(km, orc, torch_cuda, no_graphs):
    torch = torch_cuda
    from kmeans_gb300.synthetic import mixture_numpy, sample_init
    # D = 100: four 32-float k-blocks per center chunk, so every CTA's pipeline has 4 steps
    X, _, _ = mixture_numpy(N, 100, K, seed=23)
    init = X[sample_init(N, K, seed=24)].copy()
    call(km, X, init, km.ASSIGN_FP32)
    torch.cuda.synchronize()
    base = km.debug_pool_used_bytes()
    # step 2 of every CTA's pipeline is never loaded; each wait gives up after 2e6 SM cycles
    # (about a millisecond)
    km.debug_withhold_stage(2, 2_000_000)
    try:
        rc, _ = call(km, X, init, km.ASSIGN_FP32)
    finally:
        km.debug_withhold_stage(0, 0)
    assert rc == km.KMEANS_ERROR_CLOSEST_CENTERS
    assert "device error word 1" in km.last_error()  # KMGB_DEV_TIMEOUT_FULL
    check_clean(km, torch, orc, X, init, km.ASSIGN_FP32, base)


def test_failure_inside_graph_capture_falls_back(km, orc, torch_cuda):
    """With graphs on, a launch failure injected while the iteration is being captured aborts
    the capture; the run then launches kernel by kernel and returns the oracle's result."""
    X, init = data()
    call(km, X, init, km.ASSIGN_FP32)
    # the launches of one-time work come first (norms); the capture starts with the first
    # iteration's center preparation
    km.debug_fail_nth(km.FAULT_LAUNCH, 2)
    try:
        rc, res = call(km, X, init, km.ASSIGN_FP32)
    finally:
        km.debug_fail_nth(km.FAULT_LAUNCH, 0)
    assert rc == 0
    st, c, lab, sse, it = orc.lloyd(X, init, ITERS)
    assert np.array_equal(res.labels, lab) and np.array_equal(res.centers, c)
