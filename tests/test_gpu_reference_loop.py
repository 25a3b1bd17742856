"""Whole Lloyd runs of this library against the REFERENCE's own kernels run in its loop order.

oracle/ref_loop.py drives the reference's ClosestCenters / ClusterCenters / Compactness kernels
(compiled from its sources) through the iterations of its computeStandard (kmeans.cpp:1185-1247)
from the same initial centers, in lockstep with this library's iterations (the plain FP32 tier
and the split BF16 tensor-core tier). The reference's labels are its FP32 arg-min and this
library's the FP64 arg-min. Until the first iteration whose labels differ, both runs agree:
labels equal, centers to FP32 summation error (1e-5 relative), SSE to 1e-6 relative (the
reference sums it in FP32). At that iteration every differing row must be an FP32 near tie --
its two labels' FP64 distances within the FP32 band -- and none a miss of this library. Both sides keep an empty cluster's previous center: the
reference's own 0/0 = NaN centers are outside what its assignment kernel defines."""
import numpy as np
import pytest

from kmeans_gb300.synthetic import mixture_numpy, sample_init
from oracle.ref_loop import trajectory_parity

pytestmark = pytest.mark.gpu

CASES = {
    # the 100,000 x 32, K=64 configuration, 20 iterations
    "c1": dict(n=100_000, d=32, k=64, iters=20, mean_lo=-10.0, mean_hi=10.0, std=(1.0, 1.0)),
    # the 4M x 128, K=1024 configuration's distribution at 200,000 rows, 10 iterations
    "c2_200k": dict(n=200_000, d=128, k=1024, iters=10, mean_lo=-20.0, mean_hi=20.0,
                    std=(0.3, 3.0)),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_whole_loop_against_reference_kernels(km, torch_cuda, case, capsys):
    c = CASES[case]
    X, _, _ = mixture_numpy(c["n"], c["d"], c["k"], seed=31, mean_lo=c["mean_lo"],
                            mean_hi=c["mean_hi"], std=c["std"])
    init = X[sample_init(c["n"], c["k"], seed=32)].copy()
    for tier, name in ((km.ASSIGN_FP32, "fp32"), (km.ASSIGN_BF16X3, "split bf16")):
        r = trajectory_parity(km, X, init, c["iters"], tier)
        if r is None:
            pytest.skip("oracle/_ref (the reference's kernels) not built")
        with capsys.disabled():
            print(f"\n{case} {name}: {r}")
        assert r["center_max_rel_diff_while_identical"] <= 1e-5
        assert r["sse_max_rel_diff_while_identical"] <= 1e-6
        f = r["first_difference"]
        if f is not None:
            assert f["library_label_not_its_fp64_argmin"] == 0
            # the two labels are a near tie: the reference's FP32 evaluation of ||c||^2 - 2 x.c
            # and the FP32 rounding of its center sums move distances by far less than this
            assert f["pair_relative_margin_max"] <= 1e-4, f
