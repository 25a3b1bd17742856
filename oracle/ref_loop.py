"""The reference's own Lloyd loop on the GPU -- TEST INFRASTRUCTURE ONLY.

Runs the reference's kernels (main/cuda/ClosestCenters.cu, ClusterCenters.cu, Compactness.cu,
compiled from its sources into oracle/_ref, launched by oracle/ref_kernels.cpp as its
ClosestCentersF / ClusterCentersF / CompactnessF do) in the order of its full-batch iteration,
computeStandard (main/cpp/kmeans.cpp:1185-1247):

  reset        clear centers_large, counts_large and the compactness partials; ||c||^2 of the
               D x K centers (kmeans.cpp:1142-1170, Normalize.cu colNormalize)
  closest      labels of every row (kmeans.cpp:910-1014)
  cluster      new centers K x D = sums / counts (kmeans.cpp:1018-1041)
  compactness  SSE of the rows against the NEW centers (kmeans.cpp:1044-1104), FP32
  transpose    the new centers back into the D x K operand (kmeans.cpp:1108-1139)

from given initial centers, on device-resident data, for a fixed number of iterations (the
reference's criterion < 0). Its host loop (kmeans.cpp) is not built (it needs a generated config.h
and cuBLAS); this restates its order. Used by tests/test_gpu_reference_loop.py and by bench.py's
reference arm to compare whole trajectories with this library's.
"""
from __future__ import annotations

import numpy as np


def run_reference_loop(X: np.ndarray, init: np.ndarray, iters: int, history: bool = False):
    """X: n x d, init: k x d (float32, host; k a multiple of 4). Returns (labels of the last
    assignment, centers k x d after the last update, per-iteration SSE in FP32 as the reference
    computes it, number of empty-cluster updates met) or None when the reference's kernels are
    not built. history: two more entries, every iteration's labels and input centers.

    An empty cluster keeps its previous center (this library's KMGB_EMPTY_KEEP): the reference
    writes 0/0 = NaN there (ClusterCenters.cu:81), and a NaN center in its assignment operand is
    outside what its kernels define, so the comparison runs both sides with the keep rule."""
    import torch

    import oracle
    ref = oracle.ref_kernels()
    if ref is None or not getattr(ref, "has_update", False):
        return None
    n, d = X.shape
    k = init.shape[0]
    dev = torch.device("cuda")
    rows_padded = (n + 63) // 64 * 64
    # the reference's kernels read past the logical matrices (see oracle/ref_kernels.cpp)
    A = torch.zeros((rows_padded + 1) * d + 16, dtype=torch.float32, device=dev)
    A[: n * d] = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32).ravel()).to(dev)
    B = torch.zeros((d + 16) * k, dtype=torch.float32, device=dev)
    Bv = B[: d * k].view(d, k)
    Bv.copy_(torch.from_numpy(np.ascontiguousarray(init.T, dtype=np.float32)).to(dev))
    normB = torch.empty(k, dtype=torch.float32, device=dev)
    ncolsc = (k + 63) // 64
    part = torch.empty(ncolsc * n, dtype=torch.float32, device=dev)
    pidx = torch.empty(ncolsc * n, dtype=torch.int32, device=dev)
    labels = torch.empty(n, dtype=torch.int32, device=dev)
    p = torch.cuda.get_device_properties(0).multi_processor_count * 8
    cl = torch.empty(p * k * d, dtype=torch.float32, device=dev)
    nl = torch.empty(p * k, dtype=torch.int32, device=dev)
    comp = torch.empty(p, dtype=torch.float32, device=dev)
    cen = torch.empty((k, d), dtype=torch.float32, device=dev)
    cnt = torch.empty(k, dtype=torch.int32, device=dev)
    sse, empties, hl, hc = [], 0, [], []
    for _ in range(iters):
        if history:
            hc.append(Bv.t().contiguous().cpu().numpy())
        cl.zero_()
        nl.zero_()
        comp.zero_()
        torch.sum(Bv * Bv, 0, out=normB)
        rc = ref.refk_closest_centers_f(0, n, d, A.data_ptr(), k, B.data_ptr(), normB.data_ptr(),
                                        ncolsc, part.data_ptr(), pidx.data_ptr(),
                                        labels.data_ptr())
        rc |= ref.refk_cluster_centers_f(n, d, k, A.data_ptr(), labels.data_ptr(), cl.data_ptr(),
                                         nl.data_ptr(), cen.data_ptr(), cnt.data_ptr())
        rc |= ref.refk_compactness_f(n, d, k, A.data_ptr(), labels.data_ptr(), cen.data_ptr(),
                                     comp.data_ptr())
        if rc != 0:
            raise RuntimeError(ref.refk_last_error().decode())
        if history:
            hl.append(labels.cpu().numpy())
        empties += int((cnt == 0).sum().item())
        Bv.copy_(torch.where((cnt > 0)[:, None], cen, Bv.t()).t())
        sse.append(float(comp[0].item()))
    torch.cuda.synchronize()
    out = (labels.cpu().numpy(), Bv.t().contiguous().cpu().numpy(), np.array(sse, np.float64),
           empties)
    return out + (hl, hc) if history else out


def near_tie_margins(X: np.ndarray, centers: np.ndarray, rows: np.ndarray, a: np.ndarray,
                     b: np.ndarray) -> np.ndarray:
    """FP64 |d^2(x, c_a) - d^2(x, c_b)| / d^2(x, c_a) of the given rows: how close to a tie the two
    labels the runs chose are, relative to the distance."""
    x = X[rows].astype(np.float64)
    ca = centers[a].astype(np.float64)
    cb = centers[b].astype(np.float64)
    da = ((x - ca) ** 2).sum(1)
    db = ((x - cb) ** 2).sum(1)
    return np.abs(da - db) / np.maximum(da, 1e-300)


def fp64_argmin_rows(X: np.ndarray, centers: np.ndarray, rows: np.ndarray):
    """FP64 arg-min (lowest index on ties) and the smallest squared distance of the given rows."""
    x = X[rows].astype(np.float64)
    c = centers.astype(np.float64)
    d2 = ((x[:, None, :] - c[None, :, :]) ** 2).sum(-1)
    return d2.argmin(1), d2.min(1)


def trajectory_parity(km, X: np.ndarray, init: np.ndarray, iters: int, tier: int):
    """This library's Lloyd iterations (a resident handle, one iteration at a time, empty clusters
    keeping their center) in lockstep with the reference's loop from the same initial centers.
    Up to the first iteration whose labels differ, both runs must agree (labels equal, centers
    and SSE to FP32 summation error); at that iteration every differing row must be an FP32 near
    tie: the two labels' FP64 distances (on this library's centers) within the FP32 band, this
    library's label the FP64 arg-min of its centers, and (reported) whether the reference's is
    the FP64 arg-min of its own. A near tie moves a
    point between two centers; on flat directions of the SSE (a Gaussian split between two
    centers) the runs then drift apart slowly, which is reported, not compared."""
    ref = run_reference_loop(X, init, iters, history=True)
    if ref is None:
        return None
    rlab, rcen, rsse, empties, hl, hc = ref
    n, d = X.shape
    k = init.shape[0]
    h = km.Handle(n, d, k, assign_tier=tier, max_iters=1, empty_policy=km.EMPTY_KEEP)
    h.set_data(X, False)
    h.set_centers(init, False)
    first, cen_rel, sse_rel, report = None, 0.0, 0.0, {}
    for t in range(iters):
        cin = h.centers()
        h.run(1)
        h.synchronize()
        lab = h.labels()
        s = float(h.sse(1)[-1])
        diff = np.nonzero(lab != hl[t])[0]
        if diff.size and first is None:
            first = t
            ex_ref, d2min = fp64_argmin_rows(X, hc[t], diff)
            ex_our, _ = fp64_argmin_rows(X, cin, diff)
            xr = X[diff].astype(np.float64)
            d2ref = ((xr - hc[t][hl[t][diff]].astype(np.float64)) ** 2).sum(1)
            pair = near_tie_margins(X, cin, diff, lab[diff], hl[t][diff])
            report = {"first_difference_iteration": t, "rows": diff[:16].tolist(),
                      "reference_label_not_its_fp64_argmin": int((hl[t][diff] != ex_ref).sum()),
                      "library_label_not_its_fp64_argmin": int((lab[diff] != ex_our).sum()),
                      "fp64_relative_margins": ((d2ref - d2min) / d2min)[:16].tolist(),
                      "pair_relative_margins": pair[:16].tolist(),
                      "pair_relative_margin_max": float(pair.max())}
        if first is None:
            nxt = h.centers()
            ref_next = hc[t + 1] if t + 1 < iters else rcen
            scale = np.maximum(np.abs(nxt), np.abs(ref_next)).max(axis=1, keepdims=True)
            cen_rel = max(cen_rel, float(np.max(np.abs(nxt - ref_next) / np.maximum(scale, 1e-30))))
            sse_rel = max(sse_rel, abs(s - rsse[t]) / abs(s))
        last_diff, last_sse = int(diff.size), abs(s - rsse[t]) / abs(s)
    h.close()
    return {"iterations": iters, "empty_cluster_updates": empties,
            "identical_iterations": iters if first is None else first,
            "center_max_rel_diff_while_identical": cen_rel,
            "sse_max_rel_diff_while_identical": sse_rel, "first_difference": report or None,
            "final_label_differences": last_diff, "final_sse_rel_diff": last_sse}
