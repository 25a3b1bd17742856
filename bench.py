#!/usr/bin/env python
"""Benchmark of the GB300 Lloyd hot path.

A step is one Lloyd iteration (assignment + center update + SSE) over the resident data set of
the 4,000,000 x 128, K=1024 workload (1024 anisotropic Gaussians, per-component diagonal std
log-uniform in [0.3, 3], means uniform in [-20, 20]^128, initial centers a seeded sample of
points; synthetic, generated on the device). Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--tier bf16x3|bf16|fp32] [--impl reference]

`value` is Lloyd iterations/s with the data resident in HBM (CUDA events on the library's
stream); `e2e` is the same metric through the public C-ABI one-shot call (kmgb_lloyd_f32) from
pinned host memory (`pageable_value`: the same from pageable memory), host<->device copies
included, one call running the workload's 30 iterations; `roofline` covers the assignment kernel
(2*N*K*D FLOP per launch, per-launch time from CUDA events bracketing it inside the timed
region; `tensor_*` counts the tensor-core products the tier actually issues, three per element
in the split tier; `traffic` is the DRAM bytes of one launch from an ncu capture, scaled to N);
`update_roofline` puts the update phase (sort, piece sums, finalize, SSE; N*D*4 + N*4 + K*D*8
bytes per iteration) against the measured HBM copy rate; `cpu_baseline` is the CPU restatement (oracle FP32 port, all host threads) on a sample.
The reference arm (--impl reference) times that CPU path: the reference has no CPU
implementation of its own and its host code is not built (its sources are only in the x86
development container; its driver also needs a CMake-generated config.h and cuBLAS). Its line also
carries `reference_gpu`: the reference's own GPU kernels (compiled from its sources into
oracle/_ref, launched as its ClosestCentersF, ClusterCentersF and CompactnessF do) timed on the
same workload, for one assignment pass and for one device-resident iteration.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, D, K = 4_000_000, 128, 1024
NUM_CENTERS = K
L2_BYTES = 129e6  # GB300's L2
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one assignment launch per row of
# X, from one ncu capture of the current split-tier kernel on the 1,000,000 x 128, K=1024 case
# (517.0 MB read + 7.6 MB written). X is read once per launch and C stays in L2, so the traffic
# of a launch grows in proportion to its rows.
TRAFFIC_BYTES_PER_ROW = {"bf16x3": 524.64e6 / 1_000_000}
# tensor-core products per distance element: the split tier evaluates x_hi.c_hi + x_hi.c_lo +
# x_lo.c_hi
TENSOR_PRODUCTS = {"bf16x3": 3, "bf16": 1}
# the workload's run is 30 Lloyd iterations: the end-to-end leg makes that one public call
E2E_ITERS = 30
METRIC = "Lloyd iter/s (N=4M, D=128, K=1024), labels = FP64 arg-min"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return j.get("bf16_tflops", 1900.0), j.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler for the timed region."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}",
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for nme, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nme)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def replica_rate(ms: float, steps: int, world: int, dist=None, device: str = "cuda"):
    """N ranks, each processing its own 4M-row shard for `steps` iterations: the slowest rank's
    timed region sets the whole job's time (max over ranks), and the job's rate counts every
    rank's iterations over its rows. Returns (max ms, iter/s)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * steps / (ms / 1000.0)


def host_info():
    """Host cores and CPU model of the machine the CPU baseline runs on."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except Exception:  # noqa: BLE001 - informational
        pass
    return {"nproc": os.cpu_count(), "cpu_model": model}


def workload_host(n=N):
    """The GPU arm's data set and initial centers (same generator, seed and picks), on the host."""
    import torch
    from kmeans_gb300.synthetic import mixture_torch, sample_init
    X, _, _ = mixture_torch(n, D, K, seed=1234, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0))
    Xh = X.cpu().numpy()
    del X
    torch.cuda.empty_cache()
    return Xh, Xh[sample_init(n, K, seed=99)].copy()


def cpu_baseline(X, init, steps: int, warmup: int = 1):
    """The oracle's FP32 port of the reference loop (CPU restatement, OpenMP, all host threads)
    over ALL rows of the workload: `warmup` untimed iterations, then `steps` timed iterations,
    each continuing from the previous one's centers (one full Lloyd iteration per step)."""
    import oracle
    C = np.ascontiguousarray(init, dtype=np.float32)
    for _ in range(max(0, warmup)):
        C, _, _ = oracle.port_lloyd(X, C, 1)
    times = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        C, _, _ = oracle.port_lloyd(X, C, 1)
        times.append(time.perf_counter() - t0)
    t = float(np.sum(times))
    info = host_info()
    return {"value": len(times) / t, "unit": "iter/s", "cores": oracle.num_threads(),
            "kind": "port",
            "sample": f"{len(times)} full Lloyd iterations over all {len(X)} rows (D={D}, "
                      f"K={K}) of the GPU arm's data and initial centers, FP32 port of the "
                      f"reference loop, {warmup} untimed first",
            "seconds_per_iteration": t / len(times), **info}


def reference_gpu_kernels(N=N, D=D, K=K, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0)):
    """The reference's own GPU kernels (main/cuda/ClosestCenters.cu, ClusterCenters.cu and
    Compactness.cu, compiled from its sources into oracle/_ref and launched as its
    ClosestCentersF / ClusterCentersF / CompactnessF do) on an N x D, K workload (default: the
    4M x 128, K=1024 one). Times, with CUDA events on the legacy default stream, (1) one
    assignment pass and (2) one full-batch iteration as the reference's computeStandard runs it
    on the GPU: its per-iteration reset (kmeans.cpp:1142-1170: clears of centers_large,
    counts_large and the compactness partials; ||c||^2 of the centers), the assignment, the
    center update and the compactness (kmeans.cpp:1019-1060), the new centers transposed back
    for the next assignment. None when oracle/_ref or a GPU is absent."""
    try:
        import torch
        import oracle
        if not torch.cuda.is_available():
            return None
        ref = oracle.ref_kernels()
        if ref is None:
            return None
        from kmeans_gb300.synthetic import mixture_torch, sample_init
        X, _, _ = mixture_torch(N, D, K, seed=1234, mean_lo=mean_lo, mean_hi=mean_hi, std=std)
        C = X[torch.from_numpy(sample_init(N, K, seed=99)).cuda()]
        rows_padded = (N + 63) // 64 * 64
        # the reference's kernels read past the logical matrices (see oracle/ref_kernels.cpp)
        A = torch.zeros((rows_padded + 1) * D + 16, dtype=torch.float32, device="cuda")
        A[: N * D] = X.reshape(-1)
        del X
        B = torch.zeros((D + 16) * K, dtype=torch.float32, device="cuda")
        B[: D * K] = C.t().contiguous().reshape(-1)
        normB = (C * C).sum(1).contiguous()
        ncolsc = (K + 63) // 64
        part = torch.empty(ncolsc * N, dtype=torch.float32, device="cuda")
        pidx = torch.empty(ncolsc * N, dtype=torch.int32, device="cuda")
        labels = torch.empty(N, dtype=torch.int32, device="cuda")
        args = (0, N, D, A.data_ptr(), K, B.data_ptr(), normB.data_ptr(), ncolsc, part.data_ptr(),
                pidx.data_ptr(), labels.data_ptr())
        for _ in range(2):
            if ref.refk_closest_centers_f(*args) != 0:
                return None
        torch.cuda.synchronize()
        stream = torch.cuda.default_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5 if N * K * D > 1e10 else 50
        e0.record(stream)
        for _ in range(reps):
            ref.refk_closest_centers_f(*args)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out = {"kernels": "reference main/cuda/ClosestCenters.cu (ClosestCentersF), built from "
                          "its sources for sm_103a", "assign_ms": ms,
               "assign_tflops": 2.0 * N * K * D / (ms / 1000.0) / 1e12}
        if getattr(ref, "has_update", False):
            p = torch.cuda.get_device_properties(0).multi_processor_count * 8
            cl = torch.empty(p * K * D, dtype=torch.float32, device="cuda")
            nl = torch.empty(p * K, dtype=torch.int32, device="cuda")
            comp = torch.empty(p, dtype=torch.float32, device="cuda")
            cen = torch.empty((K, D), dtype=torch.float32, device="cuda")
            cnt = torch.empty(K, dtype=torch.int32, device="cuda")
            Bv = B[: D * K].view(D, K)

            def iteration():
                cl.zero_()
                nl.zero_()
                comp.zero_()
                torch.sum(Bv * Bv, 0, out=normB)
                rc = ref.refk_closest_centers_f(*args)
                rc |= ref.refk_cluster_centers_f(N, D, K, A.data_ptr(), labels.data_ptr(),
                                                 cl.data_ptr(), nl.data_ptr(), cen.data_ptr(),
                                                 cnt.data_ptr())
                rc |= ref.refk_compactness_f(N, D, K, A.data_ptr(), labels.data_ptr(),
                                             cen.data_ptr(), comp.data_ptr())
                # an empty cluster (0/0 = NaN in the reference) keeps its old center here, so
                # every center the next assignment sees is finite and every label in range
                Bv.copy_(torch.where((cnt > 0)[:, None], cen, Bv.t()).t())
                return rc

            for _ in range(2):
                if iteration() != 0:
                    out["iteration_unavailable"] = ref.refk_last_error().decode()[:200]
                    return out
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                iteration()
            e1.record(stream)
            torch.cuda.synchronize()
            it_ms = e0.elapsed_time(e1) / reps
            out["kernels"] += ", ClusterCenters.cu, Compactness.cu"
            out["iteration_ms"] = it_ms
            out["iter_per_s"] = 1000.0 / it_ms
            out["note"] = ("iteration = the reference's per-iteration clears + ||c||^2, "
                           "ClosestCentersF, ClusterCentersF, CompactnessF and the centers' "
                           "transpose (empty clusters keep their old center), device-resident; "
                           "its host loop and convergence copy are not timed")
        else:
            out["note"] = "assignment pass only (center/compactness cubins not built)"
        return out
    except Exception as e:  # noqa: BLE001 - an informational extra
        return {"unavailable": str(e)[:200]}


def reference_loop_parity():
    """Whole runs of this library (FP32 and split BF16 tiers) in lockstep with the reference's own
    kernels run in its loop order from the same initial centers (oracle/ref_loop.py): the
    100,000 x 32, K=64 configuration for its 20 iterations and the 4M x 128 distribution at
    200,000 rows for 10. Reports how many iterations agree exactly, the center / SSE differences
    while they do, and the first differing iteration's rows with their FP64 margins."""
    try:
        import torch
        if not torch.cuda.is_available():
            return None
        import kmeans_gb300 as km
        from kmeans_gb300.synthetic import mixture_numpy, sample_init
        from oracle.ref_loop import trajectory_parity
        km.build()
        out = {}
        for name, (n, d, k, iters, lo, hi, std) in {
                "100000x32_K64": (100_000, 32, 64, 20, -10.0, 10.0, (1.0, 1.0)),
                "200000x128_K1024": (200_000, 128, 1024, 10, -20.0, 20.0, (0.3, 3.0))}.items():
            X, _, _ = mixture_numpy(n, d, k, seed=31, mean_lo=lo, mean_hi=hi, std=std)
            init = X[sample_init(n, k, seed=32)].copy()
            for tier, tn in ((km.ASSIGN_FP32, "fp32"), (km.ASSIGN_BF16X3, "bf16x3")):
                r = trajectory_parity(km, X, init, iters, tier)
                if r is None:
                    return {"unavailable": "oracle/_ref (the reference's kernels) not built"}
                out[f"{name}_{tn}"] = r
        return out
    except Exception as e:  # noqa: BLE001 - an informational extra
        return {"unavailable": str(e)[:200]}


def reference_arm(args, rank: int):
    if rank != 0:
        return
    X, init = workload_host()
    cb = cpu_baseline(X, init, steps=args.steps, warmup=min(args.warmup, 2))
    del X
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "iter/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 / cb["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "lloyd_4Mx128_K1024", "n": N, "d": D, "k": K},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample",
                                                "nproc", "cpu_model")},
            "e2e": {"value": cb["value"], "unit": "iter/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "reference_gpu": reference_gpu_kernels(),
            "reference_gpu_100kx32_K64": reference_gpu_kernels(100_000, 32, 64, -10.0, 10.0,
                                                                (1.0, 1.0)),
            "reference_loop_parity": reference_loop_parity()}
    print(json.dumps(line), flush=True)


def accuracy_and_plain_fp32(km, torch, h, X, n, k):
    """Outside the timed region. One more iteration of the measured handle from its current
    centers C gives labels L, centers C' and SSE s. Checked against an independent FP64
    evaluation on the GPU (torch, float64): L on a 65,536-row sample against the arg-min of the
    direct squared distances to C (first index on ties; NaN centers of empty clusters never
    win), C' against the FP64 means of the rows
    of each label, s against the FP64 sum of ||x - C'[label]||^2 over all rows. Then the plain
    FP32 tier from the same C: its labels must equal L, and its iteration rate is the
    denominator of the tensor-core speed-up."""
    d = X.shape[1]
    C = torch.from_numpy(h.centers()).cuda()
    h.run(1)
    h.synchronize()
    L = torch.from_numpy(h.labels()).cuda().long()
    C1 = torch.from_numpy(h.centers()).cuda()
    sse = float(h.sse(1)[-1])  # the SSE of this run's single iteration
    C64 = C.double()
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    idx = torch.randperm(n, device="cuda", generator=g)[:65536]
    mism = 0
    for r0 in range(0, idx.numel(), 1024):
        xs = X[idx[r0:r0 + 1024]].double()
        dist = ((xs[:, None, :] - C64[None, :, :]) ** 2).sum(-1)
        # an empty cluster's NaN center never wins (torch's argmin would return it)
        dist = torch.nan_to_num(dist, nan=float("inf"))
        mism += int((dist.argmin(1) != L[idx[r0:r0 + 1024]]).sum())
        del xs, dist
    sums = torch.zeros((k, d), dtype=torch.float64, device="cuda")
    sq = torch.zeros((), dtype=torch.float64, device="cuda")
    for r0 in range(0, n, 1 << 20):
        sums.index_add_(0, L[r0:r0 + (1 << 20)], X[r0:r0 + (1 << 20)].double())
    cnt = torch.bincount(L, minlength=k).double()
    means = sums / cnt[:, None]
    used = cnt > 0
    cerr = ((C1.double() - means).abs() / means.abs().clamp_min(1e-30))[used].max()
    C164 = C1.double()
    for r0 in range(0, n, 1 << 20):
        diff = X[r0:r0 + (1 << 20)].double() - C164[L[r0:r0 + (1 << 20)]]
        sq += (diff * diff).sum()
    sse64 = float(sq)
    acc = {"sample_rows": int(idx.numel()), "label_mismatches": mism,
           "label_mismatch_rate": mism / idx.numel(),
           "center_max_rel_err": float(cerr), "sse_rel_err": abs(sse - sse64) / abs(sse64),
           "reference": "torch float64 on the GPU (direct squared distances, FP64 means and SSE)"}
    # plain FP32 tier from the same centers
    h32 = km.Handle(n, d, k, assign_tier=km.ASSIGN_FP32, max_iters=8)
    h32.set_data(X, True)
    h32.set_centers(C.cpu().numpy(), False)
    h32.run(1)
    h32.synchronize()
    same = bool(torch.equal(torch.from_numpy(h32.labels()).cuda().long(), L))
    stream = torch.cuda.ExternalStream(h32.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h32.set_profiling(True)
    e0.record(stream)
    h32.run(5)
    e1.record(stream)
    h32.synchronize()
    ms = e0.elapsed_time(e1) / 5
    phase, pit = h32.phase_ms()
    h32.close()
    a_ms = phase[1] / max(pit, 1)
    plain = {"iter_per_s": 1000.0 / ms, "ms_per_iteration": ms, "assign_ms": a_ms,
             "assign_tflops": 2.0 * n * k * d / (a_ms / 1000.0) / 1e12,
             "labels_equal": same}
    return {"accuracy": acc, "plain_fp32": plain}


def time_kmeanspp(km, torch, h, n, k, reps=1):
    """k-means++ initialisation on the handle's resident data (outside the Lloyd timed region):
    one untimed call, then `reps` calls bracketed by CUDA events on the handle's stream. Each
    draw reads X once (N*D*4 bytes) and D^2 three times and writes it once (4 * N*4 bytes)."""
    stream = torch.cuda.ExternalStream(h.stream)
    h.init_kmeanspp(1000)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = km.launch_count()
    e0.record(stream)
    for r in range(reps):
        h.init_kmeanspp(r)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    launches = (km.launch_count() - l0) // reps
    draw_bytes = n * D * 4 + 4 * n * 4
    gbs = draw_bytes * (k - 1) / (ms / 1000.0) / 1e9
    _, hbm, src = peaks()
    return {"ms": ms, "draws": k, "us_per_draw": ms * 1000.0 / k, "launches": launches,
            "bytes_per_draw": draw_bytes, "achieved_GBs": gbs, "peak_GBs": hbm,
            "frac": gbs / hbm, "peak_source": f"{src} HBM copy (MEASURED_PEAKS.json)"}


def batched_problems(count, seed=2024):
    """The many-problems workload: N_i log-uniform in [256, 2e5], D_i uniform in {16,32,64,128},
    K_i = clamp(round(sqrt(N_i/2)), 4, 512), K_i isotropic unit-variance Gaussians with means
    U[-10,10]^D, equal weights (seeded, synthetic)."""
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(256), np.log(2e5))))
        d = int(rng.choice([16, 32, 64, 128]))
        k = int(min(512, max(4, round(np.sqrt(n / 2)))))
        means = rng.uniform(-10, 10, (k, d)).astype(np.float32)
        X = means[rng.integers(0, k, n)] + rng.standard_normal((n, d), dtype=np.float32)
        probs.append((X, k))
    return probs


def batched_workload(args):
    """15 Lloyd iterations of every problem in one kmgb_lloyd_batched_f32 call (host data,
    reference initialisation per problem, uploads and result copies inside the call)."""
    import kmeans_gb300 as km
    km.build()
    iters = 15
    t0 = time.perf_counter()
    probs = batched_problems(args.problems)
    gen_s = time.perf_counter() - t0
    rows = sum(len(p[0]) for p in probs)
    flop = sum(2.0 * len(X) * k * X.shape[1] for X, k in probs)
    tier_id = {"fp32": km.ASSIGN_FP32, "bf16": km.ASSIGN_BF16, "bf16x3": km.ASSIGN_BF16X3,
               "auto": km.ASSIGN_AUTO}[args.tier]
    km.lloyd_batched(probs[:64], max_iters=2, assign_tier=tier_id)  # warm-up: module loading
    t0 = time.perf_counter()
    km.lloyd_batched(probs, max_iters=1, assign_tier=tier_id)
    one = time.perf_counter() - t0
    l0 = km.launch_count()
    t0 = time.perf_counter()
    _, st = km.lloyd_batched(probs, max_iters=iters, assign_tier=tier_id)
    full = time.perf_counter() - t0
    launches = km.launch_count() - l0
    per_iter = st.ms_total / 1000.0 / iters  # CUDA events around the iteration loops
    sample = probs[: min(200, len(probs))]
    km.lloyd(sample[0][0], sample[0][1], max_iters=1)
    t0 = time.perf_counter()
    for X, k in sample:
        km.lloyd(X, k, max_iters=iters, assign_tier=tier_id)
    loop = time.perf_counter() - t0
    t0 = time.perf_counter()
    km.lloyd_batched(sample, max_iters=iters, assign_tier=tier_id)
    bsample = time.perf_counter() - t0
    line = {"metric": f"batched Lloyd, {len(probs)} problems x {iters} iterations (s per call)",
            "value": full, "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "data": "synthetic", "dtype": "f32" if args.tier == "fp32" else "bf16",
            "config": {"workload": f"batched_{len(probs)}_problems", "rows": rows,
                       "gflop_per_iteration": flop / 1e9, "iterations": iters,
                       "tier": args.tier, "certified_labels": True},
            "ms_per_iteration": per_iter * 1000.0,
            "phase_ms_per_iteration": ({nm: st.reserved[1 + i] / 1000.0 / iters for i, nm in
                                        enumerate(["prep", "assign", "rerank", "update"])}
                                       if st.reserved[5] == 0 else
                                       "not recorded: iterations replayed as CUDA graphs"),
            "setup_s": full - st.ms_total / 1000.0,
            "assign_tflops_per_iteration": flop / per_iter / 1e12,
            "setup_and_one_iteration_s": one, "generation_s": gen_s,
            "reranked_points_total": st.reranked, "gpu_launches": launches,
            "iteration_graph_launches_per_iteration": st.reserved[5] / iters,
            "groups": st.reserved[6],
            "label_audit": {"rows": int(st.reserved[7]) >> 24,
                            "violations": int(st.reserved[7]) & 0xFFFFFF},
            "single_call_loop": {"problems": len(sample), "loop_s": loop, "batched_s": bsample,
                                 "speedup": loop / bsample}}
    print(json.dumps(line), flush=True)


def large_k_data(n, d, k, seed=77):
    """16M x 256, K=65,536 clusters with Zipf(1.1) sizes, unit-variance Gaussians around means
    drawn from N(0, 25 I), values rounded to BF16 (BF16 points), on the device; initial centers a
    seeded sample of points."""
    import torch
    from kmeans_gb300.synthetic import sample_init
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    w = 1.0 / torch.arange(1, k + 1, device="cuda", dtype=torch.float64) ** 1.1
    lab = torch.multinomial((w / w.sum()).float(), n, replacement=True, generator=g)
    means = torch.randn((k, d), device="cuda", generator=g) * 5.0
    X = torch.empty((n, d), device="cuda", dtype=torch.float32)
    for r0 in range(0, n, 1 << 21):
        r1 = min(n, r0 + (1 << 21))
        X[r0:r1] = (means[lab[r0:r1]] + torch.randn((r1 - r0, d), device="cuda", generator=g)
                    ).to(torch.bfloat16).float()
    del lab, means
    init = X[torch.from_numpy(sample_init(n, k, seed=5)).cuda()].cpu().numpy()
    return X, init


def timed_run(km, torch, X, init, tier, iters, warm=True, **opts):
    """`iters` iterations of a fresh handle from `init` (one untimed warm-up iteration first),
    CUDA events on the handle's stream around the run. Returns (ms per iteration, phases,
    labels, centers, SSE history, stats, router stats)."""
    n, d = X.shape
    k = init.shape[0]
    h = km.Handle(n, d, k, assign_tier=tier, max_iters=iters + 1, **opts)
    h.set_data(X, True)
    h.set_centers(init, False)
    if warm and not opts.get("router"):
        h.run(1)  # warm-up (module loading, graph capture)
        h.synchronize()
        h.set_centers(init, False)
    stream = torch.cuda.ExternalStream(h.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h.set_profiling(True)
    e0.record(stream)
    h.run(iters)
    e1.record(stream)
    h.synchronize()
    ms = e0.elapsed_time(e1) / iters
    phase, pit = h.phase_ms()
    out = (ms, {nm: p / max(pit, 1) for nm, p in zip(["prep", "assign", "rerank", "update"], phase)},
           h.labels(), h.centers(), h.sse(iters), h.stats(), h.router_stats())
    h.close()
    return out


def large_k_workload(args, n=16_000_000, d=256, k=65_536):
    """Large-K workload (16M x 256, K=65,536, Zipf cluster sizes, BF16 points): the learned
    router (split BF16 tier, MLP 256->512->256 groups, retrained every 5 iterations) for the
    configuration's 25 iterations, against (a) the split BF16 tier without the router for the
    same 25 iterations from the same centers -- labels, centers and SSE must be identical, both
    being the FP64 arg-min -- and (b) one iteration of the plain FP32 tier (the denominator of the
    >= 5x target; its labels equal the split tier's first iteration)."""
    import torch
    import kmeans_gb300 as km
    km.build()
    iters = args.iters
    X, init = large_k_data(n, d, k)
    flop = 2.0 * n * k * d
    out = {"metric": f"Lloyd iteration, N={n}, D={d}, K={k} (ms)", "unit": "ms",
           "higher_is_better": False, "data": "synthetic (Zipf 1.1 cluster sizes, BF16 points)",
           "config": {"workload": "lloyd_16Mx256_K65536", "n": n, "d": d, "k": k,
                      "iterations": iters}}
    tiers = args.tiers.split(",")
    res = {}
    if "router" in tiers:
        ms, ph, lab, cen, sse, st, rs = timed_run(km, torch, X, init, km.ASSIGN_BF16X3, iters,
                                                  router=1, router_groups=256, router_retrain=5)
        res["router"] = (lab, cen, sse)
        routed_pts = n * rs.routed_iterations
        out["router"] = {"ms_per_iteration": ms, "phase_ms_per_iter": ph, "iterations": iters,
                         "iter_per_s": 1000.0 / ms,
                         "certified_share": rs.certified / max(1, routed_pts),
                         "fallback_share": rs.fallback / max(1, routed_pts),
                         "in_group_near_tie_share": rs.flagged / max(1, rs.routed),
                         "retrain_every": 5, "groups": 256, "hidden": 512,
                         "train_ms_total": rs.train_ms, "group_ms": rs.group_ms,
                         "trainings": rs.trainings, "last_train_accuracy": rs.last_accuracy,
                         "components": rs.components, "groups_nonempty": rs.groups_nonempty,
                         "max_group_centers": rs.max_group,
                         "max_component_centers": rs.max_component,
                         "group_scan_share_of_full": rs.scan_chunks / max(1, rs.routed)
                         / ((k + 255) // 256),
                         "routed_iterations": rs.routed_iterations,
                         "stage_ms_per_routed_iter": {
                             k_: v / max(1, rs.routed_iterations)
                             for k_, v in zip(km.kmgb_router_stats.STAGES, list(rs.stage_ms))},
                         "reranked_points": st.reranked}
    if "bf16x3" in tiers:
        ms, ph, lab, cen, sse, st, _ = timed_run(km, torch, X, init, km.ASSIGN_BF16X3, iters)
        res["bf16x3"] = (lab, cen, sse)
        out["bf16x3"] = {"ms_per_iteration": ms, "phase_ms_per_iter": ph, "iterations": iters,
                         "assign_tflops": flop / (ph["assign"] / 1000.0) / 1e12,
                         "reranked_points": st.reranked, "full_rescan_points": st.reranked_fp64}
    if "fp32" in tiers:
        ms, ph, lab, _, _, _, _ = timed_run(km, torch, X, init, km.ASSIGN_FP32, 1, warm=False)
        out["fp32"] = {"ms_per_iteration": ms, "phase_ms_per_iter": ph, "iterations": 1,
                       "assign_tflops": flop / (ph["assign"] / 1000.0) / 1e12}
        h = km.Handle(n, d, k, assign_tier=km.ASSIGN_BF16X3, max_iters=1)
        h.set_data(X, True)
        h.set_centers(init, False)
        h.run(1)
        h.synchronize()
        out["fp32"]["labels_equal_split_first_iteration"] = bool(np.array_equal(h.labels(), lab))
        h.close()
    if "router" in res and "bf16x3" in res:
        a, b = res["router"], res["bf16x3"]
        out["router_vs_split"] = {
            "labels_identical": bool(np.array_equal(a[0], b[0])),
            "centers_identical": bool(np.array_equal(a[1], b[1], equal_nan=True)),
            "sse_identical": bool(np.array_equal(a[2], b[2])),
            "speedup": out["bf16x3"]["ms_per_iteration"] / out["router"]["ms_per_iteration"]}
    main_tier = "router" if "router" in out else "bf16x3"
    if main_tier in out:
        out["value"] = out[main_tier]["ms_per_iteration"]
        out["tier"] = main_tier
    if "fp32" in out and main_tier in out:
        out["speedup_vs_plain_fp32"] = (out["fp32"]["ms_per_iteration"]
                                        / out[main_tier]["ms_per_iteration"])
    print(json.dumps(out), flush=True)


def large_k_summary(km, torch, n=16_000_000, d=256, k=65_536, iters=25):
    """The large-K configuration (16M x 256, K=65,536, Zipf sizes, BF16 points, 25 iterations)
    outside the headline's timed region: the learned router's run, the same iterations of the
    split BF16 tier without it (labels, centers and SSE must be identical), and one plain FP32
    iteration (the denominator of the >= 5x target)."""
    X, init = large_k_data(n, d, k)
    rt = timed_run(km, torch, X, init, km.ASSIGN_BF16X3, iters, router=1, router_groups=256,
                   router_retrain=5)
    st = timed_run(km, torch, X, init, km.ASSIGN_BF16X3, iters)
    ft = timed_run(km, torch, X, init, km.ASSIGN_FP32, 1, warm=False)
    rs = rt[6]
    del X
    torch.cuda.empty_cache()
    routed_pts = n * max(1, rs.routed_iterations)
    return {"workload": "lloyd_16Mx256_K65536", "iterations": iters,
            "router_ms_per_iteration": rt[0], "split_bf16_ms_per_iteration": st[0],
            "plain_fp32_ms_per_iteration": ft[0],
            "speedup_vs_plain_fp32": ft[0] / rt[0], "speedup_vs_split_bf16": st[0] / rt[0],
            "labels_identical": bool(np.array_equal(rt[2], st[2])),
            "centers_identical": bool(np.array_equal(rt[3], st[3], equal_nan=True)),
            "sse_identical": bool(np.array_equal(rt[4], st[4])),
            "certified_share": rs.certified / routed_pts,
            "fallback_share": rs.fallback / routed_pts, "trainings": rs.trainings,
            "train_ms_total": rs.train_ms, "last_train_accuracy": rs.last_accuracy,
            "router_stage_ms_per_routed_iter": {
                k_: v / max(1, rs.routed_iterations)
                for k_, v in zip(km.kmgb_router_stats.STAGES, list(rs.stage_ms))},
            "router_phase_ms_per_iter": rt[1], "split_phase_ms_per_iter": st[1],
            "timing": "CUDA events on each handle's stream around the whole run (trainings "
                      "included); plain FP32: one iteration"}


def fp64_workload(args, n=4_000_000, d=128, k=1024, iters=5):
    """The FP64 entry, computeKmeansD, on the 4M x 128, K=1024 mixture in FP64 (host data,
    reference initialisation, criterion < 0): the tensor path (split BF16 tier on FP32 roundings,
    exact FP64 scan of the uncertified points) against the exact FP64 scan of every point
    (KMGB_ASSIGN=fp32). Per-iteration times come from calls of `iters` and of one iteration (the
    difference removes the call's fixed cost: upload, initialisation, result). Both give the
    FP64 arg-min labels, so one iteration of each must return the same centers bit for bit."""
    import torch
    import kmeans_gb300 as km
    from kmeans_gb300.synthetic import mixture_torch
    km.build()
    X, _, _ = mixture_torch(n, d, k, seed=1234, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0))
    Xh = X.double().cpu().numpy()
    del X
    torch.cuda.empty_cache()

    def call(its, scan):
        if scan:
            os.environ["KMGB_ASSIGN"] = "fp32"
        try:
            result = np.zeros(d * k, np.float64)
            t0 = time.perf_counter()
            rc = km.computeKmeansD(Xh, n, d, k, -1.0, its, 1, 0, 0, 0, result, 1.0)
            return rc, time.perf_counter() - t0, result
        finally:
            os.environ.pop("KMGB_ASSIGN", None)

    call(1, False)  # warm
    rc_n, t_n, _ = call(iters, False)
    rc_1, t_1, r_1 = call(1, False)
    rc_s, t_s, r_s = call(1, True)
    per_iter = (t_n - t_1) / (iters - 1)
    fixed = t_1 - per_iter
    out = {"metric": f"computeKmeansD, N={n}, D={d}, K={k} (s per iteration)", "unit": "s",
           "higher_is_better": False, "data": "synthetic (FP64)",
           "config": {"workload": "fp64_4Mx128_K1024", "n": n, "d": d, "k": k},
           "value": per_iter,
           "tensor": {"status": rc_n, "iterations": iters, "call_s": t_n,
                      "one_iteration_call_s": t_1, "s_per_iteration": per_iter,
                      "fixed_s": fixed},
           "fp64_scan": {"status": rc_s, "one_iteration_call_s": t_s,
                         "s_per_iteration": t_s - fixed},
           "same_centers_after_one_iteration": bool(np.array_equal(r_1, r_s, equal_nan=True)),
           "speedup": (t_s - fixed) / per_iter if per_iter > 0 else None}
    print(json.dumps(out), flush=True)


def streamed_workload(args, n=200_000_000, d=96, k=4096, iters=10, tile=4_000_000):
    """Host-resident data set: 200M x 96 (76.8 GB of host memory), K=4096 isotropic Gaussians
    (sigma 1.5, means U[-15,15]^96, equal weights), initial centers a seeded sample of points;
    10 Lloyd iterations of the split BF16 tier through kmgb_lloyd_f32, (a) streamed through the
    GPU in 4M-row tiles every iteration (the reference's out-of-memory path), (b) uploaded once
    and resident in HBM. Both give the FP64 arg-min labels, so they must be identical."""
    import torch
    import kmeans_gb300 as km
    from kmeans_gb300.synthetic import sample_init
    km.build()
    if args.n != N:
        n = args.n
    t0 = time.perf_counter()
    Xh = np.empty((n, d), np.float32)
    g = torch.Generator(device="cuda")
    g.manual_seed(31)
    means = torch.empty((k, d), device="cuda").uniform_(-15.0, 15.0, generator=g)
    for r0 in range(0, n, 1 << 22):
        r1 = min(n, r0 + (1 << 22))
        lab = torch.randint(0, k, (r1 - r0,), device="cuda", generator=g)
        Xh[r0:r1] = (means[lab] + 1.5 * torch.randn((r1 - r0, d), device="cuda", generator=g)
                     ).cpu().numpy()
    del means
    torch.cuda.empty_cache()
    gen_s = time.perf_counter() - t0
    init = Xh[sample_init(n, k, seed=17)]
    # one host-to-device pass of X in tiles (pageable source), the floor of a streamed iteration
    buf = torch.empty((tile, d), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r0 in range(0, n, tile):
        r1 = min(n, r0 + tile)
        buf[: r1 - r0].copy_(torch.from_numpy(Xh[r0:r1]))
    torch.cuda.synchronize()
    h2d_s = time.perf_counter() - t0
    del buf
    torch.cuda.empty_cache()
    out = {"metric": f"Lloyd iteration, host data N={n}, D={d}, K={k} (s)", "unit": "s",
           "higher_is_better": False, "data": "synthetic", "dtype": "bf16",
           "config": {"workload": f"lloyd_{n}x{d}_K{k}_host", "n": n, "d": d, "k": k,
                      "iterations": iters, "tier": "bf16x3", "tile_rows": tile},
           "generation_s": gen_s, "h2d_pass_s": h2d_s, "h2d_GBs": Xh.nbytes / h2d_s / 1e9}
    labels = {}
    for mode, rows in (("streamed", tile), ("resident", 0)):
        km.lloyd(Xh[:tile], k, init=init, max_iters=1, assign_tier=km.ASSIGN_BF16X3)  # warm-up
        t0 = time.perf_counter()
        res = km.lloyd(Xh, k, init=init, max_iters=iters, assign_tier=km.ASSIGN_BF16X3,
                       stream_tile_rows=rows)
        wall = time.perf_counter() - t0
        out[mode] = {"call_s": wall, "s_per_iteration": wall / iters,
                     "gpu_iterations_ms": res.ms_total, "reranked_points": res.reranked,
                     "sse_last": float(res.sse[-1])}
        labels[mode] = res.labels
        del res
    out["value"] = out["streamed"]["s_per_iteration"]
    out["labels_identical"] = bool(np.array_equal(labels["streamed"], labels["resident"]))
    print(json.dumps(out), flush=True)


def sharded_arm(args, rank: int, world: int, local: int, dist):
    """N > 1: the workload's rows on every rank (the job's data set is N x 4M rows, weak scaling),
    one sharded Lloyd run (kmeans_gb300/shard.py): each iteration every rank assigns its rows,
    the ranks all-gather their FP64 per-cluster sums over NCCL and add them in rank order, and
    every rank updates the same centers. Timed with CUDA events between barriers, max over ranks."""
    import torch
    import kmeans_gb300 as km
    from kmeans_gb300.shard import LibraryShard, lloyd_sharded_device
    from kmeans_gb300.synthetic import mixture_torch, sample_init
    tier = {"fp32": km.ASSIGN_FP32, "bf16": km.ASSIGN_BF16, "bf16x3": km.ASSIGN_BF16X3}[args.tier]
    X, _, _ = mixture_torch(N, D, K, seed=1234, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0))
    init = X[torch.from_numpy(sample_init(N, K, seed=99)).cuda()].cpu().numpy()
    sh = LibraryShard(X, K, init, tier)
    lloyd_sharded_device(sh, K, D, args.warmup, dist=dist)
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    l0 = km.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    res = lloyd_sharded_device(sh, K, D, args.steps, dist=dist)
    e1.record()
    torch.cuda.synchronize()
    dist.barrier()
    cl = clocks.stop()
    launches = km.launch_count() - l0
    ms, value = replica_rate(e0.elapsed_time(e1), args.steps, world, dist)
    sh.close()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if args.tier == "fp32" else "bf16", "data": "synthetic",
                "config": {"workload": "lloyd_4Mx128_K1024", "n": N, "d": D, "k": K,
                           "tier": args.tier, "certified_labels": True,
                           "parallelism": f"sharded rows over {world} GPUs (N x 4M rows), one "
                                          f"all-gather of FP64 per-cluster sums per iteration",
                           "l2": "inputs larger than L2 (X: 2.05 GB FP32 per rank)"},
                "exchanged_bytes_per_iteration": res.exchanged_bytes_per_iteration,
                "sse_last": float(res.sse[-1]), "gpu_launches": launches, "clocks": cl,
                "e2e": None, "roofline": None, "cpu_baseline": None}
        print(json.dumps(line), flush=True)


def c3_resident_workload(args, n=200_000_000, d=96, k=4096, iters=10):
    """The 200M x 96, K=4096 configuration (sigma 1.5, means U[-15,15]^96, 76.8 GB of FP32) with
    the data set uploaded once and resident in HBM, 10 Lloyd iterations from the same seeded
    initial centers in the split BF16 tier and in the FP8 E4M3 tier: GPU time per iteration
    (CUDA events around the iterations, upload excluded), points the certificate left to the exact
    settlement, and whether both give the same labels and centers (both are the FP64 arg-min)."""
    import torch
    import kmeans_gb300 as km
    from kmeans_gb300.synthetic import sample_init
    km.build()
    if args.n != N:
        n = args.n
    t0 = time.perf_counter()
    Xh = np.empty((n, d), np.float32)
    g = torch.Generator(device="cuda")
    g.manual_seed(31)
    means = torch.empty((k, d), device="cuda").uniform_(-15.0, 15.0, generator=g)
    for r0 in range(0, n, 1 << 22):
        r1 = min(n, r0 + (1 << 22))
        lab = torch.randint(0, k, (r1 - r0,), device="cuda", generator=g)
        Xh[r0:r1] = (means[lab] + 1.5 * torch.randn((r1 - r0, d), device="cuda", generator=g)
                     ).cpu().numpy()
    del means
    torch.cuda.empty_cache()
    gen_s = time.perf_counter() - t0
    init = Xh[sample_init(n, k, seed=17)]
    flop = 2.0 * n * k * d
    out = {"metric": f"Lloyd iteration, resident N={n}, D={d}, K={k} (s)", "unit": "s",
           "higher_is_better": False, "data": "synthetic", "generation_s": gen_s,
           "config": {"workload": f"lloyd_{n}x{d}_K{k}_resident", "n": n, "d": d, "k": k,
                      "iterations": iters}}
    res = {}
    for name, tier in (("bf16x3", km.ASSIGN_BF16X3), ("fp8", km.ASSIGN_FP8)):
        km.lloyd(Xh[:1 << 20], k, init=init, max_iters=1, assign_tier=tier)  # warm-up
        t0 = time.perf_counter()
        r = km.lloyd(Xh, k, init=init, max_iters=iters, assign_tier=tier)
        wall = time.perf_counter() - t0
        out[name] = {"call_s": wall, "gpu_s_per_iteration": r.ms_total / 1000.0 / iters,
                     "assign_pflop_per_iteration": flop / 1e15,
                     "reranked_share": r.reranked / (n * iters),
                     "full_rescan_points": r.reranked_fp64, "sse_last": float(r.sse[-1])}
        res[name] = (r.labels, r.centers)
        del r
    out["value"] = out["fp8"]["gpu_s_per_iteration"]
    out["fp8_vs_bf16x3"] = out["bf16x3"]["gpu_s_per_iteration"] / out["fp8"]["gpu_s_per_iteration"]
    out["labels_identical"] = bool(np.array_equal(res["fp8"][0], res["bf16x3"][0]))
    out["centers_identical"] = bool(np.array_equal(res["fp8"][1], res["bf16x3"][1], equal_nan=True))
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 100 Lloyd iterations (~0.3 s): several clock samples fall inside the timed region
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--tier", default="bf16x3",
                    help="assignment tier: bf16x3 (split BF16 tensor cores, default), bf16, fp8, "
                         "fp32")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-large-k", action="store_true",
                    help="skip the large-K (16M x 256, K=65,536) router summary")
    ap.add_argument("--n", type=int, default=N, help="rows (default: the 4M workload); smaller "
                    "values are for profiling captures only")
    ap.add_argument("--k", type=int, default=NUM_CENTERS, help="centers (default 1024); other values are "
                    "for profiling captures only")
    ap.add_argument("--no-init", action="store_true", help="skip the k-means++ timing")
    ap.add_argument("--no-checks", action="store_true",
                    help="skip the FP64 accuracy checks and the plain-FP32 comparison")
    ap.add_argument("--only-init", action="store_true",
                    help="time only the k-means++ initialisation (profiling captures)")
    ap.add_argument("--workload", default="lloyd",
                    choices=["lloyd", "batched", "large_k", "streamed", "fp64", "c3_resident"],
                    help="batched: the many-problems workload through kmgb_lloyd_batched_f32; "
                         "large_k: 16M x 256, K=65536 split BF16 vs FP32; streamed: 200M x 96, "
                         "K=4096 host data, streamed tiles vs resident (own JSON lines; not the "
                         "headline)")
    ap.add_argument("--problems", type=int, default=10_000,
                    help="problems of the batched workload")
    ap.add_argument("--tiers", default="router,bf16x3,fp32",
                    help="tiers of the large_k workload (router = split BF16 + learned router)")
    ap.add_argument("--iters", type=int, default=25, help="iterations of the large_k workload")
    ap.add_argument("--bf16-data", action="store_true",
                    help="the workload's points stored as BF16 values (the configuration's BF16 "
                         "storage variant)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return reference_arm(args, rank)
    if args.workload == "batched":
        return batched_workload(args)
    if args.workload == "large_k":
        return large_k_workload(args)
    if args.workload == "streamed":
        return streamed_workload(args)
    if args.workload == "fp64":
        fp64_workload(args)
        return
    if args.workload == "c3_resident":
        return c3_resident_workload(args)

    import torch
    import kmeans_gb300 as km
    from kmeans_gb300.synthetic import mixture_torch, sample_init

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        km.build()
        sharded_arm(args, rank, world, local, dist)
        dist.destroy_process_group()
        return
    km.build()
    lib = km.lib()
    tier = args.tier
    tier_id = {"fp32": km.ASSIGN_FP32, "bf16": km.ASSIGN_BF16, "bf16x3": km.ASSIGN_BF16X3,
               "fp8": km.ASSIGN_FP8}[tier]

    n, K = args.n, args.k
    X, _, _ = mixture_torch(n, D, K, seed=1234, mean_lo=-20.0, mean_hi=20.0, std=(0.3, 3.0))
    if args.bf16_data:
        X = X.to(torch.bfloat16).float()
    if args.only_init:
        h = km.Handle(n, D, K, assign_tier=km.ASSIGN_FP32)
        h.set_data(X, True)
        line = {"metric": f"k-means++ initialisation (N={n}, D={D}, K={K})",
                "init_kmeanspp": time_kmeanspp(km, torch, h, n, K, reps=max(1, args.steps))}
        print(json.dumps(line), flush=True)
        h.close()
        return
    idx = torch.from_numpy(sample_init(n, K, seed=99)).cuda()
    init = X[idx].cpu().numpy()
    h = km.Handle(n, D, K, assign_tier=tier_id, max_iters=args.steps + args.warmup)
    h.set_data(X, True)
    h.set_centers(init, False)
    h.run(args.warmup)
    h.synchronize()

    stream = torch.cuda.ExternalStream(h.stream)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    h.set_profiling(True)
    launches0 = km.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    ev0.record(stream)
    h.run(args.steps)
    ev1.record(stream)
    h.synchronize()
    torch.cuda.synchronize()
    cl = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = km.launch_count() - launches0
    phase, piters = h.phase_ms()
    st = h.stats()
    ms, value = replica_rate(ms, args.steps, world, dist)

    flop = 2.0 * n * K * D
    assign_ms = phase[1] / max(piters, 1)
    achieved = flop / (assign_ms / 1000.0) / 1e12
    bf16_peak, hbm_peak, src = peaks()
    traffic = TRAFFIC_BYTES_PER_ROW.get(tier)
    roofline = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved / bf16_peak,
                "traffic": traffic * n if traffic else None, "traffic_unit": "bytes",
                "kernel": "assign_fp32_kernel" if tier == "fp32" else "assign_bf16_kernel",
                "peak_source": f"{src} bf16 dense (MEASURED_PEAKS.json)",
                "flop_per_launch": flop, "ms_per_launch": assign_ms}
    if tier in TENSOR_PRODUCTS:
        tf = TENSOR_PRODUCTS[tier] * flop
        roofline["tensor_flop_per_launch"] = tf
        roofline["tensor_tflops"] = tf / (assign_ms / 1000.0) / 1e12
        roofline["tensor_frac"] = roofline["tensor_tflops"] / bf16_peak

    # the update phase (counting sort, piece sums, finalize, SSE; event-timed together) against
    # HBM: its algorithmic bytes per iteration are X once, the labels and the FP64 per-cluster
    # sums
    upd_ms = phase[3] / max(piters, 1)
    upd_bytes = n * D * 4 + n * 4 + K * D * 8
    upd_gbs = upd_bytes / (upd_ms / 1000.0) / 1e9 if upd_ms > 0 else None
    update_roofline = {"bound": "hbm", "achieved": upd_gbs, "peak": hbm_peak, "unit": "GB/s",
                       "frac": upd_gbs / hbm_peak if upd_gbs else None,
                       "bytes_per_iteration": upd_bytes, "ms_per_iteration": upd_ms,
                       "kernels": "hist, scans, scatter_multi, piece_sums_ring, finalize, sse",
                       "peak_source": f"{src} HBM copy (MEASURED_PEAKS.json)"}

    checks = None
    if not args.no_checks and rank == 0:
        checks = accuracy_and_plain_fp32(km, torch, h, X, n, K)

    init_pp = None
    if not args.no_init and rank == 0:
        init_pp = time_kmeanspp(km, torch, h, n, K, reps=1)

    e2e = None
    if not args.no_e2e and rank == 0:
        # the step's input in pinned host memory; the same rows in pageable memory as a second
        # measurement
        Xpin = torch.empty(X.shape, dtype=torch.float32, pin_memory=True)
        Xpin.copy_(X)
        Xh = Xpin.numpy()
        Xpage = np.array(Xh, copy=True)
        del X
        torch.cuda.empty_cache()

        def timed_call(src):
            t0 = time.perf_counter()
            res = km.lloyd(src, K, init=init, max_iters=E2E_ITERS, assign_tier=tier_id)
            return res, time.perf_counter() - t0

        # one untimed call first (module loading, the library's memory pool), like the device
        # path's warm-up iterations; the timed call then includes all of its own host<->device
        # copies, its allocation and its release
        km.lloyd(Xh, K, init=init, max_iters=max(1, args.warmup), assign_tier=tier_id)
        torch.cuda.synchronize()
        # three timed calls each, the median reported (one call on a shared host can take
        # tens of ms longer: a single 153 ms call was seen among 86-87 ms ones)
        runs = [timed_call(Xh) for _ in range(3)]
        secs = sorted(t for _, t in runs)
        res, sec = runs[0][0], secs[1]
        sec_page = sorted(timed_call(Xpage)[1] for _ in range(3))[1]
        # the reference's own entry point: its shuffle and initialisation on the host, the
        # workload's iterations (criterion < 0 runs them all), D x K centers back
        result = np.zeros(D * K, np.float32)
        km.computeKmeansF(Xh, n, D, K, -1.0, 1, 1, 0, 0, 0, result, 1.0)  # warm
        t0 = time.perf_counter()
        rc_ref = km.computeKmeansF(Xh, n, D, K, -1.0, E2E_ITERS, 1, 0, 0, 0, result, 1.0)
        sec_ref = time.perf_counter() - t0
        e2e = {"value": E2E_ITERS / sec, "unit": "iter/s",
               "h2d_bytes_per_step": (Xh.nbytes + init.nbytes) // E2E_ITERS,
               "d2h_bytes_per_step": (res.centers.nbytes + res.labels.nbytes + res.sse.nbytes)
               // E2E_ITERS, "iterations_per_call": E2E_ITERS,
               "call": "kmgb_lloyd_f32 (host pinned X, init, centers/labels/SSE out); "
                       "after one untimed call; median of 3 calls",
               "calls_s": secs,
               "seconds": sec, "pageable_value": E2E_ITERS / sec_page,
               "compute_kmeans_f": {"value": E2E_ITERS / sec_ref, "seconds": sec_ref,
                                    "status": rc_ref,
                                    "call": "computeKmeansF (host pinned data, reference shuffle "
                                            "and initialisation, D x K result)"}}
        del Xpin, Xh
    cb = None
    if not args.no_cpu and rank == 0:
        # the same rows and initial centers, on the host: 3 timed full iterations
        Xc = Xpage if e2e is not None else X.cpu().numpy()
        cb = cpu_baseline(Xc, init, steps=3, warmup=1)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "nproc",
                                 "cpu_model")}
        del Xc
    if e2e is not None:
        del Xpage
    h.close()
    large_k = None
    if not args.no_large_k and rank == 0 and n == N:
        torch.cuda.empty_cache()
        large_k = large_k_summary(km, torch)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if tier == "fp32" else "bf16", "data": "synthetic",
                "config": {"workload": ("lloyd_4Mx128_K1024" if (n, K) == (N, NUM_CENTERS)
                                        else f"lloyd_{n}x{D}_K{K}")
                           + ("_bf16" if args.bf16_data else ""),
                           "n": n, "d": D, "k": K,
                           "tier": tier, "certified_labels": True,
                           "storage": "bf16 values" if args.bf16_data else "fp32",
                           "l2": (f"inputs larger than L2 (X: {n * D * 4 / 1e9:.2f} GB FP32 per "
                                  f"pass)" if n * D * 4 > L2_BYTES else
                                  f"X ({n * D * 4 / 1e6:.0f} MB) fits in L2: profiling size, "
                                  f"not a bench figure"),
                           "parallelism": "single"},
                "assign_tflops": achieved,
                "phase_ms_per_iter": {n: p / max(piters, 1) for n, p in
                                      zip(["prep", "assign", "rerank", "update"], phase)},
                "reranked_points_total": st.reranked, "reranked_fp64_total": st.reranked_fp64,
                "label_audit": {"rows": int(st.reserved[6]), "violations": int(st.reserved[7]),
                                "what": "rows sampled every iteration (timed ones included) and "
                                        "checked against the FP64 arg-min over all centers"},
                "roofline": roofline, "update_roofline": update_roofline,
                "cpu_baseline": cb, "e2e": e2e,
                "init_kmeanspp": init_pp,
                "accuracy": checks["accuracy"] if checks else None,
                "plain_fp32": checks["plain_fp32"] if checks else None,
                "speedup_vs_plain_fp32": (value / checks["plain_fp32"]["iter_per_s"]
                                          if checks else None),
                "gpu_launches": launches, "clocks": cl, "large_k": large_k}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
