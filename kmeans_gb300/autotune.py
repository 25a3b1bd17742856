"""Autotuner of the batched Lloyd's kernel families: writes kmeans_gb300/csrc/tuned_batched.h.

kmgb_lloyd_batched_f32 runs every group of problems of one dimension with one of two grouped
assignment families: the FP32 SIMT kernel (128-row x 128-center tiles, TMA ring, problems padded
to 128 rows) or the split BF16 tcgen05 pair kernel (256-row x 256-center pair tiles, problems
padded to 256 rows and 256 centers). Which one is faster depends on the problems' dimension and
center count (padding waste against tensor throughput). For every (d, k) bucket this script
builds a batch of synthetic problems of that shape (k centers, n = max(256, 2 k^2) rows as in the
many-problems configuration, K_i = sqrt(N_i / 2)), runs a few Lloyd iterations with each family
on the GPU (one untimed call first), takes the GPU time per iteration from the call's CUDA events
and writes the faster family into the table that KMGB_ASSIGN_AUTO reads.

    python -m kmeans_gb300.autotune [--out PATH] [--iters 5]

then rebuild the library. The committed table was produced by this script on a GB300.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os

import numpy as np

DIMS = (16, 32, 64, 128)
KMAX = (16, 32, 64, 128, 256, 512)
HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "csrc", "tuned_batched.h")


def bucket_problems(d: int, k: int, max_rows: int = 8_000_000, seed: int = 0):
    """Problems with k centers and n = max(256, 2 k^2) rows each (device tensors), about
    max_rows rows in all (between 8 and 200 problems)."""
    import torch
    n = max(256, 2 * k * k)
    count = int(max(8, min(200, max_rows // n)))
    g = torch.Generator(device="cuda")
    g.manual_seed(seed + 1000 * d + k)
    probs = []
    for _ in range(count):
        means = torch.empty((k, d), device="cuda").uniform_(-10.0, 10.0, generator=g)
        lab = torch.randint(0, k, (n,), device="cuda", generator=g)
        X = (means[lab] + torch.randn((n, d), device="cuda", generator=g)).contiguous()
        init = X[torch.randperm(n, device="cuda", generator=g)[:k]].cpu().numpy()
        probs.append((X, k, init))
    return probs


def time_family(km, probs, tier: int, iters: int) -> float:
    km.lloyd_batched(probs, max_iters=1, assign_tier=tier)  # untimed: module loading
    _, st = km.lloyd_batched(probs, max_iters=iters, assign_tier=tier)
    return st.ms_total / iters


def tune(out: str = DEFAULT_OUT, iters: int = 5):
    import torch
    import kmeans_gb300 as km
    km.build()
    table, record = [], {}
    for d in DIMS:
        row = []
        for k in KMAX:
            probs = bucket_problems(d, k)
            t32 = time_family(km, probs, km.ASSIGN_FP32, iters)
            t16 = time_family(km, probs, km.ASSIGN_BF16X3, iters)
            tier = km.ASSIGN_FP32 if t32 <= t16 else km.ASSIGN_BF16X3
            row.append(tier)
            record[f"d{d}_k{k}"] = {"problems": len(probs), "rows_each": int(probs[0][0].shape[0]),
                                   "fp32_ms_per_iter": t32, "bf16x3_ms_per_iter": t16,
                                   "chosen": "fp32" if tier == km.ASSIGN_FP32 else "bf16x3"}
            print(f"d={d:4d} k<={k:4d}: fp32 {t32:8.3f} ms, split bf16 {t16:8.3f} ms per "
                  f"iteration -> {record[f'd{d}_k{k}']['chosen']}", flush=True)
            del probs
            torch.cuda.empty_cache()
        table.append(row)
    gpu = torch.cuda.get_device_name(0)
    when = datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%d")
    lines = ["// Tier of a batched problem by its (d, k) bucket, for kmgb_lloyd_batched_f32 with",
             f"// KMGB_ASSIGN_AUTO. Written by kmeans_gb300/autotune.py on {gpu}, {when}: per bucket",
             f"// the faster of the two grouped families over {iters} Lloyd iterations of synthetic",
             "// problems with k centers and max(256, 2 k^2) rows (ms per iteration, FP32 / split BF16):"]
    for key, v in record.items():
        lines.append(f"//   {key:10s} {v['fp32_ms_per_iter']:9.3f} / {v['bf16x3_ms_per_iter']:9.3f}"
                     f"  -> {v['chosen']}")
    lines += ["#pragma once", "", "namespace kmgb {",
              f"constexpr int kTunedDims[] = {{{', '.join(map(str, DIMS))}}};",
              f"constexpr int kTunedKMax[] = {{{', '.join(map(str, KMAX))}}};",
              "// KMGB_ASSIGN_FP32 = 0, KMGB_ASSIGN_BF16X3 = 2",
              f"constexpr int kTunedTier[{len(DIMS)}][{len(KMAX)}] = {{"]
    lines += ["    {" + ", ".join(map(str, r)) + "}," for r in table]
    lines += ["};", "}  // namespace kmgb", ""]
    with open(out, "w") as fh:
        fh.write("\n".join(lines))
    return record


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--iters", type=int, default=5)
    ap.add_argument("--json", default=None, help="also write the measurements as JSON")
    a = ap.parse_args()
    rec = tune(a.out, a.iters)
    if a.json:
        with open(a.json, "w") as fh:
            json.dump(rec, fh, indent=1)
