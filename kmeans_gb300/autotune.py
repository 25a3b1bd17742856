"""Autotuner of the batched Lloyd's kernel families: writes kmeans_gb300/csrc/tuned_batched.h.

kmgb_lloyd_batched_f32 runs every group of problems of one dimension with one of two grouped
assignment families: the FP32 SIMT kernel (128-row x 128-center tiles, TMA ring, problems padded
to 128 rows) or the split BF16 tcgen05 pair kernel (256-row x 256-center pair tiles, problems
padded to 256 rows and 256 centers). Which one is faster depends on the problems' dimension and
center count (padding waste against tensor throughput). For every (d, k) bucket this script
builds a batch of synthetic problems of that shape (k centers, n = max(256, 2 k^2) rows as in the
many-problems configuration, K_i = sqrt(N_i / 2)), runs a few Lloyd iterations with each family
on the GPU (one untimed call first), takes the GPU time per iteration from the call's CUDA events
and writes both families' cost per row and iteration into the table that KMGB_ASSIGN_AUTO reads:
the library predicts each dimension's cost under each family from its problems' rows and buckets
and runs the whole dimension with the cheaper one (one group per dimension: splitting a dimension
between the families costs a second group's set-up and saved nothing measurable on the
10,000-problem workload).

    python -m kmeans_gb300.autotune [--out PATH] [--iters 5] [--json PATH]
    python -m kmeans_gb300.autotune --from-json PATH [--out PATH]   (header from saved timings)

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
    record = {"gpu": torch.cuda.get_device_name(0), "iters": iters,
              "date": datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%d"),
              "buckets": {}}
    for d in DIMS:
        for k in KMAX:
            probs = bucket_problems(d, k)
            t32 = time_family(km, probs, km.ASSIGN_FP32, iters)
            t16 = time_family(km, probs, km.ASSIGN_BF16X3, iters)
            record["buckets"][f"d{d}_k{k}"] = {
                "problems": len(probs), "rows_each": int(probs[0][0].shape[0]),
                "fp32_ms_per_iter": t32, "bf16x3_ms_per_iter": t16}
            print(f"d={d:4d} k<={k:4d}: fp32 {t32:8.3f} ms, split bf16 {t16:8.3f} ms per "
                  f"iteration", flush=True)
            del probs
            torch.cuda.empty_cache()
    write_header(record, out)
    return record


def write_header(record: dict, out: str = DEFAULT_OUT):
    """tuned_batched.h from a record of bucket timings (as tune() returns it)."""
    b = record["buckets"]

    def ns_per_row(key, fam):
        v = b[key]
        return v[f"{fam}_ms_per_iter"] * 1e6 / (v["problems"] * v["rows_each"])

    lines = ["// Cost of a batched problem's row per Lloyd iteration (ns) by (d, k) bucket and assignment",
             "// family, for kmgb_lloyd_batched_f32 with KMGB_ASSIGN_AUTO. Written by",
             f"// kmeans_gb300/autotune.py on {record['gpu']}, {record['date']}: per bucket the GPU time of",
             f"// {record['iters']} Lloyd iterations of synthetic problems with k centers and max(256, 2 k^2)",
             "// rows (ms per iteration, FP32 / split BF16, problems x rows):"]
    for key, v in b.items():
        lines.append(f"//   {key:10s} {v['fp32_ms_per_iter']:9.3f} / {v['bf16x3_ms_per_iter']:9.3f}"
                     f"   {v['problems']} x {v['rows_each']}")
    lines += ["#pragma once", "", "namespace kmgb {",
              f"constexpr int kTunedDims[] = {{{', '.join(map(str, DIMS))}}};",
              f"constexpr int kTunedKMax[] = {{{', '.join(map(str, KMAX))}}};",
              "// [family: 0 FP32, 1 split BF16][dimension bucket][center bucket]",
              f"constexpr float kTunedNsPerRow[2][{len(DIMS)}][{len(KMAX)}] = {{"]
    for fam in ("fp32", "bf16x3"):
        lines.append("    {")
        for d in DIMS:
            vals = ", ".join(f"{ns_per_row(f'd{d}_k{k}', fam):.5g}f" for k in KMAX)
            lines.append(f"        {{{vals}}},")
        lines.append("    },")
    lines += ["};", "}  // namespace kmgb", ""]
    with open(out, "w") as fh:
        fh.write("\n".join(lines))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--iters", type=int, default=5)
    ap.add_argument("--json", default=None, help="also write the measurements as JSON")
    ap.add_argument("--from-json", default=None,
                    help="write the header from measurements saved with --json (no GPU)")
    a = ap.parse_args()
    if a.from_json:
        with open(a.from_json) as fh:
            write_header(json.load(fh), a.out)
    else:
        rec = tune(a.out, a.iters)
        if a.json:
            with open(a.json, "w") as fh:
                json.dump(rec, fh, indent=1)
