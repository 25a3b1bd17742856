// Tier of a batched problem by its (d, k) bucket, for kmgb_lloyd_batched_f32 with
// KMGB_ASSIGN_AUTO. Written by kmeans_gb300/autotune.py on NVIDIA GB300, 2026-12-04: per bucket
// the faster of the two grouped families over 5 Lloyd iterations of synthetic
// problems with k centers and max(256, 2 k^2) rows (ms per iteration, FP32 / split BF16):
//   d16_k16        0.153 /     0.203  -> fp32
//   d16_k32        0.328 /     0.317  -> bf16x3
//   d16_k64        1.006 /     0.722  -> bf16x3
//   d16_k128       3.567 /     2.273  -> bf16x3
//   d16_k256       5.935 /     2.717  -> bf16x3
//   d16_k512       9.136 /     4.199  -> bf16x3
//   d32_k16        0.157 /     0.199  -> fp32
//   d32_k32        0.333 /     0.340  -> fp32
//   d32_k64        1.022 /     0.748  -> bf16x3
//   d32_k128       3.628 /     2.380  -> bf16x3
//   d32_k256       5.985 /     2.873  -> bf16x3
//   d32_k512       9.193 /     4.557  -> bf16x3
//   d64_k16        0.186 /     0.256  -> fp32
//   d64_k32        0.448 /     0.389  -> bf16x3
//   d64_k64        1.366 /     0.866  -> bf16x3
//   d64_k128       4.937 /     2.783  -> bf16x3
//   d64_k256       8.957 /     3.467  -> bf16x3
//   d64_k512      14.866 /     5.445  -> bf16x3
//   d128_k16       0.244 /     0.351  -> fp32
//   d128_k32       0.659 /     0.522  -> bf16x3
//   d128_k64       2.119 /     1.171  -> bf16x3
//   d128_k128      7.800 /     4.053  -> bf16x3
//   d128_k256     15.329 /     5.591  -> bf16x3
//   d128_k512     26.834 /     8.769  -> bf16x3
#pragma once

namespace kmgb {
constexpr int kTunedDims[] = {16, 32, 64, 128};
constexpr int kTunedKMax[] = {16, 32, 64, 128, 256, 512};
// KMGB_ASSIGN_FP32 = 0, KMGB_ASSIGN_BF16X3 = 2
constexpr int kTunedTier[4][6] = {
    {0, 2, 2, 2, 2, 2},
    {0, 0, 2, 2, 2, 2},
    {0, 2, 2, 2, 2, 2},
    {0, 2, 2, 2, 2, 2},
};
}  // namespace kmgb
