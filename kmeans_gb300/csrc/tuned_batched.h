// Cost of a batched problem's row per Lloyd iteration (ns) by (d, k) bucket and assignment
// family, for kmgb_lloyd_batched_f32 with KMGB_ASSIGN_AUTO. Written by
// kmeans_gb300/autotune.py on NVIDIA GB300, 2026-12-04: per bucket the GPU time of
// 5 Lloyd iterations of synthetic problems with k centers and max(256, 2 k^2)
// rows (ms per iteration, FP32 / split BF16, problems x rows):
//   d16_k16        0.154 /     0.200   200 x 512
//   d16_k32        0.332 /     0.291   200 x 2048
//   d16_k64        1.012 /     0.630   200 x 8192
//   d16_k128       3.583 /     1.877   200 x 32768
//   d16_k256       5.948 /     2.224   61 x 131072
//   d16_k512       9.171 /     3.071   15 x 524288
//   d32_k16        0.159 /     0.195   200 x 512
//   d32_k32        0.330 /     0.313   200 x 2048
//   d32_k64        1.028 /     0.650   200 x 8192
//   d32_k128       3.640 /     1.985   200 x 32768
//   d32_k256       6.008 /     2.380   61 x 131072
//   d32_k512       9.223 /     3.349   15 x 524288
//   d64_k16        0.186 /     0.250   200 x 512
//   d64_k32        0.451 /     0.365   200 x 2048
//   d64_k64        1.374 /     0.766   200 x 8192
//   d64_k128       4.962 /     2.385   200 x 32768
//   d64_k256       8.996 /     2.965   61 x 131072
//   d64_k512      14.916 /     4.266   15 x 524288
//   d128_k16       0.244 /     0.342   200 x 512
//   d128_k32       0.662 /     0.497   200 x 2048
//   d128_k64       2.122 /     1.060   200 x 8192
//   d128_k128      7.836 /     3.596   200 x 32768
//   d128_k256     15.368 /     4.986   61 x 131072
//   d128_k512     26.907 /     7.568   15 x 524288
#pragma once

namespace kmgb {
constexpr int kTunedDims[] = {16, 32, 64, 128};
constexpr int kTunedKMax[] = {16, 32, 64, 128, 256, 512};
// [family: 0 FP32, 1 split BF16][dimension bucket][center bucket]
constexpr float kTunedNsPerRow[2][4][6] = {
    {
        {1.5001f, 0.8097f, 0.61781f, 0.54675f, 0.74397f, 1.1661f},
        {1.5534f, 0.80617f, 0.62761f, 0.55545f, 0.75146f, 1.1727f},
        {1.816f, 1.1021f, 0.83851f, 0.75711f, 1.1252f, 1.8966f},
        {2.3839f, 1.6152f, 1.2949f, 1.1957f, 1.9221f, 3.4214f},
    },
    {
        {1.9489f, 0.71084f, 0.38425f, 0.28634f, 0.27815f, 0.39049f},
        {1.9048f, 0.76425f, 0.39654f, 0.30288f, 0.29766f, 0.42584f},
        {2.4391f, 0.88995f, 0.46748f, 0.36387f, 0.37086f, 0.54246f},
        {3.343f, 1.214f, 0.64674f, 0.54872f, 0.6236f, 0.96238f},
    },
};
}  // namespace kmgb
