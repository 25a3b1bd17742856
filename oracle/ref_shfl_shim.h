// Force-included when the reference's ClosestCenters.cu is compiled into a cubin for sm_103a
// (test infrastructure: the oracle drives the reference's own assignment kernels on the GPU).
// The reference calls the pre-Volta three-argument warp shuffles, which CUDA 13 no longer
// provides; these map them onto the synchronising forms with a full-warp mask (every lane of the
// reference's 16x16 blocks executes its reductions).
#pragma once
#define __shfl_down(v, d, w) __shfl_down_sync(0xffffffffu, (v), (d), (w))
#define __shfl_up(v, d, w) __shfl_up_sync(0xffffffffu, (v), (d), (w))
