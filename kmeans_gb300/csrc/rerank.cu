// Exact re-rank of the points whose approximate top-2 margin did not certify the arg-min.
//
// One warp per flagged point, lanes over centers. Pass 1 evaluates every usable center in
// FP32 together with a rigorous interval [lo_j, hi_j] around the exact value and takes
// best_hi = min_j hi_j. Pass 2 re-evaluates the centers with lo_j <= best_hi (the only ones
// that can be the FP64 arg-min) in FP64 exactly as the oracle does and keeps the smallest,
// lowest index on ties (the reference's tie rule, RowTransformMinimum.cu:43-50). A point with
// a single candidate is settled by FP32 alone; the others are counted as FP64 re-ranks.
//
// mode 0 (Lloyd):      value = sum_d (x_d - c_d)^2     FP32: fma chain of fl(x-c)^2,
//                      |err| <= ((1+u)^2 (1+gamma_D) - 1) * value (all terms non-negative).
// mode 1 (expansion):  value = nb_j - 2 x.c_j with the caller's norms nb (per-kernel ABI,
//                      KmeansCudaKernels.h:238-244); absolute bound from ||x|| and max ||c||.
#include <cfloat>

#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

__device__ __forceinline__ float approx_value(int mode, const float* __restrict__ xs,
                                              const float* __restrict__ c, int d, float nbj) {
  float a = 0.0f;
  if (mode == 0) {
    for (int t = 0; t < d; ++t) {
      const float u = xs[t] - __ldg(c + t);
      a = fmaf(u, u, a);
    }
    return a;
  }
  for (int t = 0; t < d; ++t) a = fmaf(xs[t], __ldg(c + t), a);
  return fmaf(-2.0f, a, nbj);
}

__device__ __forceinline__ double exact_value(int mode, const float* __restrict__ xs,
                                              const float* __restrict__ c, int d, float nbj) {
  double s = 0.0;
  if (mode == 0) {
    for (int t = 0; t < d; ++t) {
      const double u = (double)xs[t] - (double)__ldg(c + t);
      s = fma(u, u, s);
    }
    return s;
  }
  for (int t = 0; t < d; ++t) s = fma((double)xs[t], (double)__ldg(c + t), s);
  return fma(-2.0, s, (double)nbj);
}

__global__ void rerank_kernel(RerankArgs a) {
  if (stopped(a.stop)) return;
  extern __shared__ float xs_all[];
  const int warps = blockDim.x >> 5;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xs = xs_all + (size_t)w * a.d;
  const long long cnt = min((long long)*(volatile const int*)a.count, a.max_list);
  const float u = 5.9604645e-8f;
  const float gam = (float)(a.d + 4) * 2.0f * u * 1.01f;  // mode 0 relative bound (doubled)
  for (long long slot = (long long)blockIdx.x * warps + w; slot < cnt;
       slot += (long long)gridDim.x * warps) {
    const int pt = a.list[slot];
    const float* x = a.X + (size_t)pt * a.ldx;
    for (int t = lane; t < a.d; t += 32) xs[t] = x[t];
    __syncwarp();
    float e1 = 0.0f;
    if (a.mode == 1) {
      const float xn = a.xnorm[pt], cm = *a.cmax;
      const float gd = (float)a.d * u * 1.001f;
      e1 = (2.0f * gd * xn * cm + u * 2.01f * xn * cm +
            (float)(a.d + 2) * 2.3e-16f * xn * cm) * 1.01f;
    }
    // pass 1: best upper end
    float best_hi = INFINITY;
    for (int j = lane; j < a.k; j += 32) {
      float nbj = 0.0f;
      if (a.mode == 0) {
        if (!(a.cn[j] < INFINITY)) continue;  // unusable (empty-cluster) center
      } else {
        nbj = a.nb[j];
      }
      const float v = approx_value(a.mode, xs, a.C + (size_t)j * a.ldc, a.d, nbj);
      float hi;
      if (a.mode == 0) hi = v * (1.0f + gam) + 1e-30f;
      else hi = v + e1 + u * 1.01f * fabsf(nbj) + 1e-30f;
      if (hi < best_hi) best_hi = hi;  // NaN never passes
    }
    for (int o = 16; o > 0; o >>= 1) best_hi = fminf(best_hi, __shfl_xor_sync(0xffffffffu, best_hi, o));
    // pass 2: exact value of every candidate
    double best = INFINITY;
    int bidx = -1;
    int ncand = 0;
    for (int j = lane; j < a.k; j += 32) {
      float nbj = 0.0f;
      if (a.mode == 0) {
        if (!(a.cn[j] < INFINITY)) continue;
      } else {
        nbj = a.nb[j];
      }
      const float* c = a.C + (size_t)j * a.ldc;
      const float v = approx_value(a.mode, xs, c, a.d, nbj);
      float lo;
      if (a.mode == 0) lo = v * (1.0f - gam) - 1e-30f;
      else lo = v - e1 - u * 1.01f * fabsf(nbj) - 1e-30f;
      if (!(lo <= best_hi)) continue;
      ++ncand;
      const double ex = exact_value(a.mode, xs, c, a.d, nbj);
      if (ex < best) {  // lanes visit their centers in increasing j: first wins ties
        best = ex;
        bidx = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
      const bool take = (ob < best) || (ob == best && (unsigned)oi < (unsigned)bidx);
      best = take ? ob : best;
      bidx = take ? oi : bidx;
      ncand += __shfl_xor_sync(0xffffffffu, ncand, o);
    }
    if (lane == 0) {
      a.labels[pt] = bidx < 0 ? 0 : bidx;
      if (a.stats) {
        atomicAdd(a.stats, 1ull);
        if (ncand > 1) atomicAdd(a.stats + 1, 1ull);
      }
    }
    __syncwarp();
  }
}

}  // namespace

cudaError_t launch_rerank(const RerankArgs& a, cudaStream_t s) {
  if (a.n <= 0 || a.k <= 0) return cudaSuccess;
  const int threads = 256;
  const size_t smem = sizeof(float) * (size_t)a.d * (threads / 32);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    KMGB_CUDA_TRY(cudaFuncSetAttribute(rerank_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
  }
  // Persistent grid: the flagged count lives on the device, so no host round trip is needed.
  rerank_kernel<<<152 * 4, threads, smem, s>>>(a); kmgb::count_launches(1);
  return cudaGetLastError();
}

}  // namespace kmgb
