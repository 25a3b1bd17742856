// Exact re-rank of the points whose approximate top-2 margin did not certify the arg-min.
//
// Stages in this file: the candidate path of the tensor tiers (gather_flagged_kernel copies the
// flagged rows for the candidate pass; resolve_candidates_kernel settles each point from its
// recorded candidates in FP32, then float-float, then exact FP64), the tiled FP32 stage and the
// tiled exact FP64 stage for everything else, the per-point kernel described next (both modes),
// and the grouped kernel of batched problems.
//
// Per-point kernel: one warp per flagged point, lanes over centers. Pass 1 evaluates every usable center in
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
#include <cstdint>

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

// Tiled FP32 stage of the Lloyd re-rank (mode 0): 32 flagged points per CTA iteration against
// 64-center blocks staged in shared memory; each thread accumulates 4 points x 2 centers of
// sum_d (x_d - c_d)^2 with float4 loads. Per point (best, index, second) is merged over the 32
// threads that share it (lowest index on ties) and certified with the relative bound of the
// direct form; uncertified points go to list2 for the exact FP64 stage.
constexpr int TP = 32;   // points per CTA iteration
constexpr int TC = 64;   // centers per block

__global__ void __launch_bounds__(256)
rerank_tiled_kernel(RerankArgs a, int* __restrict__ list2, int* __restrict__ count2,
                    float* __restrict__ hi2) {
  if (stopped(a.stop)) return;
  extern __shared__ float4 sm4[];
  const int dq = (a.d + 3) >> 2;          // float4 per row
  const int rs = dq + 1;                  // row stride in float4 (padded: conflict-free)
  float4* xs = sm4;                       // [TP][rs]
  float4* cs = xs + TP * rs;              // [TC][rs]
  float* cflag = reinterpret_cast<float*>(cs + TC * rs);  // [TC] 0 usable, +inf unusable
  __shared__ float mb1[8][TP], mb2[8][TP];
  __shared__ int mi1[8][TP];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int pq = tid & 7;                 // points pq*4 .. pq*4+3
  const int cq = tid >> 3;                // centers cq*2, cq*2+1 of the block
  const long long cnt = min((long long)*(volatile const int*)a.count, a.max_list);
  const float u = 5.9604645e-8f;
  const float gam = (float)(a.d + 4) * 2.0f * u * 1.01f;

  for (long long g0 = (long long)blockIdx.x * TP; g0 < cnt; g0 += (long long)gridDim.x * TP) {
    __syncthreads();
    // stage the points (zero rows past the list end)
    for (int e = tid; e < TP * dq; e += blockDim.x) {
      const int r = e / dq, q = e % dq;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (g0 + r < cnt) {
        const float* x = a.X + (size_t)a.list[g0 + r] * a.ldx;
        const int c0 = q * 4;
        v.x = c0 < a.d ? x[c0] : 0.f;
        v.y = c0 + 1 < a.d ? x[c0 + 1] : 0.f;
        v.z = c0 + 2 < a.d ? x[c0 + 2] : 0.f;
        v.w = c0 + 3 < a.d ? x[c0 + 3] : 0.f;
      }
      xs[r * rs + q] = v;
    }
    float b1[4], b2[4];
    int i1[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      b1[i] = INFINITY;
      b2[i] = INFINITY;
      i1[i] = -1;
    }
    for (int j0 = 0; j0 < a.k; j0 += TC) {
      __syncthreads();
      for (int e = tid; e < TC * dq; e += blockDim.x) {
        const int r = e / dq, q = e % dq;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j0 + r < a.k) {
          const float* c = a.C + (size_t)(j0 + r) * a.ldc;
          const int c0 = q * 4;  // ldc is a multiple of 4 and rows are zero padded
          v = *reinterpret_cast<const float4*>(c + c0);
        }
        cs[r * rs + q] = v;
      }
      if (tid < TC) {
        const int j = j0 + tid;
        cflag[tid] = (j < a.k && a.cn[j] < INFINITY) ? 0.0f : INFINITY;
      }
      __syncthreads();
      float acc[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = 0.0f;
      for (int q = 0; q < dq; ++q) {
        const float4 c0 = cs[(cq * 2) * rs + q];
        const float4 c1 = cs[(cq * 2 + 1) * rs + q];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 x = xs[(pq * 4 + i) * rs + q];
          float t;
          t = x.x - c0.x; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.y - c0.y; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.z - c0.z; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.w - c0.w; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.x - c1.x; acc[i][1] = fmaf(t, t, acc[i][1]);
          t = x.y - c1.y; acc[i][1] = fmaf(t, t, acc[i][1]);
          t = x.z - c1.z; acc[i][1] = fmaf(t, t, acc[i][1]);
          t = x.w - c1.w; acc[i][1] = fmaf(t, t, acc[i][1]);
        }
      }
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const int j = j0 + cq * 2 + jj;
        const float f = cflag[cq * 2 + jj];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float v = acc[i][jj] + f;  // +inf for unusable / padding centers
          const float nb2 = fminf(b2[i], fmaxf(b1[i], v));
          const bool lt = v < b1[i];
          b1[i] = lt ? v : b1[i];
          i1[i] = lt ? j : i1[i];
          b2[i] = nb2;
        }
      }
    }
    // merge the 32 threads of each point: lanes pq, pq+8, pq+16, pq+24 of every warp
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
      for (int off = 8; off < 32; off <<= 1) {
        const float ob1 = __shfl_xor_sync(0xffffffffu, b1[i], off);
        const float ob2 = __shfl_xor_sync(0xffffffffu, b2[i], off);
        const int oi1 = __shfl_xor_sync(0xffffffffu, i1[i], off);
        const float nb2 = fminf(fminf(b2[i], ob2), fmaxf(b1[i], ob1));
        const bool take = (ob1 < b1[i]) || (ob1 == b1[i] && (unsigned)oi1 < (unsigned)i1[i]);
        b1[i] = take ? ob1 : b1[i];
        i1[i] = take ? oi1 : i1[i];
        b2[i] = nb2;
      }
      if (lane < 8) {
        mb1[w][pq * 4 + i] = b1[i];
        mb2[w][pq * 4 + i] = b2[i];
        mi1[w][pq * 4 + i] = i1[i];
      }
    }
    __syncthreads();
    if (tid < TP && g0 + tid < cnt) {
      float f1 = mb1[0][tid], f2 = mb2[0][tid];
      int fi = mi1[0][tid];
      for (int ww = 1; ww < 8; ++ww) {
        const float ob1 = mb1[ww][tid], ob2 = mb2[ww][tid];
        const int oi1 = mi1[ww][tid];
        const float nb2 = fminf(fminf(f2, ob2), fmaxf(f1, ob1));
        const bool take = (ob1 < f1) || (ob1 == f1 && (unsigned)oi1 < (unsigned)fi);
        f1 = take ? ob1 : f1;
        fi = take ? oi1 : fi;
        f2 = nb2;
      }
      const int pt = a.list[g0 + tid];
      // certified when every other center's lower end exceeds the best's upper end
      if (fi >= 0 && f2 * (1.0f - gam) - 1e-30f > f1 * (1.0f + gam) + 1e-30f) {
        a.labels[pt] = fi;
      } else {
        const int slot = atomicAdd(count2, 1);
        list2[slot] = pt;
        hi2[slot] = f1 * (1.0f + gam) + 1e-30f;  // no usable center: +inf
      }
    }
  }
}

// Exact stage of the Lloyd re-rank (mode 0), tiled like the FP32 stage: 32 residual points per
// CTA iteration against 64-center blocks staged in shared memory. Every (point, usable center)
// pair whose FP32 direct-form lower end is within the point's best upper end (hi2, from the FP32
// stage) is evaluated in FP64 in the oracle's order (sequential fma over the dimensions); the
// smallest value wins, lowest index on ties. Centers are read once per 32 points, so the cost
// stays that of one tiled FP32 scan however many points reach this stage.
__global__ void __launch_bounds__(256)
rerank_exact_kernel(RerankArgs a, const float* __restrict__ hi2) {
  if (stopped(a.stop)) return;
  extern __shared__ float4 sm4[];
  const int dq = (a.d + 3) >> 2;
  const int rs = dq + 1;
  float4* xs = sm4;                       // [TP][rs]
  float4* cs = xs + TP * rs;              // [TC][rs]
  float* cflag = reinterpret_cast<float*>(cs + TC * rs);  // [TC] 0 usable, +inf unusable
  __shared__ double mb[8][TP];
  __shared__ int mi[8][TP];
  __shared__ float hs[TP];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int pq = tid & 7;                 // points pq*4 .. pq*4+3
  const int cq = tid >> 3;                // centers cq*2, cq*2+1 of the block
  const long long cnt = min((long long)*(volatile const int*)a.count, a.max_list);
  const float u = 5.9604645e-8f;
  const float gam = (float)(a.d + 4) * 2.0f * u * 1.01f;

  for (long long g0 = (long long)blockIdx.x * TP; g0 < cnt; g0 += (long long)gridDim.x * TP) {
    __syncthreads();
    for (int e = tid; e < TP * dq; e += blockDim.x) {
      const int r = e / dq, q = e % dq;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (g0 + r < cnt) {
        const float* x = a.X + (size_t)a.list[g0 + r] * a.ldx;
        const int c0 = q * 4;
        v.x = c0 < a.d ? x[c0] : 0.f;
        v.y = c0 + 1 < a.d ? x[c0 + 1] : 0.f;
        v.z = c0 + 2 < a.d ? x[c0 + 2] : 0.f;
        v.w = c0 + 3 < a.d ? x[c0 + 3] : 0.f;
      }
      xs[r * rs + q] = v;
    }
    if (tid < TP) hs[tid] = (g0 + tid < cnt) ? hi2[g0 + tid] : -INFINITY;
    double be[4];
    int bi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      be[i] = INFINITY;
      bi[i] = -1;
    }
    for (int j0 = 0; j0 < a.k; j0 += TC) {
      __syncthreads();
      for (int e = tid; e < TC * dq; e += blockDim.x) {
        const int r = e / dq, q = e % dq;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j0 + r < a.k) v = *reinterpret_cast<const float4*>(a.C + (size_t)(j0 + r) * a.ldc + q * 4);
        cs[r * rs + q] = v;
      }
      if (tid < TC) {
        const int j = j0 + tid;
        cflag[tid] = (j < a.k && a.cn[j] < INFINITY) ? 0.0f : INFINITY;
      }
      __syncthreads();
      float acc[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = 0.0f;
      for (int q = 0; q < dq; ++q) {
        const float4 c0 = cs[(cq * 2) * rs + q];
        const float4 c1 = cs[(cq * 2 + 1) * rs + q];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 x = xs[(pq * 4 + i) * rs + q];
          float t;
          t = x.x - c0.x; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.y - c0.y; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.z - c0.z; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.w - c0.w; acc[i][0] = fmaf(t, t, acc[i][0]);
          t = x.x - c1.x; acc[i][1] = fmaf(t, t, acc[i][1]);
          t = x.y - c1.y; acc[i][1] = fmaf(t, t, acc[i][1]);
          t = x.z - c1.z; acc[i][1] = fmaf(t, t, acc[i][1]);
          t = x.w - c1.w; acc[i][1] = fmaf(t, t, acc[i][1]);
        }
      }
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const int cl = cq * 2 + jj;
        const int j = j0 + cl;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int pl = pq * 4 + i;
          if (cflag[cl] != 0.0f) continue;  // unusable (empty-cluster) or padding center
          const float v = acc[i][jj];
          if (!(v * (1.0f - gam) - 1e-30f <= hs[pl])) continue;
          // FP64 in the oracle's order: dimensions 0 .. d-1 (padding dimensions are zero)
          double ex = 0.0;
          for (int q = 0; q < dq; ++q) {
            const float4 x = xs[pl * rs + q];
            const float4 c = cs[cl * rs + q];
            double dd;
            dd = (double)x.x - (double)c.x; ex = fma(dd, dd, ex);
            dd = (double)x.y - (double)c.y; ex = fma(dd, dd, ex);
            dd = (double)x.z - (double)c.z; ex = fma(dd, dd, ex);
            dd = (double)x.w - (double)c.w; ex = fma(dd, dd, ex);
          }
          if (ex < INFINITY && (ex < be[i] || (ex == be[i] && (unsigned)j < (unsigned)bi[i]))) {
            be[i] = ex;
            bi[i] = j;
          }
        }
      }
    }
    // merge the 32 threads of each point: lanes pq, pq+8, pq+16, pq+24 of every warp
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
      for (int off = 8; off < 32; off <<= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, be[i], off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi[i], off);
        const bool take = (ob < be[i]) || (ob == be[i] && (unsigned)oi < (unsigned)bi[i]);
        be[i] = take ? ob : be[i];
        bi[i] = take ? oi : bi[i];
      }
      if (lane < 8) {
        mb[w][pq * 4 + i] = be[i];
        mi[w][pq * 4 + i] = bi[i];
      }
    }
    __syncthreads();
    if (tid < TP && g0 + tid < cnt) {
      double fb = mb[0][tid];
      int fi = mi[0][tid];
      for (int ww = 1; ww < 8; ++ww) {
        const bool take = (mb[ww][tid] < fb) || (mb[ww][tid] == fb && (unsigned)mi[ww][tid] < (unsigned)fi);
        fb = take ? mb[ww][tid] : fb;
        fi = take ? mi[ww][tid] : fi;
      }
      a.labels[a.list[g0 + tid]] = fi < 0 ? 0 : fi;
    }
  }
}

// Grouped (batched Lloyd) re-rank, one warp per flagged row of any problem; the row's own
// problem (tile_prob[row / 128]) gives its center range. Pass 1, FP32 direct form: the lanes
// split the dimensions of four centers at a time (coalesced rows, a tree sum per center -- like
// any order it stays within the (d+4) 2u relative bound of a sum of non-negative terms); the
// values of up to RG_VCAP centers stay in shared memory. Pass 2: every usable center whose FP32
// lower end is within the smallest upper end is evaluated in FP64 in the oracle's order
// (sequential fma over the dimensions), the smallest value winning, lowest index on ties.
// Labels are global center indices.
constexpr int RG_VCAP = 512;
constexpr int RG_WARPS = 8;

__global__ void __launch_bounds__(RG_WARPS * 32)
rerank_grouped_kernel(RerankArgs a, GroupArgs g, int* __restrict__ cand, int* __restrict__ cand_cnt,
                      long long cand_cap) {
  if (stopped(a.stop)) return;
  extern __shared__ float rg_smem[];  // [warps][RG_VCAP] values, then [warps][d] rows
  const long long cnt = min((long long)*(volatile const int*)a.count, a.max_list);
  const float u = 5.9604645e-8f;
  const float gam = (float)(a.d + 4) * 2.0f * u * 1.01f;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float* vals = rg_smem + (size_t)w * RG_VCAP;
  float* xs = rg_smem + (size_t)RG_WARPS * RG_VCAP + (size_t)w * a.d;
  for (long long slot = (long long)blockIdx.x * RG_WARPS + w; slot < cnt;
       slot += (long long)gridDim.x * RG_WARPS) {
    const int pt = a.list[slot];
    const int prob = g.tile_prob[pt >> 7];
    const int cbeg = g.c_off[prob], kp = g.k[prob];
    const bool keep = kp <= RG_VCAP;
    const float* x = a.X + (size_t)pt * a.ldx;
    __syncwarp();
    for (int t = lane; t < a.d; t += 32) xs[t] = x[t];
    __syncwarp();
    float lo = INFINITY;
    for (int j0 = 0; j0 < kp; j0 += 4) {
      float sv[4] = {0.f, 0.f, 0.f, 0.f};
      const float* cr[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        cr[r] = a.C + (size_t)(cbeg + min(j0 + r, kp - 1)) * a.ldc;
      for (int t = lane; t < a.d; t += 32) {
        const float xt = xs[t];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const float df = xt - __ldg(cr[r] + t);
          sv[r] = fmaf(df, df, sv[r]);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int r = 0; r < 4; ++r) sv[r] += __shfl_xor_sync(0xffffffffu, sv[r], o);
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int j = j0 + r;
        if (j < kp) {
          const float v = (a.cn[cbeg + j] < INFINITY) ? sv[r] : INFINITY;  // unusable center
          lo = fminf(lo, v);
          if (keep && lane == 0) vals[j] = v;
        }
      }
    }
    __syncwarp();
    const float best_hi = lo * (1.0f + gam) + 1e-30f;
    if (cand && slot < cand_cap) {
      // record the band (every center whose FP64 distance can be the minimum) for the
      // candidate resolve's FP32 and float-float tiers; more than kMaxCand: the exact pass
      int n_in = 0;
      for (int j0 = 0; j0 < kp; j0 += 32) {
        const int j = j0 + lane;
        bool in = false;
        if (j < kp && a.cn[cbeg + j] < INFINITY) {
          const float v = keep ? vals[j] : approx_value(0, xs, a.C + (size_t)(cbeg + j) * a.ldc,
                                                        a.d, 0.0f);
          in = v * (1.0f - gam) - 1e-30f <= best_hi;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, in);
        const int at = n_in + __popc(bal & ((1u << lane) - 1u));
        if (in && at < kMaxCand) cand[slot * kMaxCand + at] = cbeg + j;
        n_in += __popc(bal);
      }
      if (lane == 0) {
        cand_cnt[slot] = n_in <= kMaxCand ? n_in : -1;
        if (a.stats) atomicAdd(a.stats, 1ull);
      }
      continue;
    }
    double best = INFINITY;
    int bidx = -1;
    for (int j = lane; j < kp; j += 32) {
      if (!(a.cn[cbeg + j] < INFINITY)) continue;
      const float* c = a.C + (size_t)(cbeg + j) * a.ldc;
      const float v = keep ? vals[j] : approx_value(0, xs, c, a.d, 0.0f);
      if (!(v * (1.0f - gam) - 1e-30f <= best_hi)) continue;
      const double ex = exact_value(0, xs, c, a.d, 0.0f);
      if (ex < best) {  // a lane's centers come in increasing index order
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
    }
    if (lane == 0) {
      a.labels[pt] = cbeg + (bidx < 0 ? 0 : bidx);
      if (a.stats) atomicAdd(a.stats, 1ull);
    }
  }
}

}  // namespace

namespace {
__global__ void count_stats_kernel(const int* counts, int full_idx, unsigned long long* stats,
                                   const int* stop) {
  if (stopped(stop)) return;
  stats[0] += (unsigned long long)counts[0];
  stats[1] += (unsigned long long)counts[full_idx];
}

// Copies the BF16 rows (and residual rows) of the flagged points into a compact buffer, row
// `slot` for list[slot], with the point's candidate floor. One warp per row, 16-byte moves. The
// compact buffer holds `cap` rows; flagged points beyond it go straight to `over` (the full
// rescan), so any number of flagged points is settled exactly.
__global__ void gather_flagged_kernel(const int* __restrict__ list, const int* __restrict__ count,
                                      long long cap, const uint4* __restrict__ Xb,
                                      const uint4* __restrict__ Xl, long long row_vec,
                                      const float* __restrict__ thr, uint4* __restrict__ XbC,
                                      uint4* __restrict__ XlC, float* __restrict__ thrC,
                                      int* __restrict__ over, int* __restrict__ over_count,
                                      const int* stop, const float* __restrict__ xs,
                                      float* __restrict__ xsC) {
  if (stopped(stop)) return;
  const long long total = *(volatile const int*)count;
  const long long cnt = min(total, cap);
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long slot = cap + w0 * 32 + lane; slot < total; slot += nw * 32)
    over[atomicAdd(over_count, 1)] = list[slot];
  for (long long slot = w0; slot < cnt; slot += nw) {
    const long long pt = list[slot];
    for (long long v = lane; v < row_vec; v += 32) {
      XbC[slot * row_vec + v] = Xb[pt * row_vec + v];
      if (Xl) XlC[slot * row_vec + v] = Xl[pt * row_vec + v];
    }
    if (lane == 0) {
      thrC[slot] = thr[pt];
      if (xs) xsC[slot] = xs[pt];
    }
  }
}

// Error-free float-float helpers (FP32 pipe). two_sum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

constexpr int kGroupLanes = 8;  // lanes per candidate in the fast path: 4 candidates at a time
static_assert(kMaxCand <= 32, "one lane per recorded candidate");

// One term of ||x - c||^2 into the float-float (hi, lo): u = x - c is split exactly into uh + ul
// (two_sum), uh^2 = p + e exactly (FMA), and the remaining 2*uh*ul + ul^2 + e is added with one
// rounding; hi collects the p's by two_sum, lo the rest.
__device__ __forceinline__ void ff_term(float xv, float cv, float& hi, float& lo) {
  float uh, ul;
  two_sum(xv, -cv, uh, ul);
  const float p = __fmul_rn(uh, uh);
  const float e = __fmaf_rn(uh, uh, -p);
  const float r = __fmaf_rn(ul, ul, __fmaf_rn(__fadd_rn(uh, uh), ul, e));
  float s, err;
  two_sum(hi, p, s, err);
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(err, r));
}

// ||x - c||^2 over the first d dimensions as a float-float (hi, lo), summed over each group of
// 8 consecutive lanes (every lane of a group ends with its group's total; all 32 lanes call it,
// a group with nothing to do passes d = 0). Lane r of a group takes dimensions 4r..4r+3,
// 4r+32.. with 16-byte loads (VEC: d, both row strides and both bases multiples of 4 floats),
// else r, r+8, ...: at most m = 4 ceil(d/32) terms per lane, then three reduction levels.
template <bool VEC>
__device__ __forceinline__ void ff_dist8(const float* __restrict__ x, const float* __restrict__ c,
                                         int d, int r, float& hi, float& lo) {
  hi = 0.0f;
  lo = 0.0f;
  if (VEC) {
    for (int t = 4 * r; t < d; t += 4 * kGroupLanes) {
      const float4 xv = __ldg(reinterpret_cast<const float4*>(x + t));
      const float4 cv = __ldg(reinterpret_cast<const float4*>(c + t));
      ff_term(xv.x, cv.x, hi, lo);
      ff_term(xv.y, cv.y, hi, lo);
      ff_term(xv.z, cv.z, hi, lo);
      ff_term(xv.w, cv.w, hi, lo);
    }
  } else {
    for (int t = r; t < d; t += kGroupLanes) ff_term(__ldg(x + t), __ldg(c + t), hi, lo);
  }
  for (int o = kGroupLanes / 2; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    float s, err;
    two_sum(hi, oh, s, err);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(ol, err));
  }
}

// ||x - c||^2 over the first d dimensions in FP32, summed over each group of 8 consecutive lanes
// (all 32 lanes call it; a group with nothing to do passes d = 0). Every step is one explicitly
// rounded operation: u = x - c, then s = u*u + s by FMA. VEC: four independent chains per lane
// (the float4 components, at most ceil(d/32) terms each) merged in two levels, then three
// butterfly levels; scalar: one chain of at most ceil(d/8) terms, then three levels.
template <bool VEC>
__device__ __forceinline__ float f32_dist8(const float* __restrict__ x, const float* __restrict__ c,
                                           int d, int r) {
  float s;
  if (VEC) {
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int t = 4 * r; t < d; t += 4 * kGroupLanes) {
      const float4 xv = __ldg(reinterpret_cast<const float4*>(x + t));
      const float4 cv = __ldg(reinterpret_cast<const float4*>(c + t));
      const float u0 = __fsub_rn(xv.x, cv.x), u1 = __fsub_rn(xv.y, cv.y);
      const float u2 = __fsub_rn(xv.z, cv.z), u3 = __fsub_rn(xv.w, cv.w);
      a0 = __fmaf_rn(u0, u0, a0);
      a1 = __fmaf_rn(u1, u1, a1);
      a2 = __fmaf_rn(u2, u2, a2);
      a3 = __fmaf_rn(u3, u3, a3);
    }
    s = __fadd_rn(__fadd_rn(a0, a1), __fadd_rn(a2, a3));
  } else {
    s = 0.0f;
    for (int t = r; t < d; t += kGroupLanes) {
      const float u = __fsub_rn(__ldg(x + t), __ldg(c + t));
      s = __fmaf_rn(u, u, s);
    }
  }
  for (int o = kGroupLanes / 2; o > 0; o >>= 1)
    s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
  return s;
}

// Resolves every flagged point from its recorded candidates. The candidate set holds every center
// whose FP64 distance can be the minimum; the label is the oracle's: smallest FP64 distance
// (sequential fma over the dimensions), lowest index on ties.
//
// First tier (FP32, 8 lanes per candidate, 4 candidates at a time): every term of the FP32 value
// is non-negative and passes through at most m + 7 roundings of 2^-24 (the subtraction twice, as
// u^2, then at most m = ceil(d/8) FMAs, two merges and three butterfly levels), so it is within
// rel32 = (m + 8) 2^-24 (x1.1) of the exact distance, plus abs32 for results in the subnormal
// range; with the oracle's own (d+2) 2^-52, a best candidate ahead of the runner-up by more than
// both is the oracle's arg-min. Flagged points are mostly ahead by far more than that.
//
// Second tier (FP32 pipe, 8 lanes per candidate, 4 candidates at a time): the float-float distance
// v of each candidate is within rel*v + abs of the exact distance, and the oracle's FP64 value is
// within (d+2)*2^-52 relative of it. Per lane (m = 4 ceil(d/32) terms) the lo accumulator's
// roundings are bounded by (m+1)^2 * 2^-47 relative, the 2*uh*ul + ul^2 + e terms by 2^-46, the
// three reduction levels by 3 * (m+6) * 2^-47; rel takes 8x that sum. abs covers products that
// reach the subnormal range. If the best candidate beats the runner-up by more than both
// tolerances, it is the oracle's arg-min. Otherwise (near ties, duplicate centers, non-finite
// values) the point's candidates are evaluated exactly as the oracle does, one lane per
// candidate, in FP64. Points with more candidates than recorded (or none) go to `over` for the
// full re-rank.
template <bool VEC>
__global__ void resolve_candidates_kernel(const int* __restrict__ list, const int* __restrict__ count,
                                          long long max_list, const int* __restrict__ cand,
                                          const int* __restrict__ cand_cnt,
                                          const float* __restrict__ X, long long ldx,
                                          const float* __restrict__ C, long long ldc,
                                          const float* __restrict__ cn, int d,
                                          int* __restrict__ labels, int* __restrict__ over,
                                          int* __restrict__ over_count, const int* stop,
                                          const int* __restrict__ row_map) {
  if (stopped(stop)) return;
  const long long cnt = min((long long)*(volatile const int*)count, max_list);
  const int lane = threadIdx.x & 31;
  const int grp = lane / kGroupLanes, sub = lane % kGroupLanes;
  constexpr int kGroups = 32 / kGroupLanes;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const double m = 4.0 * (double)((d + 31) / 32);
  const double rel = 8.0 * ((m + 1.0) * (m + 1.0) + 2.0 + 3.0 * (m + 6.0)) * 0x1p-47 +
                     (double)(d + 2) * 0x1p-52;
  const double abs_tol = (double)(d + 32) * 0x1p-118;
  const double m32 = (double)((d + kGroupLanes - 1) / kGroupLanes);
  const double rel32 = 1.1 * (m32 + 8.0) * 0x1p-24 + (double)(d + 2) * 0x1p-52;
  const double abs32 = (double)(d + 32) * (m32 + 8.0) * 0x1p-149;
  for (long long slot = w0; slot < cnt; slot += nw) {
    const int pt = list[slot];
    // with row_map (routed scan) the candidates are kept per routed row pt, and the point's FP32
    // row is row_map[pt]; otherwise per list slot, and the row is pt
    const long long ci = row_map ? (long long)pt : slot;
    const int nc = cand_cnt[ci];
    if (nc <= 0 || nc > kMaxCand) {
      if (lane == 0) over[atomicAdd(over_count, 1)] = pt;
      continue;
    }
    const float* x = X + (size_t)(row_map ? row_map[pt] : pt) * ldx;
    // lane q holds candidate q and whether it is usable
    const int myj = lane < nc ? cand[ci * kMaxCand + lane] : -1;
    const int myok = (myj >= 0 && cn[myj] < INFINITY) ? 1 : 0;
    // both fast tiers certify only a strict separation, so the list order (column slice by
    // column slice) does not matter
    double v1 = INFINITY, v2 = INFINITY;
    int i1 = -1;
    bool finite = true;
    for (int q0 = 0; q0 < nc; q0 += kGroups) {
      const int q = q0 + grp;  // <= 31: q0 is a multiple of 4 below nc <= kMaxCand = 32
      const int j = __shfl_sync(0xffffffffu, myj, q);
      const int ok = __shfl_sync(0xffffffffu, myok, q) && q < nc;
      const float v = f32_dist8<VEC>(x, ok ? C + (size_t)j * ldc : x, ok ? d : 0, sub);
      for (int g = 0; g < kGroups; ++g) {
        const double vg = (double)__shfl_sync(0xffffffffu, v, g * kGroupLanes);
        const int jg = __shfl_sync(0xffffffffu, j, g * kGroupLanes);
        if (!__shfl_sync(0xffffffffu, ok, g * kGroupLanes)) continue;
        if (!(vg < 3.0e38)) finite = false;  // overflow, inf or NaN
        if (vg < v1) {
          v2 = v1;
          v1 = vg;
          i1 = jg;
        } else if (vg < v2) {
          v2 = vg;
        }
      }
    }
    if (i1 < 0) {  // no usable candidate
      if (lane == 0) over[atomicAdd(over_count, 1)] = pt;
      continue;
    }
    // one usable candidate (v2 infinite, its value finite) is the arg-min itself
    if (finite && (v2 == INFINITY || v2 - v1 > (v1 + v2) * rel32 + 2.0 * abs32)) {
      if (lane == 0) labels[pt] = i1;
      continue;
    }
    v1 = INFINITY;
    v2 = INFINITY;
    i1 = -1;
    finite = true;
    for (int q0 = 0; q0 < nc; q0 += kGroups) {
      const int q = q0 + grp;  // <= 31: q0 is a multiple of 4 below nc <= kMaxCand = 32
      const int j = __shfl_sync(0xffffffffu, myj, q);
      const int ok = __shfl_sync(0xffffffffu, myok, q) && q < nc;
      float hi, lo;
      ff_dist8<VEC>(x, ok ? C + (size_t)j * ldc : x, ok ? d : 0, sub, hi, lo);
      const double v = (double)hi + (double)lo;
      for (int g = 0; g < kGroups; ++g) {
        const double vg = __shfl_sync(0xffffffffu, v, g * kGroupLanes);
        const int jg = __shfl_sync(0xffffffffu, j, g * kGroupLanes);
        if (!__shfl_sync(0xffffffffu, ok, g * kGroupLanes)) continue;
        if (!(vg < 1.0e300)) finite = false;  // overflow, inf or NaN on the FP32 pipe
        if (vg < v1) {
          v2 = v1;
          v1 = vg;
          i1 = jg;
        } else if (vg < v2) {
          v2 = vg;
        }
      }
    }
    if (i1 < 0) {  // no usable candidate
      if (lane == 0) over[atomicAdd(over_count, 1)] = pt;
      continue;
    }
    // one usable candidate (v2 infinite, every value finite) is the arg-min itself; the
    // comparison below would read inf > inf
    if (finite && (v2 == INFINITY || v2 - v1 > (v1 + v2) * rel + 2.0 * abs_tol)) {
      if (lane == 0) labels[pt] = i1;
      continue;
    }
    // exact path: the oracle's sequential FP64 evaluation, lane l taking candidates l, l+32, ...;
    // equal values go to the lowest center index, within a lane and across lanes
    double best = INFINITY;
    int bidx = -1;
    for (int q = lane; q < nc; q += 32) {
      const int j = cand[ci * kMaxCand + q];
      if (cn[j] < INFINITY) {
        const float* c = C + (size_t)j * ldc;
        double s = 0.0;
        for (int t = 0; t < d; ++t) {
          const double u = (double)__ldg(x + t) - (double)__ldg(c + t);
          s = fma(u, u, s);
        }
        if (s < INFINITY && (s < best || (s == best && (unsigned)j < (unsigned)bidx))) {
          best = s;  // the oracle never takes a NaN or infinite distance
          bidx = j;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
      const bool take = (ob < best) || (ob == best && (unsigned)oi < (unsigned)bidx);
      best = take ? ob : best;
      bidx = take ? oi : bidx;
    }
    if (lane == 0) {
      if (bidx < 0) over[atomicAdd(over_count, 1)] = pt;
      else labels[pt] = bidx;
    }
  }
}

// ------------------------------- audit of certified labels -------------------------------
// A rotating sample of rows is checked against the FP64 arg-min over every center, so that a
// failure of a rounding model the certificate relies on (the tensor tiers' accumulation bound,
// the router's separation bound) shows as a counted violation instead of a silently wrong label.
// A violation is a center strictly nearer than the label in FP64 (exact_value, the oracle's
// expression and order); ties are not judged. Distances are first evaluated in FP32, one warp
// per center with the lanes over the dimensions (coalesced rows), each with an interval: any
// summation order of the d non-negative rounded squares stays within (d + 2) 2^-24 relative to
// first order, 2.02x that plus an absolute d 2^-125 for underflow is used. A center whose
// interval lies below the label's is a violation; only overlapping intervals (near ties) are
// decided in FP64, which keeps the narrow FP64 pipe of GB300 out of the scan.
// ws: [0] rows audited, [1] violations, [2] sampling sequence, [3] 1 + the last violating row,
// then per sampled row a violation flag [rows] and the row [rows].
__device__ __forceinline__ unsigned long long audit_hash(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// FP32 squared distance of the shared row to center c, lanes over the dimensions (every lane
// returns the warp's sum).
__device__ __forceinline__ float audit_dist32(const float* ax, const float* __restrict__ c, int d,
                                              int lane) {
  float a = 0.0f;
  for (int t = lane; t < d; t += 32) {
    const float u = ax[t] - __ldg(c + t);
    a = fmaf(u, u, a);
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  return a;
}

// The same for four consecutive centers j .. j + 3 (clamped to jend - 1), their loads and trees
// interleaved; every center's sum is formed exactly as audit_dist32 forms it.
__device__ __forceinline__ void audit_dist32x4(const float* ax, const float* __restrict__ C,
                                               long long ldc, int j, int jend, int d, int lane,
                                               float out[4]) {
  const float* c[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    c[u] = C + (size_t)min(j + u, jend - 1) * ldc;
    out[u] = 0.0f;
  }
  for (int t = lane; t < d; t += 32) {
    const float xt = ax[t];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float v = xt - __ldg(c[u] + t);
      out[u] = fmaf(v, v, out[u]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int u = 0; u < 4; ++u) out[u] += __shfl_xor_sync(0xffffffffu, out[u], o);
  }
}

__global__ void __launch_bounds__(256)
audit_scan_kernel(const float* __restrict__ X, long long ldx, long long n, int d,
                  const float* __restrict__ C, long long ldc, int k,
                  const int* __restrict__ labels, unsigned long long* ws, int rows, int parts,
                  GroupArgs g, const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ float ax[];
  __shared__ int viol_sh;
  const int r = blockIdx.x / parts, part = blockIdx.x % parts;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const unsigned long long seq = *reinterpret_cast<volatile unsigned long long*>(ws + 2);
  const long long row = (long long)(audit_hash(seq + (unsigned long long)r) % (unsigned long long)n);
  // batched problems: the row's problem and its centers; padding rows and rows of stopped
  // problems (their labels belong to the centers before the last update) are not audited
  int cbeg = 0, kk = k;
  if (g.tile_prob) {
    const int prob = g.tile_prob[row >> 7];
    if (row >= g.row_end[prob] || (g.done && g.done[prob])) {  // uniform over the block
      if (threadIdx.x == 0 && part == 0) ws[4 + rows + r] = ~0ull;
      return;
    }
    cbeg = g.c_off[prob];
    kk = g.k[prob];
  }
  for (int t = threadIdx.x; t < d; t += blockDim.x) ax[t] = X[(size_t)row * ldx + t];
  if (threadIdx.x == 0) viol_sh = 0;
  __syncthreads();
  const float rel = 2.02f * (float)(d + 2) * 5.9604645e-8f;
  const float slack = (float)d * 2.3509887e-38f;  // d 2^-125
  const int lab = labels[row];
  const bool valid = lab >= cbeg && lab < cbeg + kk;
  // the label's interval (every warp evaluates it; an invalid label or one on an unusable
  // center is [inf, inf]: every usable center is nearer)
  float lab_lo = INFINITY, lab_hi = INFINITY;
  if (valid) {
    const float a = audit_dist32(ax, C + (size_t)lab * ldc, d, lane);
    if (a == a) {
      lab_lo = a * (1.0f - rel) - slack;
      lab_hi = a * (1.0f + rel) + slack;
    }
  }
  double dl = -1.0;  // the label's FP64 distance, evaluated when first needed
  const int per = (kk + parts - 1) / parts;
  const int j0 = cbeg + part * per, j1 = min(cbeg + kk, j0 + per);
  bool viol = false;
  for (int jb = j0 + 4 * warp; jb < j1; jb += 4 * nw) {  // four centers per warp step
    float a4[4];
    audit_dist32x4(ax, C, ldc, jb, j1, d, lane, a4);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = jb + u;
      if (j >= j1 || j == lab) continue;
      const float a = a4[u];
      if (!(a == a)) continue;  // an unusable (NaN) center
      const float lo = a * (1.0f - rel) - slack, hi = a * (1.0f + rel) + slack;
      if (hi < lab_lo) {
        viol = true;
      } else if (lo <= lab_hi && lane == 0) {  // overlapping intervals: decide in FP64
        if (dl < 0.0) {
          dl = valid ? exact_value(0, ax, C + (size_t)lab * ldc, d, 0.0f) : INFINITY;
          if (!(dl == dl)) dl = INFINITY;
        }
        if (exact_value(0, ax, C + (size_t)j * ldc, d, 0.0f) < dl) viol = true;
      }
    }
  }
  if (viol) viol_sh = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (viol_sh) atomicOr(ws + 4 + r, 1ull);
    if (part == 0) ws[4 + rows + r] = (unsigned long long)row;
  }
}

__global__ void audit_finish_kernel(unsigned long long* ws, int rows, const int* stop) {
  if (stopped(stop)) return;
  __shared__ int nviol, naud;
  __shared__ unsigned long long last;
  if (threadIdx.x == 0) {
    nviol = 0;
    naud = 0;
    last = 0;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    if (ws[4 + rows + r] != ~0ull) atomicAdd(&naud, 1);  // not a skipped row
    if (ws[4 + r]) {
      atomicAdd(&nviol, 1);
      atomicMax(&last, ws[4 + rows + r] + 1);
    }
    ws[4 + r] = 0;  // ready for the next audit
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ws[0] += (unsigned long long)naud;
    ws[1] += (unsigned long long)nviol;
    ws[2] += (unsigned long long)rows;
    if (last) ws[3] = last;
  }
}
}  // namespace

cudaError_t launch_gather_flagged(const int* list, const int* count, long long cap,
                                  const void* Xb, const void* Xl, long long row_bytes,
                                  const float* thr, void* XbC, void* XlC, float* thrC, int* over,
                                  int* over_count, const int* stop, cudaStream_t s,
                                  const float* xs, float* xsC) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (row_bytes % 16) return cudaErrorInvalidValue;
  gather_flagged_kernel<<<kmgb::num_sms() * 8, 256, 0, s>>>(
      list, count, cap, reinterpret_cast<const uint4*>(Xb), reinterpret_cast<const uint4*>(Xl),
      row_bytes / 16, thr, reinterpret_cast<uint4*>(XbC), reinterpret_cast<uint4*>(XlC), thrC, over,
      over_count, stop, xs, xsC);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_resolve_candidates(const int* list, const int* count, long long max_list,
                                      const int* cand, const int* cand_cnt, const float* X,
                                      long long ldx, const float* C, long long ldc, const float* cn,
                                      int d, int* labels, int* over, int* over_count,
                                      const int* stop, cudaStream_t s, const int* row_map) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  const bool vec = d % 4 == 0 && ldx % 4 == 0 && ldc % 4 == 0 &&
                   reinterpret_cast<uintptr_t>(X) % 16 == 0 && reinterpret_cast<uintptr_t>(C) % 16 == 0;
  if (vec)
    resolve_candidates_kernel<true><<<kmgb::num_sms() * 8, 256, 0, s>>>(list, count, max_list, cand, cand_cnt,
                                                            X, ldx, C, ldc, cn, d, labels, over,
                                                            over_count, stop, row_map);
  else
    resolve_candidates_kernel<false><<<kmgb::num_sms() * 8, 256, 0, s>>>(list, count, max_list, cand, cand_cnt,
                                                             X, ldx, C, ldc, cn, d, labels, over,
                                                             over_count, stop, row_map);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_count_stats(const int* counts, int full_idx, unsigned long long* stats,
                               const int* stop, cudaStream_t s) {
  count_stats_kernel<<<1, 1, 0, s>>>(counts, full_idx, stats, stop);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_rerank_exact(const RerankArgs& a, const float* hi2, cudaStream_t s) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (a.n <= 0 || a.k <= 0) return cudaSuccess;
  const int dq = (a.d + 3) / 4;
  const size_t smem = sizeof(float4) * (size_t)(TP + TC) * (dq + 1) + sizeof(float) * TC;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    KMGB_CUDA_TRY(cudaFuncSetAttribute(rerank_exact_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  rerank_exact_kernel<<<kmgb::num_sms() * 2, 256, smem, s>>>(a, hi2);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_rerank_tiled(const RerankArgs& a, int* list2, int* count2, float* hi2,
                                cudaStream_t s) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (a.n <= 0 || a.k <= 0) return cudaSuccess;
  const int dq = (a.d + 3) / 4;
  const size_t smem = sizeof(float4) * (size_t)(TP + TC) * (dq + 1) + sizeof(float) * TC;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    KMGB_CUDA_TRY(cudaFuncSetAttribute(rerank_tiled_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  rerank_tiled_kernel<<<kmgb::num_sms() * 2, 256, smem, s>>>(a, list2, count2, hi2);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_rerank_grouped(const RerankArgs& a, const GroupArgs& g, cudaStream_t s,
                                  int* cand, int* cand_cnt, long long cand_cap) {
  if (a.n <= 0 || a.k <= 0) return cudaSuccess;
  const size_t smem = sizeof(float) * (size_t)RG_WARPS * (RG_VCAP + (size_t)a.d);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    KMGB_CUDA_TRY(cudaFuncSetAttribute(rerank_grouped_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  rerank_grouped_kernel<<<kmgb::num_sms() * 4, RG_WARPS * 32, smem, s>>>(a, g, cand, cand_cnt,
                                                                          cand_cap);
  count_launches(1);
  return cudaGetLastError();
}

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
  rerank_kernel<<<kmgb::num_sms() * 4, threads, smem, s>>>(a); kmgb::count_launches(1);
  return cudaGetLastError();
}

int audit_parts(int rows) {
  const int p = 8 * kmgb::num_sms() / (rows > 0 ? rows : 1);
  return p < 1 ? 1 : (p > 32 ? 32 : p);
}

cudaError_t launch_audit_labels(const float* X, long long ldx, long long n, int d, const float* C,
                                long long ldc, int k, const int* labels, unsigned long long* ws,
                                int rows, const int* stop, cudaStream_t s, const GroupArgs* grp) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (n <= 0 || k <= 0 || rows <= 0) return cudaSuccess;
  if (rows > kAuditMaxRows || (size_t)d * sizeof(float) > 48 * 1024) return cudaErrorInvalidValue;
  const int parts = audit_parts(rows);
  const GroupArgs g = grp ? *grp : GroupArgs{};
  audit_scan_kernel<<<rows * parts, 256, sizeof(float) * (size_t)d, s>>>(X, ldx, n, d, C, ldc, k,
                                                                        labels, ws, rows, parts, g,
                                                                        stop);
  audit_finish_kernel<<<1, 256, 0, s>>>(ws, rows, stop);
  count_launches(2);
  return cudaGetLastError();
}

}  // namespace kmgb
