// Learned router: groups of centers, routed scan and certificate.
//
// The reference scans every center for every point (main/cuda/ClosestCenters.cu:46-83,
// kmeans.cpp:910-1014). With many centers that cluster in space (K = 65,536 centers drawn from
// Zipf-sized Gaussian clusters) most of that scan is wasted. Here:
//   1. Groups. On the first training the usable centers are linked into components: c and c'
//      are linked when d(c, c') <= min(max(t_c, t_c'), cap), t_c = 2.4 x the median distance of
//      c's members (from a sample of points), cap = 2.5 x the median of those medians over the
//      centers (a union-find over all center pairs, centers_pair_kernel). (With 3.6 x, chains
//      of centers lying between clusters merged half of the 65,536 centers of the Zipf-sized
//      16M x 256 workload into one component.) Components are
//      bin-packed, largest first into the lightest, into G groups; the groups stay fixed.
//   2. Network. An MLP (router_mlp.cu) learns, from a sample of (point, group of its label)
//      pairs, to predict the group; it is retrained every `retrain` iterations on the labels of
//      the iteration before. Inference on every point runs on the tensor cores: the pair kernel
//      of assign_bf16.cu in store mode (hidden layer, BF16 out with bias and ReLU) and in arg-max
//      mode (the group).
//   3. Routed scan. Points are sorted by their routed group (rows of a group padded to 256) and
//      the grouped pair kernel scans each point against its group's centers only (the centers
//      in group order, each group's slots padded to 256 with unusable centers), certifying the
//      arg-min within the group with the tier's rounding bound; near ties take the candidate
//      pass and the exact resolve as in the full scan. The in-group winner c* is then certified
//      as the arg-min over ALL centers when 2 d(x, c*) < m(c*), m(c*) a lower bound of the
//      distance from c* to every usable center outside its group: for such a center c,
//      d(x, c) >= d(c*, c) - d(x, c*) > 2 d(x, c*) - d(x, c*) = d(x, c*). m is computed for the
//      current centers every routed iteration: on the tensor cores by the pair kernel's
//      separation mode over the centers in group order (each row's largest key over the other
//      groups, plus the tier's rounding bound), or by centers_pair_kernel's min mode (FP32 SIMT,
//      with a rigorous bound of its FP32 rounding) where that mode cannot launch. (A bound
//      carried over from the last training and lowered by
//      the centers' movement since was tried first: one far-moving center in an early iteration
//      lowered every center's bound and left 16% of the points certified instead of most.)
//      Points that fail any step go to the full scan, so labels equal the FP64 arg-min.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/kmeans_gb300.h"
#include "common.cuh"
#include "kernels.h"
#include "router.h"

namespace kmgb {

namespace {

constexpr int kUnitRows = 256;      // rows of a pair-kernel unit / centers of a chunk
constexpr int kSample = 262144;     // training rows per epoch
constexpr int kBatch = 4096;        // training batch
constexpr int kChunkRows = 4 << 20; // inference rows per pass (hidden layer buffer)
constexpr int kPairTile = 128;      // centers per tile of the center-pair kernel
constexpr float kNoFloor = 3.3e38f; // candidate floor of rows that record nothing

__host__ __device__ __forceinline__ long long rup(long long v, long long m) {
  return (v + m - 1) / m * m;
}

// Arena carving (sizing pass with base == nullptr).
struct Carve {
  char* base = nullptr;
  size_t off = 0;
  template <typename T>
  void take(T** p, size_t count) {
    *p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += (sizeof(T) * (count ? count : 1) + 255) / 256 * 256;
  }
  void take_bytes(void** p, size_t bytes) {
    *p = base ? base + off : nullptr;
    off += ((bytes ? bytes : 1) + 255) / 256 * 256;
  }
};

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// ------------------------------- union-find (lock-free) -------------------------------
// Roots are the smallest index of their set (a larger root is hooked under a smaller one), so
// parent[v] <= v always and every walk ends.
__device__ __forceinline__ int uf_find(int* par, int v) {
  int cur = *reinterpret_cast<volatile int*>(par + v);
  if (cur != v) {
    int prev = v, next;
    while (cur > (next = *reinterpret_cast<volatile int*>(par + cur))) {
      par[prev] = next;  // path halving: a benign race, next is an ancestor of prev
      prev = cur;
      cur = next;
    }
  }
  return cur;
}

__device__ void uf_unite(int* par, int a, int b) {
  int ra = uf_find(par, a), rb = uf_find(par, b);
  while (ra != rb) {
    if (ra > rb) {
      const int t = ra;
      ra = rb;
      rb = t;
    }
    const int old = atomicCAS(par + rb, rb, ra);
    if (old == rb) return;
    rb = uf_find(par, old);  // rb was hooked meanwhile: continue from its new root
    ra = uf_find(par, ra);
  }
}

__global__ void uf_init_kernel(int* par, int k) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) par[i] = i;
}

__global__ void uf_flatten_kernel(int* par, int k) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x)
    par[i] = uf_find(par, i);
}

// ------------------------------- center-pair kernel -------------------------------
// Dot products of every pair of centers (upper triangle of 128 x 128 tiles, FP32 FMA, 8 x 8 per
// thread) with one of two epilogues:
//   kLink: unite(i, j) when d^2 = cn_i + cn_j - 2 c_i.c_j <= min(max(t_i, t_j), cap)^2;
//   kMinOut: for centers of different groups, the rigorous lower bound
//            d^2 >= fl(cn_i + cn_j - 2 fl(c_i.c_j)) - err_rel (cn_i + cn_j)
//            is min-reduced into m2[i] and m2[j] (atomicMin on the bits of non-negative floats).
// Only usable centers (cn < inf) take part.
enum { kLink = 0, kMinOut = 1 };

template <int MODE>
__global__ void __launch_bounds__(256)
centers_pair_kernel(const float* __restrict__ Cx, long long ldx, int k, int d,
                    const float* __restrict__ cn, const float* __restrict__ thr, float cap,
                    const int* __restrict__ group, int* __restrict__ par,
                    int* __restrict__ m2bits, float err_rel, int ntiles) {
  constexpr int TM = 8, T = 128, BKk = 16, PER = T * BKk / 256;
  __shared__ float As[BKk][T + 4];
  __shared__ float Bs[BKk][T + 4];
  __shared__ int tile_ij[2];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  if (tid == 0) {  // upper-triangle tile index -> (bi, bj), bi <= bj
    long long t = blockIdx.x;
    int bi = 0;
    while (t >= ntiles - bi) {
      t -= ntiles - bi;
      ++bi;
    }
    tile_ij[0] = bi;
    tile_ij[1] = bi + (int)t;
  }
  __syncthreads();
  const int bi = tile_ij[0], bj = tile_ij[1];
  const int i0 = bi * T, j0 = bj * T;
  float acc[TM][TM];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TM; ++b) acc[a][b] = 0.0f;
  for (int k0 = 0; k0 < d; k0 += BKk) {
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int e = tid + r * 256;
      const int mm = e / BKk, kk = e % BKk;
      const int gi = i0 + mm, gj = j0 + mm, gk = k0 + kk;
      As[kk][mm] = (gi < k && gk < d) ? Cx[(size_t)gi * ldx + gk] : 0.0f;
      Bs[kk][mm] = (gj < k && gk < d) ? Cx[(size_t)gj * ldx + gk] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BKk; ++kk) {
      float a[TM], b[TM];
#pragma unroll
      for (int q = 0; q < TM; ++q) a[q] = As[kk][ty + 16 * q];
#pragma unroll
      for (int q = 0; q < TM; ++q) b[q] = Bs[kk][tx + 16 * q];
#pragma unroll
      for (int q = 0; q < TM; ++q)
#pragma unroll
        for (int w = 0; w < TM; ++w) acc[q][w] = fmaf(a[q], b[w], acc[q][w]);
    }
    __syncthreads();
  }
  float rowmin[TM], colmin[TM];
#pragma unroll
  for (int q = 0; q < TM; ++q) rowmin[q] = colmin[q] = INFINITY;
#pragma unroll
  for (int q = 0; q < TM; ++q) {
    const int gi = i0 + ty + 16 * q;
    if (gi >= k) continue;
    const float ni = cn[gi];
    if (!(ni < INFINITY)) continue;
#pragma unroll
    for (int w = 0; w < TM; ++w) {
      const int gj = j0 + tx + 16 * w;
      if (gj >= k || (bi == bj && gj <= gi)) continue;
      const float nj = cn[gj];
      if (!(nj < INFINITY)) continue;
      const float d2 = fmaf(-2.0f, acc[q][w], ni + nj);
      if (MODE == kLink) {
        const float t = fminf(fmaxf(thr[gi], thr[gj]), cap);
        if (d2 <= t * t) uf_unite(par, gi, gj);
      } else {
        const int g1 = group[gi], g2 = group[gj];
        if (g1 == g2 && g1 >= 0) continue;
        const float lb = fmaxf(d2 - err_rel * (ni + nj), 0.0f);
        rowmin[q] = fminf(rowmin[q], lb);
        colmin[w] = fminf(colmin[w], lb);
      }
    }
  }
  if (MODE == kMinOut) {
#pragma unroll
    for (int q = 0; q < TM; ++q) {
      float v = rowmin[q];
#pragma unroll
      for (int o = 1; o < 16; o <<= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
      const int gi = i0 + ty + 16 * q;
      if (tx == 0 && gi < k && v < INFINITY) atomicMin(m2bits + gi, __float_as_int(v));
    }
#pragma unroll
    for (int w = 0; w < TM; ++w) {
      const int gj = j0 + tx + 16 * w;
      if (gj < k && colmin[w] < INFINITY) atomicMin(m2bits + gj, __float_as_int(colmin[w]));
    }
  }
}

__global__ void fill_int_kernel(int* p, long long n, int v) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

// m0[c] = sqrt(m2[c]) rounded down (+inf when no center lies outside the group).
__global__ void m0_kernel(const int* m2bits, int k, double* m0) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) {
    const float v = __int_as_float(m2bits[i]);
    m0[i] = v < INFINITY ? sqrt((double)v) * (1.0 - 0x1p-50) : INFINITY;
  }
}

// Separation from the tensor-core pass: for slot j (center c = cperm[j]) every center c' of
// another group has d^2(c, c') = ||c||^2 - 2 key(c, c') >= cn (1 - 2^-23) - 2 xmax[j] (xmax an
// upper bound of the exact keys, cn ||c||^2 rounded to nearest), evaluated with downward
// rounding; min-reduced like the SIMT kernel's output (non-negative float bits).
__global__ void m2_from_xmax_kernel(const int* __restrict__ cperm, long long KP,
                                    const float* __restrict__ cnP, const float* __restrict__ xmax,
                                    int* __restrict__ m2bits, const int* stop) {
  if (stopped(stop)) return;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < KP;
       j += (long long)gridDim.x * blockDim.x) {
    const int c = cperm[j];
    if (c < 0 || !(cnP[j] < INFINITY)) continue;
    const float xm = xmax[j];
    float v = INFINITY;  // no usable center in another group
    if (xm > -INFINITY) {
      const double lb = __dsub_rd(__dmul_rd((double)cnP[j], 1.0 - 0x1p-23), 2.0 * (double)xm);
      v = lb > 0.0 ? __double2float_rd(lb) : 0.0f;
    }
    m2bits[c] = __float_as_int(v);
  }
}

// Centers in group order: slot j holds center cperm[j] (or padding: zero rows, unusable).
__global__ void permute_centers_kernel(const int* __restrict__ cperm, long long KP,
                                       const uint4* __restrict__ Cb, const uint4* __restrict__ Cl,
                                       long long vb, const float4* __restrict__ Cop,
                                       long long vx, const float* __restrict__ cinit,
                                       const float* __restrict__ cn, uint4* __restrict__ CbP,
                                       uint4* __restrict__ ClP, float4* __restrict__ CopP,
                                       float* __restrict__ cinitP, float* __restrict__ cnP,
                                       const uint4* __restrict__ cbias, uint4* __restrict__ cbiasP,
                                       float* __restrict__ xnP, const int* stop) {
  if (stopped(stop)) return;
  const int lane = threadIdx.x & 31;
  // the start-value row of a padding slot: -3e38 as three BF16 pieces, then zeros
  uint4 pad_bias = make_uint4(0, 0, 0, 0);
  if (cbias) {
    const __nv_bfloat16 hi = __float2bfloat16_rn(-3.0e38f);
    const float r1 = -3.0e38f - __bfloat162float(hi);
    const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
    const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
    pad_bias.x = (uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(mid) << 16);
    pad_bias.y = (uint32_t)__bfloat16_as_ushort(lo);
  }
  for (long long j = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < KP;
       j += ((long long)gridDim.x * blockDim.x) >> 5) {
    const int c = cperm[j];
    for (long long t = lane; t < vb; t += 32) {
      CbP[j * vb + t] = c >= 0 ? Cb[(size_t)c * vb + t] : make_uint4(0, 0, 0, 0);
      if (ClP) ClP[j * vb + t] = c >= 0 ? Cl[(size_t)c * vb + t] : make_uint4(0, 0, 0, 0);
    }
    for (long long t = lane; t < vx; t += 32)
      CopP[j * vx + t] = c >= 0 ? Cop[(size_t)c * vx + t] : make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane == 0) {
      cinitP[j] = c >= 0 ? cinit[c] : -3.0e38f;
      cnP[j] = c >= 0 ? cn[c] : INFINITY;
      // ||c|| <= sqrt(cn (1 + 2^-24)): cn is ||c||^2 rounded to nearest
      if (xnP) xnP[j] = (c >= 0 && cn[c] < INFINITY) ? __fsqrt_ru(cn[c]) * 1.000001f : 0.0f;
    }
    if (cbias && lane < kBiasCols * 2 / 16)  // 32-byte rows: two uint4 per slot
      cbiasP[j * 2 + lane] = c >= 0 ? cbias[(size_t)c * 2 + lane] : (lane ? make_uint4(0, 0, 0, 0) : pad_bias);
  }
}

// Per-group counts of the routed points (shared-memory histogram, one global add per group and
// block); points routed to an empty group go to the full scan.
__global__ void route_count_kernel(const int* __restrict__ route, long long n, int G,
                                   const int* __restrict__ gk, int* __restrict__ gcnt,
                                   int* __restrict__ fb_list, int* __restrict__ fb_count,
                                   const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ int hist[];
  for (int g = threadIdx.x; g < G; g += blockDim.x) hist[g] = 0;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int g = route[i];
    if (g >= 0 && g < G && gk[g] > 0) atomicAdd(hist + g, 1);
    else fb_list[atomicAdd(fb_count, 1)] = (int)i;
  }
  __syncthreads();
  for (int g = threadIdx.x; g < G; g += blockDim.x)
    if (hist[g]) atomicAdd(gcnt + g, hist[g]);
}

// One block: group row offsets (each group's rows padded to 256), the unit table of the pair
// kernel (unit u -> group, or G for units past the last group), and the routed-point counter.
__global__ void route_tables_kernel(const int* __restrict__ gcnt, const int* __restrict__ gk,
                                    int G, long long max_units,
                                    long long* __restrict__ row_off, long long* __restrict__ rend,
                                    int* __restrict__ gdone, int* __restrict__ fill,
                                    int* __restrict__ uprob, unsigned long long* rows_stat,
                                    unsigned long long* chunks_stat, const int* stop) {
  if (stopped(stop)) return;
  __shared__ long long off[1025];
  if (threadIdx.x == 0) {
    long long o = 0, routed = 0, chunks = 0;
    for (int g = 0; g < G; ++g) {
      off[g] = o;
      o += rup(gcnt[g], kUnitRows);
      routed += gcnt[g];
      chunks += (long long)gcnt[g] * ((gk[g] + kUnitRows - 1) / kUnitRows);
    }
    off[G] = o;
    *rows_stat += (unsigned long long)routed;
    *chunks_stat += (unsigned long long)chunks;
  }
  __syncthreads();
  for (int g = threadIdx.x; g <= G; g += blockDim.x) {
    row_off[g] = off[g];
    if (g < G) {
      rend[g] = off[g] + gcnt[g];
      gdone[g] = gcnt[g] == 0;
      fill[g] = 0;
    } else {
      rend[g] = off[g];
      gdone[g] = 1;
    }
  }
  for (long long u = threadIdx.x; u < max_units; u += blockDim.x) {
    const long long r = u * kUnitRows;
    int lo = 0, hi = G;  // last g with off[g] <= r
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= r) lo = mid;
      else hi = mid - 1;
    }
    uprob[u] = (lo < G && r < off[lo + 1]) ? lo : G;
  }
}

// Routed rows: every point of a non-empty group gets a row of its group (block-level
// reservation, then shared-memory atomics), its BF16 row(s) and norm bound are copied there.
constexpr int kScatterPts = 2048;
__global__ void __launch_bounds__(256)
route_scatter_kernel(const int* __restrict__ route, long long n, int G, const int* __restrict__ gk,
                     const long long* __restrict__ row_off, int* __restrict__ fill,
                     const uint4* __restrict__ Xb, const uint4* __restrict__ Xl, long long vb,
                     const float* __restrict__ xn, int* __restrict__ rowmap,
                     uint4* __restrict__ XbR, uint4* __restrict__ XlR, float* __restrict__ xnR,
                     const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ int sm[];
  int* cnt = sm;              // [G]
  int* base = sm + G;         // [G]
  int* slot = sm + 2 * G;     // [kScatterPts]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long p0 = (long long)blockIdx.x * kScatterPts; p0 < n;
       p0 += (long long)gridDim.x * kScatterPts) {
    for (int g = threadIdx.x; g < G; g += blockDim.x) cnt[g] = 0;
    __syncthreads();
    for (int q = threadIdx.x; q < kScatterPts; q += blockDim.x) {
      const long long i = p0 + q;
      int s = -1;
      if (i < n) {
        const int g = route[i];
        if (g >= 0 && g < G && gk[g] > 0) s = atomicAdd(cnt + g, 1);
      }
      slot[q] = s;
    }
    __syncthreads();
    for (int g = threadIdx.x; g < G; g += blockDim.x)
      base[g] = cnt[g] ? atomicAdd(fill + g, cnt[g]) : 0;
    __syncthreads();
    for (int q = warp; q < kScatterPts; q += blockDim.x / 32) {
      if (slot[q] < 0) continue;  // uniform over the warp
      const long long i = p0 + q;
      const int g = route[i];
      const long long r = row_off[g] + base[g] + slot[q];
      for (long long t = lane; t < vb; t += 32) {
        XbR[r * vb + t] = Xb[(size_t)i * vb + t];
        if (XlR) XlR[r * vb + t] = Xl[(size_t)i * vb + t];
      }
      if (lane == 0) {
        rowmap[r] = (int)i;
        xnR[r] = xn[i];
      }
    }
    __syncthreads();
  }
}

// Near ties of the group scan, compacted: the flagged routed rows counted per group
// (shared-memory histogram), ...
__global__ void flag_count_kernel(const int* __restrict__ flag, const int* __restrict__ count,
                                  long long cap, const int* __restrict__ uprob, int G,
                                  int* __restrict__ gcnt, const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ int hist[];
  for (int g = threadIdx.x; g < G; g += blockDim.x) hist[g] = 0;
  __syncthreads();
  const long long c = min((long long)*count, cap);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < c;
       i += (long long)gridDim.x * blockDim.x)
    atomicAdd(hist + uprob[flag[i] / kUnitRows], 1);
  __syncthreads();
  for (int g = threadIdx.x; g < G; g += blockDim.x)
    if (hist[g]) atomicAdd(gcnt + g, hist[g]);
}

// ... then copied, one warp per flagged row, into rows of their group in a second layout (row
// q of group g in [row_off2[g], rend2[g]); one atomic per group and warp reserves the rows), with
// their floors, routed rows and data rows; list2[i] = the compact row of flagged entry i.
__global__ void flag_scatter_kernel(const int* __restrict__ flag, const int* __restrict__ count,
                                    long long cap, const int* __restrict__ uprob,
                                    const long long* __restrict__ row_off2, int* __restrict__ fill2,
                                    const uint4* __restrict__ XbR, const uint4* __restrict__ XlR,
                                    long long vb, const float* __restrict__ thrR,
                                    const int* __restrict__ rowmap, uint4* __restrict__ Xb2,
                                    uint4* __restrict__ Xl2, float* __restrict__ thr2,
                                    int* __restrict__ xrow2, int* __restrict__ rmap2,
                                    int* __restrict__ list2, const int* stop) {
  if (stopped(stop)) return;
  const long long c = min((long long)*count, cap);
  const int lane = threadIdx.x & 31;
  for (long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x) & ~31LL; base < c;
       base += (long long)gridDim.x * blockDim.x) {
    const long long i = base + lane;
    const bool live = i < c;
    const int r = live ? flag[i] : 0;
    const int g = live ? uprob[r / kUnitRows] : -1;
    // lanes of the same group reserve their rows with one atomic (the lowest lane)
    const unsigned peers = __match_any_sync(0xffffffffu, g);
    const int leader = __ffs(peers) - 1;
    const int rank = __popc(peers & lanemask_lt());
    int q0 = 0;
    if (live && lane == leader) q0 = atomicAdd(fill2 + g, __popc(peers));
    q0 = __shfl_sync(0xffffffffu, q0, leader);
    const long long q = live ? row_off2[g] + q0 + rank : -1;
    if (live) {
      thr2[q] = thrR[r];
      xrow2[q] = rowmap[r];
      rmap2[q] = r;
      list2[i] = (int)q;
    }
    // the rows, one warp per row
    for (int t = 0; t < 32; ++t) {
      const long long qt = __shfl_sync(0xffffffffu, q, t);
      const int rt = __shfl_sync(0xffffffffu, r, t);
      if (qt < 0) continue;
      for (long long v = lane; v < vb; v += 32) {
        Xb2[qt * vb + v] = XbR[(size_t)rt * vb + v];
        if (Xl2) Xl2[qt * vb + v] = XlR[(size_t)rt * vb + v];
      }
    }
  }
}

// The compact rows' labels back to their routed rows.
__global__ void flag_copy_back_kernel(const int* __restrict__ list2, const int* __restrict__ count,
                                      long long cap, const int* __restrict__ rmap2,
                                      const int* __restrict__ lab2, int* __restrict__ labR,
                                      const int* stop) {
  if (stopped(stop)) return;
  const long long c = min((long long)*count, cap);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < c;
       i += (long long)gridDim.x * blockDim.x) {
    const int q = list2[i];
    labR[rmap2[q]] = lab2[q];
  }
}

__global__ void mark_over_kernel(const int* __restrict__ over, const int* __restrict__ count,
                                 long long cap, int* __restrict__ labR, const int* stop) {
  if (stopped(stop)) return;
  const long long c = min((long long)*count, cap);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < c;
       i += (long long)gridDim.x * blockDim.x)
    labR[over[i]] = -1;
}

// Certificate of the routed points: one warp per routed row. The FP32 direct-form distance to
// the in-group winner (non-negative terms: within (m + 8) 2^-24 relative, m = ceil(d/32) terms
// per lane, plus subnormal slack) gives an upper bound of d(x, c*); the point is certified when
// twice that is below the lower bound m0(c*) of c*'s distance to every center outside its
// group.
__global__ void router_finish_kernel(long long rows_cap, int G, const int* __restrict__ uprob,
                                     const long long* __restrict__ rend,
                                     const int* __restrict__ rowmap, const int* __restrict__ labR,
                                     long long KP, const int* __restrict__ cperm,
                                     const float* __restrict__ cnP, const float* __restrict__ X,
                                     long long ldx, const float* __restrict__ C, int d,
                                     const double* __restrict__ m0, int* __restrict__ labels,
                                     int* __restrict__ fb_list, int* __restrict__ fb_count,
                                     unsigned long long* stats, const int* stop) {
  if (stopped(stop)) return;
  const int lane = threadIdx.x & 31;
  const double m = (double)((d + 31) / 32);
  const double rel = 1.1 * (m + 8.0) * 0x1p-24;
  const double abs_tol = (double)(d + 32) * (m + 8.0) * 0x1p-149;
  unsigned long long cert = 0;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows_cap;
       r += ((long long)gridDim.x * blockDim.x) >> 5) {
    const int g = uprob[r / kUnitRows];
    if (g >= G || r >= rend[g]) continue;  // padding row (uniform over the warp)
    const int i = rowmap[r];
    const int j = labR[r];
    const int c = (j >= 0 && j < KP && cnP[j] < INFINITY) ? cperm[j] : -1;
    bool ok = c >= 0;
    if (ok) {
      const float* x = X + (size_t)i * ldx;
      const float* cc = C + (size_t)c * ldx;
      float s = 0.0f;
      for (int t = lane; t < d; t += 32) {
        const float u = x[t] - cc[t];
        s = fmaf(u, u, s);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
      const double dub = sqrt((double)s * (1.0 + rel) + abs_tol) * (1.0 + 0x1p-50);
      ok = 2.0 * dub < m0[c];
    }
    if (lane == 0) {
      if (ok) {
        labels[i] = c;
        ++cert;
      } else {
        fb_list[atomicAdd(fb_count, 1)] = i;
      }
    }
  }
  if (lane == 0 && cert) atomicAdd(stats + 2, cert);
}

__global__ void add_count_kernel(const int* __restrict__ count, unsigned long long* dst,
                                 const int* stop) {
  if (stopped(stop)) return;
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst += (unsigned long long)*count;
}

// Training sample: rows drawn by a seeded hash, scaled into Xs, with the group of their label.
__global__ void sample_kernel(const float* __restrict__ X, long long ldx, long long n, int d,
                              const int* __restrict__ labels, int k,
                              const int* __restrict__ group, unsigned long long seed, int S,
                              float scale, float* __restrict__ Xs, int* __restrict__ ys) {
  const int lane = threadIdx.x & 31;
  for (long long s = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < S;
       s += ((long long)gridDim.x * blockDim.x) >> 5) {
    const long long row = (long long)(splitmix64(seed * 0x100000001B3ull + (unsigned long long)s) %
                                      (unsigned long long)n);
    for (int t = lane; t < d; t += 32) Xs[(size_t)s * d + t] = X[(size_t)row * ldx + t] * scale;
    if (lane == 0) {
      const int l = labels[row];
      const int g = (l >= 0 && l < k) ? group[l] : -1;
      ys[s] = g >= 0 ? g : 0;
    }
  }
}

// Labels and member distances of a sample of points (grouping radius; norm scale).
__global__ void radius_sample_kernel(const float* __restrict__ X, long long ldx, long long n,
                                     int d, const int* __restrict__ labels,
                                     const float* __restrict__ C, int k,
                                     const float* __restrict__ xn, unsigned long long seed, int S,
                                     int* __restrict__ lab_out, float* __restrict__ dist_out,
                                     float* __restrict__ xn_out) {
  const int lane = threadIdx.x & 31;
  for (long long s = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < S;
       s += ((long long)gridDim.x * blockDim.x) >> 5) {
    const long long row = (long long)(splitmix64(seed * 0x100000001B3ull + (unsigned long long)s) %
                                      (unsigned long long)n);
    const int l = labels[row];
    float acc = 0.0f;
    if (l >= 0 && l < k)
      for (int t = lane; t < d; t += 32) {
        const float u = X[(size_t)row * ldx + t] - C[(size_t)l * ldx + t];
        acc = fmaf(u, u, acc);
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      lab_out[s] = l;
      dist_out[s] = sqrtf(acc);
      xn_out[s] = xn[row];
    }
  }
}

// Tensor-core copies of the network: W1 scaled by the input scale, rows padded to ldb.
__global__ void export_kernel(const float* __restrict__ P, int d, int hidden, int G, long long ldb,
                              float scale, __nv_bfloat16* __restrict__ W1b,
                              float* __restrict__ cin1, __nv_bfloat16* __restrict__ W2b,
                              float* __restrict__ cin2, int G_pad) {
  const float* W1 = P;
  const float* b1 = W1 + (size_t)hidden * d;
  const float* W2 = b1 + hidden;
  const float* b2 = W2 + (size_t)G * hidden;
  const long long n1 = (long long)hidden * ldb, n2 = (long long)G * hidden;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n1 + n2 + hidden + G_pad;
       i += (long long)gridDim.x * blockDim.x) {
    if (i < n1) {
      const long long h = i / ldb, j = i % ldb;
      W1b[i] = __float2bfloat16_rn(j < d ? W1[h * d + j] * scale : 0.0f);
    } else if (i < n1 + n2) {
      W2b[i - n1] = __float2bfloat16_rn(W2[i - n1]);
    } else if (i < n1 + n2 + hidden) {
      cin1[i - n1 - n2] = b1[i - n1 - n2];
    } else {
      const long long g = i - n1 - n2 - hidden;
      cin2[g] = g < G ? b2[g] : -3.0e38f;
    }
  }
}

// Points sent to the full scan, as a compact data set: row r of the compact buffers is point
// fb_list[r] (FP32 row, norm bound, BF16 planes). One warp per row.
__global__ void gather_fallback_kernel(const int* __restrict__ fb_list, const int* __restrict__ fb_count,
                                       long long cap, const float4* __restrict__ X, long long vx,
                                       const float* __restrict__ xn, const uint4* __restrict__ Xb,
                                       const uint4* __restrict__ Xl, long long vb,
                                       float4* __restrict__ XF, float* __restrict__ xnF,
                                       uint4* __restrict__ XbF, uint4* __restrict__ XlF,
                                       const int* stop) {
  if (stopped(stop)) return;
  const long long cnt = min((long long)*fb_count, cap);
  const int lane = threadIdx.x & 31;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < cnt;
       r += ((long long)gridDim.x * blockDim.x) >> 5) {
    const long long i = fb_list[r];
    for (long long t = lane; t < vx; t += 32) XF[r * vx + t] = X[i * vx + t];
    for (long long t = lane; t < vb; t += 32) {
      XbF[r * vb + t] = Xb[i * vb + t];
      if (XlF) XlF[r * vb + t] = Xl[i * vb + t];
    }
    if (lane == 0) xnF[r] = xn[i];
  }
}

__global__ void scatter_fallback_kernel(const int* __restrict__ fb_list,
                                        const int* __restrict__ fb_count, long long cap,
                                        const int* __restrict__ labF, int* __restrict__ labels,
                                        const int* stop) {
  if (stopped(stop)) return;
  const long long cnt = min((long long)*fb_count, cap);
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < cnt;
       r += (long long)gridDim.x * blockDim.x)
    labels[fb_list[r]] = labF[r];
}

// Linking cap as a multiple of the median member distance (KMGB_ROUTER_CAP overrides it).
float cap_factor() {
  const char* v = std::getenv("KMGB_ROUTER_CAP");
  const float f = v ? (float)std::atof(v) : 0.0f;
  return f > 0.0f ? f : 2.5f;
}

cudaError_t sync_err(cudaStream_t s) {
  cudaError_t e = cudaStreamSynchronize(s);
  return e != cudaSuccess ? e : cudaGetLastError();
}

}  // namespace

struct Router {
  long long n = 0;
  int d = 0, k = 0, G = 0, hidden = 0;
  long long ldx = 0, ldb = 0;
  bool split = false;
  long long KPmax = 0, KP = 0, rows_cap = 0, max_units = 0;
  int S = 0, Sg = 0;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  bool grouped = false, trained = false;
  std::vector<int> group_h;
  std::vector<int> slot_group_h;  // host copy kept alive for the asynchronous upload
  // groups and certificate
  int *group = nullptr, *cperm = nullptr, *gcoff = nullptr, *gk = nullptr, *par = nullptr;
  float* thr = nullptr;
  int* m2 = nullptr;
  double* m0 = nullptr;
  // permuted centers
  void *CbP = nullptr, *ClP = nullptr, *cbiasP = nullptr;
  float *CopP = nullptr, *cinitP = nullptr, *cnP = nullptr;
  // separation on the tensor cores: the group of every slot, ||c|| bounds of the slots, and
  // the bound of every slot's largest key over the other groups
  int* slot_group = nullptr;
  float *xnP = nullptr, *xmaxP = nullptr;
  // routing
  int *route = nullptr, *rowmap = nullptr, *labR = nullptr, *flagR = nullptr;
  int *candR = nullptr, *ccntR = nullptr, *uprob = nullptr, *gcnt = nullptr, *fill = nullptr;
  int *gdone = nullptr, *rcount = nullptr;
  long long *row_off = nullptr, *rend = nullptr;
  void *XbR = nullptr, *XlR = nullptr;
  float *xnR = nullptr, *thrR = nullptr;
  // the routed rows with near ties, compacted by group for the candidate pass
  void *Xb2 = nullptr, *Xl2 = nullptr;
  float* thr2 = nullptr;
  int *xrow2 = nullptr, *rmap2 = nullptr, *list2 = nullptr, *lab2 = nullptr, *over2 = nullptr;
  int *uprob2 = nullptr, *gcnt2 = nullptr, *fill2 = nullptr, *gdone2 = nullptr;
  long long *row_off2 = nullptr, *rend2 = nullptr;
  unsigned long long* dstats = nullptr;
  // network
  MlpShape sh{};
  long long np = 0;
  float *P = nullptr, *Gr = nullptr, *Am = nullptr, *Av = nullptr;
  float *Xs = nullptr, *Hd = nullptr, *Z = nullptr, *dZ = nullptr, *dH = nullptr,
        *lrows = nullptr, *gpart = nullptr;
  int* ys = nullptr;
  int* slab = nullptr;
  float *sdist = nullptr, *sxn = nullptr;
  float scale = 1.0f;
  long long adam_t = 0;
  // tensor-core copies
  void *W1b = nullptr, *W2b = nullptr, *Hbuf = nullptr;
  float *cin1 = nullptr, *cin2 = nullptr;
  int G_pad = 0;
  RouterStats st;
  // stage events (profiling): 8 per routed iteration, read out by router_stats
  bool prof = false;
  std::vector<cudaEvent_t> ev;
  size_t ev_used = 0, ev_read = 0;
  cudaError_t mark(cudaStream_t s) {
    if (!prof) return cudaSuccess;
    if (ev_used == ev.size()) {
      cudaEvent_t e;
      cudaError_t r = cudaEventCreate(&e);
      if (r != cudaSuccess) return r;
      ev.push_back(e);
    }
    return cudaEventRecord(ev[ev_used++], s);
  }

  void carve(Carve& c) {
    c.take(&group, k);
    c.take(&cperm, KPmax);
    c.take(&gcoff, G + 1);
    c.take(&gk, G + 1);
    c.take(&par, k);
    c.take(&thr, k);
    c.take(&m2, k);
    c.take(&m0, k);
    c.take_bytes(&CbP, (size_t)KPmax * ldb * 2);
    if (split) c.take_bytes(&ClP, (size_t)KPmax * ldb * 2);
    c.take(&CopP, (size_t)KPmax * ldx);
    c.take(&cinitP, KPmax);
    c.take_bytes(&cbiasP, (size_t)KPmax * kBiasCols * 2);
    c.take(&slot_group, KPmax);
    c.take(&xnP, KPmax);
    c.take(&xmaxP, KPmax);
    c.take(&cnP, KPmax);
    c.take(&route, n);
    c.take(&rowmap, rows_cap);
    c.take(&labR, rows_cap);
    c.take(&flagR, rows_cap);
    c.take(&candR, (size_t)rows_cap * kMaxCand);
    c.take(&ccntR, rows_cap);
    c.take(&uprob, max_units);
    c.take(&gcnt, G + 1);
    c.take(&fill, G + 1);
    c.take(&gdone, G + 1);
    c.take(&rcount, 4);
    c.take(&row_off, G + 1);
    c.take(&rend, G + 1);
    c.take_bytes(&XbR, (size_t)rows_cap * ldb * 2);
    c.take(&xnR, rows_cap);
    c.take(&thrR, rows_cap);
    c.take(&dstats, 8);
    c.take_bytes(&Xb2, (size_t)rows_cap * ldb * 2);
    c.take(&thr2, rows_cap);
    c.take(&xrow2, rows_cap);
    c.take(&rmap2, rows_cap);
    c.take(&list2, rows_cap);
    c.take(&lab2, rows_cap);
    c.take(&over2, rows_cap);
    c.take(&uprob2, max_units);
    c.take(&gcnt2, G + 1);
    c.take(&fill2, G + 1);
    c.take(&gdone2, G + 1);
    c.take(&row_off2, G + 1);
    c.take(&rend2, G + 1);
    c.take(&P, np);
    c.take(&Gr, np);
    c.take(&Am, np);
    c.take(&Av, np);
    c.take(&Xs, (size_t)S * d);
    c.take(&ys, S);
    c.take(&Hd, (size_t)kBatch * hidden);
    c.take(&Z, (size_t)kBatch * G);
    c.take(&dZ, (size_t)kBatch * G);
    c.take(&dH, (size_t)kBatch * hidden);
    c.take(&lrows, kBatch);
    c.take(&gpart, mlp_split_scratch(sh));
    c.take(&slab, Sg);
    c.take(&sdist, Sg);
    c.take(&sxn, Sg);
    c.take_bytes(&W1b, (size_t)hidden * ldb * 2);
    c.take_bytes(&W2b, (size_t)G * hidden * 2);
    c.take(&cin1, rup(hidden, kUnitRows));
    c.take(&cin2, G_pad);
    c.take_bytes(&Hbuf, (size_t)std::min<long long>(n, kChunkRows) * hidden * 2);
  }
};

cudaError_t router_create(Router** out, const RouterIO& io, int groups, int hidden, bool split,
                          cudaStream_t s) {
  *out = nullptr;
  if (groups < 2 || groups > 1024 || hidden < 32 || hidden % kUnitRows != 0 || hidden > 512)
    return cudaErrorInvalidValue;
  Router* r = new Router();
  r->n = io.n;
  r->d = io.d;
  r->k = io.k;
  r->G = groups;
  r->hidden = hidden;
  r->ldx = io.ldx;
  r->ldb = io.ldb;
  r->split = split;
  r->KPmax = rup(io.k, kUnitRows) + (long long)kUnitRows * groups;
  r->rows_cap = rup(io.n, kUnitRows) + (long long)kUnitRows * groups;
  r->max_units = r->rows_cap / kUnitRows;
  r->S = (int)std::min<long long>(io.n, kSample);
  r->Sg = (int)std::min<long long>(io.n, std::max<long long>(kSample, 8LL * io.k));
  r->sh = MlpShape{io.d, hidden, groups};
  r->np = mlp_param_count(r->sh);
  r->G_pad = (int)rup(groups, kUnitRows);
  r->group_h.assign(io.k, -1);
  Carve sizing;
  r->carve(sizing);
  r->arena_bytes = sizing.off;
  cudaError_t e = dev_alloc(&r->arena, sizing.off, s);
  if (e != cudaSuccess) {
    delete r;
    return e;
  }
  Carve cut;
  cut.base = static_cast<char*>(r->arena);
  r->carve(cut);
  e = cudaMemsetAsync(r->dstats, 0, 8 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) {
    router_destroy(r, s);
    return e;
  }
  *out = r;
  return cudaSuccess;
}

void router_destroy(Router* r, cudaStream_t s) {
  if (!r) return;
  for (cudaEvent_t e : r->ev) cudaEventDestroy(e);
  if (r->XlR) dev_free(r->XlR, s);
  if (r->Xl2) dev_free(r->Xl2, s);
  dev_free(r->arena, s);
  delete r;
}

bool router_trained(const Router* r) { return r && r->trained; }
void router_set_profiling(Router* r, bool on) {
  if (r) r->prof = on;
}
size_t router_device_bytes(const Router* r) { return r ? r->arena_bytes : 0; }

// Components of the usable centers and their packing into groups (first training only).
static cudaError_t form_groups(Router* r, const RouterIO& io, cudaStream_t s) {
  const int k = r->k, G = r->G;
  // member distances of a sample of points: per-center median -> linking radius
  radius_sample_kernel<<<num_sms() * 8, 256, 0, s>>>(io.X, io.ldx, io.n, io.d, io.labels, io.C,
                                                      k, io.xn, 0x5eedULL, r->Sg, r->slab,
                                                      r->sdist, r->sxn);
  count_launches(1);
  std::vector<int> lab(r->Sg);
  std::vector<float> dist(r->Sg), cn(k);
  KMGB_CUDA_TRY(cudaMemcpyAsync(lab.data(), r->slab, sizeof(int) * r->Sg, cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(dist.data(), r->sdist, sizeof(float) * r->Sg, cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(cn.data(), io.cn, sizeof(float) * k, cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(sync_err(s));
  std::vector<std::vector<float>> mem(k);
  for (int i = 0; i < r->Sg; ++i)
    if (lab[i] >= 0 && lab[i] < k && std::isfinite(dist[i])) mem[lab[i]].push_back(dist[i]);
  std::vector<float> thr(k, 0.0f), meds;
  for (int c = 0; c < k; ++c) {
    if (mem[c].empty()) continue;
    auto mid = mem[c].begin() + mem[c].size() / 2;
    std::nth_element(mem[c].begin(), mid, mem[c].end());
    thr[c] = 2.4f * *mid;
    meds.push_back(*mid);
  }
  float cap = 0.0f;
  if (!meds.empty()) {
    auto mid = meds.begin() + meds.size() / 2;
    std::nth_element(meds.begin(), mid, meds.end());
    cap = cap_factor() * *mid;
  }
  KMGB_CUDA_TRY(cudaMemcpyAsync(r->thr, thr.data(), sizeof(float) * k, cudaMemcpyHostToDevice, s));
  uf_init_kernel<<<num_sms() * 4, 256, 0, s>>>(r->par, k);
  const int nt = (k + kPairTile - 1) / kPairTile;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  centers_pair_kernel<kLink><<<(unsigned)tiles, 256, 0, s>>>(io.Cop, io.ldx, k, io.d, io.cn,
                                                             r->thr, cap, nullptr, r->par,
                                                             nullptr, 0.0f, nt);
  uf_flatten_kernel<<<num_sms() * 4, 256, 0, s>>>(r->par, k);
  count_launches(3);
  std::vector<int> comp(k);
  KMGB_CUDA_TRY(cudaMemcpyAsync(comp.data(), r->par, sizeof(int) * k, cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(sync_err(s));
  // components of usable centers, largest first into the lightest group (ties: lowest group)
  std::vector<int> size(k, 0);
  for (int c = 0; c < k; ++c)
    if (cn[c] < INFINITY) ++size[comp[c]];
  std::vector<int> roots;
  for (int c = 0; c < k; ++c)
    if (size[c] > 0) roots.push_back(c);
  std::stable_sort(roots.begin(), roots.end(), [&](int a, int b) { return size[a] > size[b]; });
  std::vector<long long> load(G, 0);
  std::vector<int> gof(k, -1);
  for (int root : roots) {
    int best = 0;
    for (int g = 1; g < G; ++g)
      if (load[g] < load[best]) best = g;
    gof[root] = best;
    load[best] += size[root];
  }
  std::vector<int> gkh(G + 1, 0), gcoff(G + 1, 0);
  for (int c = 0; c < k; ++c) {
    r->group_h[c] = cn[c] < INFINITY ? gof[comp[c]] : -1;
    if (r->group_h[c] >= 0) ++gkh[r->group_h[c]];
  }
  std::vector<int> cperm(r->KPmax, -1);
  long long cur = 0;
  std::vector<long long> pos(G);
  for (int g = 0; g < G; ++g) {
    gcoff[g] = (int)cur;
    pos[g] = cur;
    cur += rup(gkh[g], kUnitRows);
  }
  gcoff[G] = (int)cur;
  r->KP = cur;
  for (int c = 0; c < k; ++c)  // ascending center index inside a group: lowest index on ties
    if (r->group_h[c] >= 0) cperm[pos[r->group_h[c]]++] = c;
  r->st.components = (int)roots.size();
  r->st.max_group = *std::max_element(gkh.begin(), gkh.begin() + G);
  r->st.max_component = roots.empty() ? 0 : size[roots[0]];
  r->st.groups_nonempty = (int)std::count_if(gkh.begin(), gkh.begin() + G, [](int v) { return v > 0; });
  KMGB_CUDA_TRY(cudaMemcpyAsync(r->group, r->group_h.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(r->cperm, cperm.data(), sizeof(int) * r->KPmax, cudaMemcpyHostToDevice, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(r->gcoff, gcoff.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(r->gk, gkh.data(), sizeof(int) * (G + 1), cudaMemcpyHostToDevice, s));
  r->slot_group_h.assign(r->KPmax, -1);
  for (int g = 0; g < G; ++g)
    for (int j = gcoff[g]; j < gcoff[g + 1]; ++j) r->slot_group_h[j] = g;
  KMGB_CUDA_TRY(cudaMemcpyAsync(r->slot_group, r->slot_group_h.data(), sizeof(int) * r->KPmax,
                                cudaMemcpyHostToDevice, s));
  // input scale of the network: unit mean square per dimension over the sample
  std::vector<float> xn(r->Sg);
  KMGB_CUDA_TRY(cudaMemcpyAsync(xn.data(), r->sxn, sizeof(float) * r->Sg, cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(sync_err(s));
  double ms = 0.0;
  for (float v : xn) ms += (double)v * v;
  ms /= std::max(1, r->Sg);
  r->scale = ms > 0 ? (float)(1.0 / std::sqrt(ms / r->d)) : 1.0f;
  r->grouped = true;
  return cudaSuccess;
}

// Lower bounds of every center's distance to the centers outside its group, for the current
// centers (io.Cop / io.cn must belong to them).
static cudaError_t refresh_separation(Router* r, const RouterIO& io, cudaStream_t s) {
  const int k = r->k;
  fill_int_kernel<<<num_sms() * 4, 256, 0, s>>>(r->m2, k, 0x7f800000);  // +inf
  count_launches(1);
  if (io.cbias) {
    // on the tensor cores: the permuted centers against themselves in separation mode, every
    // 256-row unit skipping its own group's chunks (K^2 D work at tensor rate instead of FP32)
    AssignArgs a{};
    a.n = r->KP;
    a.k = (int)r->KP;
    a.d = r->d;
    a.cn = r->cnP;
    a.xnorm = r->xnP;
    a.cmax = io.cmax;
    a.cinit = r->cinitP;
    a.cbias = r->cbiasP;
    a.err = io.err;
    a.stop = io.stop;
    a.xmax_out = r->xmaxP;
    a.slot_group = r->slot_group;
    const void* ClP = io.Cl ? r->ClP : nullptr;
    const cudaError_t e =
        launch_assign_bf16(r->CbP, ClP, r->ldb, r->CbP, ClP, r->ldb, a, s);
    if (e == cudaSuccess) {
      m2_from_xmax_kernel<<<num_sms() * 4, 256, 0, s>>>(r->cperm, r->KP, r->cnP, r->xmaxP, r->m2,
                                                       io.stop);
      m0_kernel<<<num_sms() * 4, 256, 0, s>>>(r->m2, k, r->m0);
      count_launches(2);
      return cudaGetLastError();
    }
    if (e != cudaErrorInvalidValue && e != cudaErrorInvalidConfiguration) return e;
    cudaGetLastError();  // not launched: the SIMT kernel below
  }
  const int nt = (k + kPairTile - 1) / kPairTile;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  // |fl(c.c') - c.c'| <= gamma_d |c||c'| <= gamma_d (cn + cn')/2, doubled; the FP32 norms, the
  // FMA and the sum add at most 8 roundings of 2^-24 of (cn + cn')
  const double u = 0x1p-24;
  const double gam = io.d * u / (1.0 - io.d * u);
  const float err_rel = (float)(1.1 * (gam + 8.0 * u));
  centers_pair_kernel<kMinOut><<<(unsigned)tiles, 256, 0, s>>>(io.Cop, io.ldx, k, io.d, io.cn,
                                                               nullptr, 0.0f, r->group, nullptr,
                                                               r->m2, err_rel, nt);
  m0_kernel<<<num_sms() * 4, 256, 0, s>>>(r->m2, k, r->m0);
  count_launches(2);
  return cudaGetLastError();
}

cudaError_t router_train(Router* r, const RouterIO& io, cudaStream_t s) {
  // the iterations queued before the training are not part of its time
  KMGB_CUDA_TRY(sync_err(s));
  const auto t0 = std::chrono::steady_clock::now();
  if (!r->grouped) {
    KMGB_CUDA_TRY(form_groups(r, io, s));
    r->st.group_ms = std::chrono::duration<double, std::milli>(
                         std::chrono::steady_clock::now() - t0).count();
    // initial weights: He normal for W1 (inputs scaled to unit mean square), N(0, 1/H) for W2
    std::vector<float> p(r->np, 0.0f);
    std::mt19937_64 gen(12345);
    std::normal_distribution<float> n1(0.0f, std::sqrt(2.0f / r->d)),
        n2(0.0f, std::sqrt(1.0f / r->hidden));
    const long long w1 = (long long)r->hidden * r->d;
    for (long long i = 0; i < w1; ++i) p[i] = n1(gen);
    const long long w2o = w1 + r->hidden;
    for (long long i = 0; i < (long long)r->G * r->hidden; ++i) p[w2o + i] = n2(gen);
    KMGB_CUDA_TRY(cudaMemcpyAsync(r->P, p.data(), sizeof(float) * r->np, cudaMemcpyHostToDevice, s));
    KMGB_CUDA_TRY(cudaMemsetAsync(r->Am, 0, sizeof(float) * r->np, s));
    KMGB_CUDA_TRY(cudaMemsetAsync(r->Av, 0, sizeof(float) * r->np, s));
    KMGB_CUDA_TRY(sync_err(s));
  }
  const bool first = r->st.trainings == 0;
  const int epochs = first ? 6 : 2;
  const AdamCfg cfg{first ? 1e-3f : 5e-4f, 0.9f, 0.999f, 1e-8f};
  const int batch = std::min(kBatch, r->S);
  for (int ep = 0; ep < epochs; ++ep) {
    sample_kernel<<<num_sms() * 8, 256, 0, s>>>(
        io.X, io.ldx, io.n, io.d, io.labels, io.k, r->group,
        (unsigned long long)(r->st.trainings * 64 + ep + 1), r->S, r->scale, r->Xs, r->ys);
    count_launches(1);
    for (int b0 = 0; b0 + batch <= r->S; b0 += batch) {
      KMGB_CUDA_TRY(mlp_backward(r->sh, r->P, r->Xs + (size_t)b0 * r->d, r->ys + b0, batch, batch,
                                 r->Hd, r->Z, r->dZ, r->dH, r->Gr, r->lrows, s, r->gpart,
                                 mlp_split_scratch(r->sh)));
      KMGB_CUDA_TRY(mlp_adam(r->P, r->Gr, r->Am, r->Av, r->np, cfg, ++r->adam_t, s));
    }
  }
  // loss and accuracy of the last batch (forward before its update), for the statistics
  std::vector<float> lr(batch), z((size_t)batch * r->G);
  std::vector<int> y(batch);
  const long long last = (long long)(r->S / batch - 1) * batch;
  KMGB_CUDA_TRY(cudaMemcpyAsync(lr.data(), r->lrows, sizeof(float) * batch, cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(z.data(), r->Z, sizeof(float) * z.size(), cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(cudaMemcpyAsync(y.data(), r->ys + last, sizeof(int) * batch, cudaMemcpyDeviceToHost, s));
  // tensor-core copies for inference
  export_kernel<<<num_sms() * 4, 256, 0, s>>>(
      r->P, r->d, r->hidden, r->G, r->ldb, r->scale, static_cast<__nv_bfloat16*>(r->W1b), r->cin1,
      static_cast<__nv_bfloat16*>(r->W2b), r->cin2, r->G_pad);
  count_launches(1);
  KMGB_CUDA_TRY(sync_err(s));
  double ls = 0.0;
  long long hit = 0;
  for (int i = 0; i < batch; ++i) {
    ls += lr[i];
    const float* zi = z.data() + (size_t)i * r->G;
    hit += (int)(std::max_element(zi, zi + r->G) - zi) == y[i];
  }
  r->st.last_loss = ls / batch;
  r->st.last_accuracy = (double)hit / batch;
  r->st.trainings += 1;
  r->st.train_ms += std::chrono::duration<double, std::milli>(
                        std::chrono::steady_clock::now() - t0).count();
  r->trained = true;
  return cudaSuccess;
}

cudaError_t router_assign(Router* r, const RouterIO& io, int* fb_list, int* fb_count,
                          cudaStream_t s) {
  const int G = r->G;
  const long long vb = r->ldb * 2 / 16, vx = r->ldx / 4;
  if (r->prof && r->ev_used - r->ev_read > 4096) {  // read out what has accumulated
    RouterStats tmp;
    KMGB_CUDA_TRY(router_stats(r, &tmp, s));
  }
  KMGB_CUDA_TRY(r->mark(s));
  // centers in group order
  permute_centers_kernel<<<num_sms() * 8, 256, 0, s>>>(
      r->cperm, r->KP, static_cast<const uint4*>(io.Cb), static_cast<const uint4*>(io.Cl), vb,
      reinterpret_cast<const float4*>(io.Cop), vx, io.cinit, io.cn, static_cast<uint4*>(r->CbP),
      io.Cl ? static_cast<uint4*>(r->ClP) : nullptr, reinterpret_cast<float4*>(r->CopP), r->cinitP,
      r->cnP, static_cast<const uint4*>(io.cbias), static_cast<uint4*>(r->cbiasP), r->xnP,
      io.stop);
  count_launches(1);
  KMGB_CUDA_TRY(r->mark(s));
  // the separation bound for the current centers (from the permuted ones)
  KMGB_CUDA_TRY(refresh_separation(r, io, s));
  KMGB_CUDA_TRY(r->mark(s));
  // inference: hidden layer (store mode), then the group (arg-max mode), in row chunks
  for (long long r0 = 0; r0 < r->n; r0 += kChunkRows) {
    const long long rows = std::min<long long>(kChunkRows, r->n - r0);
    AssignArgs a{};
    a.n = rows;
    a.k = r->hidden;
    a.d = r->d;
    a.cinit = r->cin1;
    a.err = io.err;
    a.stop = io.stop;
    a.store_out = r->Hbuf;
    a.store_ld = r->hidden;
    a.store_relu = 1;
    KMGB_CUDA_TRY(launch_assign_bf16(static_cast<const char*>(io.Xb) + (size_t)r0 * r->ldb * 2,
                                     nullptr, r->ldb, r->W1b, nullptr, r->ldb, a, s));
    AssignArgs b{};
    b.n = rows;
    b.k = G;
    b.d = r->hidden;
    b.cinit = r->cin2;
    b.labels = r->route;
    b.out0 = r0;
    b.err = io.err;
    b.stop = io.stop;
    KMGB_CUDA_TRY(launch_assign_bf16(r->Hbuf, nullptr, r->hidden, r->W2b, nullptr, r->hidden, b, s));
  }
  KMGB_CUDA_TRY(r->mark(s));
  // sort the points by group
  KMGB_CUDA_TRY(cudaMemsetAsync(r->gcnt, 0, sizeof(int) * (G + 1), s));
  route_count_kernel<<<num_sms() * 4, 1024, sizeof(int) * G, s>>>(r->route, r->n, G, r->gk,
                                                                   r->gcnt, fb_list, fb_count,
                                                                   io.stop);
  route_tables_kernel<<<1, 1024, 0, s>>>(r->gcnt, r->gk, G, r->max_units, r->row_off, r->rend,
                                         r->gdone, r->fill, r->uprob, r->dstats, r->dstats + 4,
                                         io.stop);
  count_launches(2);
  if (io.Xl && !r->XlR) KMGB_CUDA_TRY(dev_alloc(&r->XlR, (size_t)r->rows_cap * r->ldb * 2, s));
  route_scatter_kernel<<<num_sms() * 2, 256, sizeof(int) * (2 * G + kScatterPts), s>>>(
      r->route, r->n, G, r->gk, r->row_off, r->fill, static_cast<const uint4*>(io.Xb),
      static_cast<const uint4*>(io.Xl), vb, io.xn, r->rowmap, static_cast<uint4*>(r->XbR),
      io.Xl ? static_cast<uint4*>(r->XlR) : nullptr, r->xnR, io.stop);
  count_launches(1);
  KMGB_CUDA_TRY(r->mark(s));
  // scan of each point's group, certified within the group
  KMGB_CUDA_TRY(cudaMemsetAsync(r->rcount, 0, sizeof(int) * 4, s));
  int no_floor_bits;
  std::memcpy(&no_floor_bits, &kNoFloor, sizeof(int));
  fill_int_kernel<<<num_sms() * 4, 256, 0, s>>>(reinterpret_cast<int*>(r->thrR), r->rows_cap,
                                                no_floor_bits);
  count_launches(1);
  AssignArgs a{};
  a.cn = r->cnP;
  a.xnorm = r->xnR;
  a.cmax = io.cmax;
  a.cinit = r->cinitP;
  a.cbias = io.cbias ? r->cbiasP : nullptr;  // start values by MMA, padding blocks skipped
  a.labels = r->labR;
  a.rerank_list = r->flagR;
  a.rerank_count = r->rcount;
  a.thr_out = r->thrR;
  a.err = io.err;
  a.n = r->rows_cap;
  a.k = (int)r->KP;
  a.d = r->d;
  a.certify = 1;
  a.gamma = assign_bf16_gamma(r->d);
  a.stop = io.stop;
  a.u_prob = r->uprob;
  a.g_coff = r->gcoff;
  a.g_k = r->gk;
  a.g_rend = r->rend;
  a.g_done = r->gdone;
  const void* XlR = io.Xl ? r->XlR : nullptr;
  const void* ClP = io.Cl ? r->ClP : nullptr;
  KMGB_CUDA_TRY(launch_assign_bf16(r->XbR, XlR, r->ldb, r->CbP, ClP, r->ldb, a, s));
  add_count_kernel<<<1, 32, 0, s>>>(r->rcount, r->dstats + 1, io.stop);
  count_launches(1);
  KMGB_CUDA_TRY(r->mark(s));
  // near ties inside the group: the flagged rows, compacted by group, take a second scan of
  // their group that records every center whose key reaches the point's floor; those
  // candidates are resolved exactly
  KMGB_CUDA_TRY(cudaMemsetAsync(r->gcnt2, 0, sizeof(int) * (G + 1), s));
  flag_count_kernel<<<num_sms() * 2, 1024, sizeof(int) * G, s>>>(r->flagR, r->rcount, r->rows_cap,
                                                                  r->uprob, G, r->gcnt2, io.stop);
  route_tables_kernel<<<1, 1024, 0, s>>>(r->gcnt2, r->gk, G, r->max_units, r->row_off2,
                                         r->rend2, r->gdone2, r->fill2, r->uprob2, r->dstats + 6,
                                         r->dstats + 7, io.stop);
  if (XlR && !r->Xl2) KMGB_CUDA_TRY(dev_alloc(&r->Xl2, (size_t)r->rows_cap * r->ldb * 2, s));
  flag_scatter_kernel<<<num_sms() * 4, 256, 0, s>>>(
      r->flagR, r->rcount, r->rows_cap, r->uprob, r->row_off2, r->fill2,
      static_cast<const uint4*>(r->XbR), static_cast<const uint4*>(XlR), vb, r->thrR, r->rowmap,
      static_cast<uint4*>(r->Xb2), XlR ? static_cast<uint4*>(r->Xl2) : nullptr, r->thr2, r->xrow2,
      r->rmap2, r->list2, io.stop);
  count_launches(3);
  AssignArgs c2 = a;
  c2.labels = nullptr;
  c2.certify = 0;
  c2.thr_out = nullptr;
  c2.xnorm = nullptr;
  c2.thr_in = r->thr2;
  c2.cand = r->candR;
  c2.cand_cnt = r->ccntR;
  c2.u_prob = r->uprob2;
  c2.g_rend = r->rend2;
  c2.g_done = r->gdone2;
  KMGB_CUDA_TRY(launch_assign_bf16(r->Xb2, XlR ? r->Xl2 : nullptr, r->ldb, r->CbP, ClP, r->ldb,
                                   c2, s));
  KMGB_CUDA_TRY(launch_resolve_candidates(r->list2, r->rcount, r->rows_cap, r->candR, r->ccntR,
                                          io.X, r->ldx, r->CopP, r->ldx, r->cnP, r->d, r->lab2,
                                          r->over2, r->rcount + 1, io.stop, s, r->xrow2));
  mark_over_kernel<<<num_sms() * 2, 256, 0, s>>>(r->over2, r->rcount + 1, r->rows_cap, r->lab2,
                                                 io.stop);
  flag_copy_back_kernel<<<num_sms() * 2, 256, 0, s>>>(r->list2, r->rcount, r->rows_cap, r->rmap2,
                                                      r->lab2, r->labR, io.stop);
  count_launches(2);
  KMGB_CUDA_TRY(r->mark(s));
  // certificate against every center outside the group
  router_finish_kernel<<<num_sms() * 8, 256, 0, s>>>(
      r->rows_cap, G, r->uprob, r->rend, r->rowmap, r->labR, r->KP, r->cperm, r->cnP, io.X,
      r->ldx, io.C, r->d, r->m0, io.labels, fb_list, fb_count, r->dstats, io.stop);
  add_count_kernel<<<1, 32, 0, s>>>(fb_count, r->dstats + 3, io.stop);
  count_launches(3);
  KMGB_CUDA_TRY(r->mark(s));
  r->st.routed_iterations += 1;
  return cudaGetLastError();
}

cudaError_t router_gather_fallback(const int* fb_list, const int* fb_count, long long cap,
                                   const float* X, long long ldx, const float* xn, const void* Xb,
                                   const void* Xl, long long ldb, float* XF, float* xnF, void* XbF,
                                   void* XlF, const int* stop, cudaStream_t s) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (ldx % 4 || (ldb * 2) % 16) return cudaErrorInvalidValue;
  gather_fallback_kernel<<<num_sms() * 8, 256, 0, s>>>(
      fb_list, fb_count, cap, reinterpret_cast<const float4*>(X), ldx / 4, xn,
      static_cast<const uint4*>(Xb), static_cast<const uint4*>(Xl), ldb * 2 / 16,
      reinterpret_cast<float4*>(XF), xnF, static_cast<uint4*>(XbF),
      XlF ? static_cast<uint4*>(XlF) : nullptr, stop);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t router_scatter_labels(const int* fb_list, const int* fb_count, long long cap,
                                  const int* labF, int* labels, const int* stop, cudaStream_t s) {
  scatter_fallback_kernel<<<num_sms() * 4, 256, 0, s>>>(fb_list, fb_count, cap, labF, labels, stop);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t router_stats(Router* r, RouterStats* out, cudaStream_t s) {
  unsigned long long v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  KMGB_CUDA_TRY(cudaMemcpyAsync(v, r->dstats, sizeof(v), cudaMemcpyDeviceToHost, s));
  KMGB_CUDA_TRY(cudaStreamSynchronize(s));
  // stage times of the routed iterations recorded since the last read (8 events each)
  for (; r->ev_read + 8 <= r->ev_used; r->ev_read += 8)
    for (int t = 0; t < 7; ++t) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, r->ev[r->ev_read + t], r->ev[r->ev_read + t + 1]) ==
          cudaSuccess)
        r->st.stage_ms[t] += ms;
    }
  if (r->ev_read == r->ev_used) r->ev_read = r->ev_used = 0;  // reuse the events
  r->st.scan_chunks = v[4];
  r->st.routed = v[0];
  r->st.flagged = v[1];
  r->st.certified = v[2];
  r->st.fallback = v[3];
  *out = r->st;
  return cudaSuccess;
}

}  // namespace kmgb
