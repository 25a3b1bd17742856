// Plain FP32 fused assignment for sm_103a.
//
// Replaces the reference's register-tiled SGEMM + partial arg-max (main/cuda/ClosestCenters.cu:
// 46-83 with multiply.hcu / reduction.hcu, and _dev_ClosestCentersEndNew :105-123) and the
// cuBLAS + rowTransformMinimum option (kmeans.cpp:918-955). The N x K distance matrix is never
// written:
//   * thread 0 streams 128-point x 32-float tiles of X and 128-center x 32-float tiles of C
//     through a 4-stage shared-memory ring with TMA (128-byte swizzle, mbarrier complete_tx),
//     zero-filling past N, K and D, refilling a stage once all 8 warps released it;
//   * 8 consumer warps accumulate x.c in FP32 FFMA register tiles (8 points x 8 centers per
//     thread) reading the swizzled tiles bank-conflict free;
//   * per 128-center chunk the epilogue folds d = ||c||^2 - 2 x.c into a running
//     (best, index, second best) per point; the 16 threads sharing a point merge with
//     shuffles, lowest index on ties;
//   * a point is certified when second - best > 2E, E the rigorous rounding bound of the
//     FP32 evaluation; other points are appended to a re-rank list that the exact (FP64)
//     re-rank resolves, so labels equal the FP64 arg-min.
#include <cfloat>

#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

constexpr int BM = 128;        // points per CTA tile
constexpr int BN = 128;        // centers per chunk
constexpr int BKF = 32;        // floats per k-block (128 bytes: one swizzle row)
constexpr int STAGES = 4;
constexpr int NTHREADS = 256;  // 8 warps, all computing; thread 0 also drives TMA
constexpr uint32_t TILE_BYTES = BM * BKF * 4;  // 16 KB (C tile identical)
constexpr uint32_t STAGE_BYTES = 2 * TILE_BYTES;
constexpr size_t SMEM_BYTES = STAGES * STAGE_BYTES + 1024;

__device__ __forceinline__ float bound_e(float xn, float cm, float gamma, int d) {
  // |d~ - (||c||^2 - 2 x.c)| <= u cm^2 + 2 gamma xn cm + u (cm^2 + 2.001 xn cm), plus the FP64
  // reference's own error (d+2) 2^-52 (xn + cm)^2; 1% slack covers FP32 evaluation of E.
  const float u = 5.9604645e-8f;  // 2^-24
  const float xc = xn * cm;
  const float s64 = (float)(d + 2) * 2.220446e-16f * (xn + cm) * (xn + cm);
  const float e = u * cm * cm + 2.0f * gamma * xc + u * (cm * cm + 2.001f * xc) + s64;
  return e * 1.01f + 1e-30f;
}

__global__ void __launch_bounds__(NTHREADS, 1)
assign_fp32_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmC,
                   AssignArgs p) {
  if (stopped(p.stop)) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ int abort_flag;

  const int tid = threadIdx.x;
  const long long row0 = (long long)blockIdx.x * BM;
  const int nkb = (p.d + BKF - 1) / BKF;
  const int nchunks = (p.k + BN - 1) / BN;
  const int total = nchunks * nkb;

  // Thread 0 doubles as the TMA producer: it fills the ring, then refills each stage as soon
  // as all 8 warps have released it.
  // test hook: steps from p.test_withhold on are never loaded, so the wait for the first of them
  // runs out (every step before it has been loaded and consumed: no copy is left in flight)
  const unsigned long long wait_lim = p.test_wait_cycles ? p.test_wait_cycles : KMGB_WAIT_CYCLES;
  auto issue = [&](int step) {
    if (p.test_withhold > 0 && step >= p.test_withhold) return;
    const int stage = step % STAGES;
    const int chunk = step / nkb, kb = step % nkb;
    const uint32_t dst = smem_u32(smem + stage * STAGE_BYTES);
    const uint32_t bar = smem_u32(&full_bar[stage]);
    mbar_arrive_expect_tx(bar, STAGE_BYTES);
    tma_load_2d(dst, &tmX, bar, kb * BKF, (int)row0);
    tma_load_2d(dst + TILE_BYTES, &tmC, bar, kb * BKF, chunk * BN);
  };

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), NTHREADS / 32);
    }
    fence_mbar_init();
    prefetch_tmap(&tmX);
    prefetch_tmap(&tmC);
  }
  __syncthreads();
  if (tid == 0)
    for (int s = 0; s < STAGES && s < total; ++s) issue(s);

  // ---------------- consumer warps ----------------
  const int lane = tid & 31;
  const int tx = tid & 15;   // center group
  const int ty = tid >> 4;   // point group
  float b1[8], b2[8];
  int i1[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    b1[i] = INFINITY;
    b2[i] = INFINITY;
    i1[i] = -1;
  }

  int s = 0;
  bool alive = true;
  for (int chunk = 0; chunk < nchunks && alive; ++chunk) {
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    for (int kb = 0; kb < nkb; ++kb, ++s) {
      const int stage = s % STAGES;
      const uint32_t parity = (s / STAGES) & 1;
      bool ok = mbar_wait(smem_u32(&full_bar[stage]), parity, &abort_flag, p.err,
                          KMGB_DEV_TIMEOUT_FULL, wait_lim);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        alive = false;
        break;
      }
      const uint8_t* xs = smem + stage * STAGE_BYTES;
      const uint8_t* cs = xs + TILE_BYTES;
#pragma unroll
      for (int q = 0; q < BKF / 4; ++q) {
        float4 cv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j)
          cv[j] = *reinterpret_cast<const float4*>(cs + swz128(tx + 16 * j, q));
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float4 xv = *reinterpret_cast<const float4*>(xs + swz128(ty + 16 * i, q));
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            acc[i][j] = fmaf(xv.x, cv[j].x, acc[i][j]);
            acc[i][j] = fmaf(xv.y, cv[j].y, acc[i][j]);
            acc[i][j] = fmaf(xv.z, cv[j].z, acc[i][j]);
            acc[i][j] = fmaf(xv.w, cv[j].w, acc[i][j]);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&empty_bar[stage]));
      if (tid < 32) {  // warp 0: thread 0 refills the stage once every warp released it
        bool ok2 = true;
        if (tid == 0 && s + STAGES < total) {
          ok2 = mbar_wait(smem_u32(&empty_bar[stage]), parity, &abort_flag, p.err,
                          KMGB_DEV_TIMEOUT_EMPTY, wait_lim);
          if (ok2) issue(s + STAGES);
        }
        if (!__all_sync(0xffffffffu, ok2)) {
          alive = false;
          break;
        }
      }
    }
    if (!alive) break;

    // epilogue: fold this chunk into (best, index, second) per point
    float cnv[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = chunk * BN + tx + 16 * j;
      cnv[j] = (c < p.k) ? __ldg(p.cn + c) : INFINITY;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float dv = fmaf(-2.0f, acc[i][j], cnv[j]);
        const float nb2 = fminf(b2[i], fmaxf(b1[i], dv));
        const bool lt = dv < b1[i];
        b1[i] = lt ? dv : b1[i];
        i1[i] = lt ? (chunk * BN + tx + 16 * j) : i1[i];
        b2[i] = nb2;
      }
    }
  }
  if (!alive) return;

  // merge across the 16 threads that share each point (lanes differing in tx)
#pragma unroll
  for (int off = 1; off < 16; off <<= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float ob1 = __shfl_xor_sync(0xffffffffu, b1[i], off);
      const float ob2 = __shfl_xor_sync(0xffffffffu, b2[i], off);
      const int oi1 = __shfl_xor_sync(0xffffffffu, i1[i], off);
      const float nb2 = fminf(fminf(b2[i], ob2), fmaxf(b1[i], ob1));
      const bool take = (ob1 < b1[i]) || (ob1 == b1[i] && (unsigned)oi1 < (unsigned)i1[i]);
      b1[i] = take ? ob1 : b1[i];
      i1[i] = take ? oi1 : i1[i];
      b2[i] = nb2;
    }
  }

  if (tx == 0) {
    const float cm = p.certify ? __ldg(p.cmax) : 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const long long pt = row0 + ty + 16 * i;
      if (pt < p.n) {
        p.labels[pt] = i1[i] < 0 ? 0 : i1[i];
        if (p.certify) {
          const float e = bound_e(__ldg(p.xnorm + pt), cm, p.gamma, p.d);
          const float margin = b2[i] - b1[i];
          if (!(margin > 2.0f * e)) {
            const int slot = atomicAdd(p.rerank_count, 1);
            p.rerank_list[slot] = (int)pt;
          }
        }
      }
    }
  }
}

// Batched problems of one dimension (GroupArgs): tile t = rows 128t .. 128t+127 belongs to
// problem g.tile_prob[t], whose centers are rows c_off .. c_off + k - 1 of the shared center
// matrix. A persistent grid walks the tiles t = blockIdx.x, += gridDim.x; thread 0 keeps a cursor
// over the flattened (tile, chunk, k-block) steps so the TMA ring runs on across tile boundaries
// (a problem of ~100 centers is one or two chunks: without it every tile would wait for a full
// round trip). Per tile the arithmetic, the fold and the certificate are those of
// assign_fp32_kernel; labels are global center indices; rows past a problem's end (padding to
// its next 128-row boundary) are not written; tiles of stopped problems are skipped.
struct TileCursor {
  long long tile;
  int chunk, kb, cbeg, nchunks;
};

__global__ void __launch_bounds__(NTHREADS, 1)
assign_fp32_grouped_kernel(const __grid_constant__ CUtensorMap tmX,
                           const __grid_constant__ CUtensorMap tmC, AssignArgs p, GroupArgs g,
                           long long ntiles) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ int abort_flag;

  const int tid = threadIdx.x;
  const int nkb = (p.d + BKF - 1) / BKF;
  auto live = [&](long long t) { return !(g.done && g.done[g.tile_prob[t]]); };
  auto first_tile = [&](long long t) {
    while (t < ntiles && !live(t)) t += gridDim.x;
    return t;
  };
  auto open_tile = [&](TileCursor& c, long long t) {
    c.tile = t;
    c.chunk = 0;
    c.kb = 0;
    if (t < ntiles) {
      const int prob = g.tile_prob[t];
      c.cbeg = g.c_off[prob];
      c.nchunks = (g.k[prob] + BN - 1) / BN;
    }
  };
  // producer cursor (thread 0 only)
  TileCursor pc{};
  auto issue_next = [&](int stage) -> bool {
    if (pc.tile >= ntiles) return false;
    const uint32_t dst = smem_u32(smem + stage * STAGE_BYTES);
    const uint32_t bar = smem_u32(&full_bar[stage]);
    mbar_arrive_expect_tx(bar, STAGE_BYTES);
    tma_load_2d(dst, &tmX, bar, pc.kb * BKF, (int)(pc.tile * BM));
    tma_load_2d(dst + TILE_BYTES, &tmC, bar, pc.kb * BKF, pc.cbeg + pc.chunk * BN);
    if (++pc.kb == nkb) {
      pc.kb = 0;
      if (++pc.chunk == pc.nchunks) open_tile(pc, first_tile(pc.tile + gridDim.x));
    }
    return true;
  };

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), NTHREADS / 32);
    }
    fence_mbar_init();
    prefetch_tmap(&tmX);
    prefetch_tmap(&tmC);
  }
  __syncthreads();
  if (tid == 0) {
    open_tile(pc, first_tile(blockIdx.x));
    for (int s = 0; s < STAGES; ++s)
      if (!issue_next(s)) break;
  }

  const int lane = tid & 31;
  const int tx = tid & 15;
  const int ty = tid >> 4;
  const float cm = p.certify ? __ldg(p.cmax) : 0.0f;
  long long s = 0;  // steps consumed
  bool alive = true;
  for (long long t = first_tile(blockIdx.x); t < ntiles && alive; t = first_tile(t + gridDim.x)) {
    const int prob = g.tile_prob[t];
    const int cbeg = g.c_off[prob], kp = g.k[prob];
    const long long rend = g.row_end[prob];
    const long long row0 = t * BM;
    const int nchunks = (kp + BN - 1) / BN;
    float b1[8], b2[8];
    int i1[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      b1[i] = INFINITY;
      b2[i] = INFINITY;
      i1[i] = -1;
    }
    for (int chunk = 0; chunk < nchunks && alive; ++chunk) {
      float acc[8][8];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
      for (int kb = 0; kb < nkb; ++kb, ++s) {
        const int stage = (int)(s % STAGES);
        const uint32_t parity = (uint32_t)((s / STAGES) & 1);
        bool ok = mbar_wait(smem_u32(&full_bar[stage]), parity, &abort_flag, p.err,
                            KMGB_DEV_TIMEOUT_FULL);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) {
          alive = false;
          break;
        }
        const uint8_t* xs = smem + stage * STAGE_BYTES;
        const uint8_t* cs = xs + TILE_BYTES;
#pragma unroll
        for (int q = 0; q < BKF / 4; ++q) {
          float4 cv[8];
#pragma unroll
          for (int j = 0; j < 8; ++j)
            cv[j] = *reinterpret_cast<const float4*>(cs + swz128(tx + 16 * j, q));
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float4 xv = *reinterpret_cast<const float4*>(xs + swz128(ty + 16 * i, q));
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              acc[i][j] = fmaf(xv.x, cv[j].x, acc[i][j]);
              acc[i][j] = fmaf(xv.y, cv[j].y, acc[i][j]);
              acc[i][j] = fmaf(xv.z, cv[j].z, acc[i][j]);
              acc[i][j] = fmaf(xv.w, cv[j].w, acc[i][j]);
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&empty_bar[stage]));
        if (tid < 32) {  // warp 0: thread 0 refills the stage once every warp released it
          bool ok2 = true;
          if (tid == 0 && pc.tile < ntiles) {
            ok2 = mbar_wait(smem_u32(&empty_bar[stage]), parity, &abort_flag, p.err,
                            KMGB_DEV_TIMEOUT_EMPTY);
            if (ok2) issue_next(stage);
          }
          if (!__all_sync(0xffffffffu, ok2)) {
            alive = false;
            break;
          }
        }
      }
      if (!alive) break;
      float cnv[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = chunk * BN + tx + 16 * j;
        cnv[j] = (c < kp) ? __ldg(p.cn + cbeg + c) : INFINITY;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float dv = fmaf(-2.0f, acc[i][j], cnv[j]);
          const float nb2 = fminf(b2[i], fmaxf(b1[i], dv));
          const bool lt = dv < b1[i];
          b1[i] = lt ? dv : b1[i];
          i1[i] = lt ? (chunk * BN + tx + 16 * j) : i1[i];
          b2[i] = nb2;
        }
      }
    }
    if (!alive) break;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const float ob1 = __shfl_xor_sync(0xffffffffu, b1[i], off);
        const float ob2 = __shfl_xor_sync(0xffffffffu, b2[i], off);
        const int oi1 = __shfl_xor_sync(0xffffffffu, i1[i], off);
        const float nb2 = fminf(fminf(b2[i], ob2), fmaxf(b1[i], ob1));
        const bool take = (ob1 < b1[i]) || (ob1 == b1[i] && (unsigned)oi1 < (unsigned)i1[i]);
        b1[i] = take ? ob1 : b1[i];
        i1[i] = take ? oi1 : i1[i];
        b2[i] = nb2;
      }
    }
    if (tx == 0) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const long long pt = row0 + ty + 16 * i;
        if (pt < rend) {
          p.labels[pt] = cbeg + (i1[i] < 0 ? 0 : i1[i]);
          if (p.certify) {
            const float e = bound_e(__ldg(p.xnorm + pt), cm, p.gamma, p.d);
            const float margin = b2[i] - b1[i];
            if (!(margin > 2.0f * e)) {
              const int slot = atomicAdd(p.rerank_count, 1);
              p.rerank_list[slot] = (int)pt;
            }
          }
        }
      }
    }
  }
}

}  // namespace

float assign_fp32_gamma(int d) {
  const double u = 5.9604644775390625e-8;  // 2^-24
  const double g = d * u / (1.0 - d * u);
  return (float)(g * 1.0001);
}

cudaError_t launch_assign_fp32(const float* X, long long ldx, const float* Cop, long long ldc,
                               const AssignArgs& a, cudaStream_t s, const GroupArgs* grp,
                               long long tiles) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (a.n <= 0 || a.k <= 0 || a.d <= 0) return cudaSuccess;
  if ((ldx % 4) || (ldc % 4) || (reinterpret_cast<uintptr_t>(X) & 15) ||
      (reinterpret_cast<uintptr_t>(Cop) & 15))
    return cudaErrorInvalidValue;
  CUtensorMap tmX, tmC;
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmX, X, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (uint64_t)a.d,
                                  (uint64_t)a.n, (uint64_t)ldx * 4, BKF, BM));
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmC, Cop, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (uint64_t)a.d,
                                  (uint64_t)a.k, (uint64_t)ldc * 4, BKF, BN));
  static bool attr_set = false;
  if (!attr_set) {
    KMGB_CUDA_TRY(cudaFuncSetAttribute(assign_fp32_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)SMEM_BYTES));
    KMGB_CUDA_TRY(cudaFuncSetAttribute(assign_fp32_grouped_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)SMEM_BYTES));
    attr_set = true;
  }
  if (grp) {
    if (tiles <= 0) return cudaSuccess;
    if (tiles * BM > a.n) return cudaErrorInvalidConfiguration;
    int dev = 0, sms = 0;
    KMGB_CUDA_TRY(cudaGetDevice(&dev));
    KMGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long grid = tiles < sms ? tiles : sms;
    assign_fp32_grouped_kernel<<<(unsigned)grid, NTHREADS, SMEM_BYTES, s>>>(tmX, tmC, a, *grp,
                                                                           tiles);
  } else {
    const long long grid = (a.n + BM - 1) / BM;
    if (grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    assign_fp32_kernel<<<(unsigned)grid, NTHREADS, SMEM_BYTES, s>>>(tmX, tmC, a);
  }
  kmgb::count_launches(1);
  return cudaGetLastError();
}

}  // namespace kmgb
