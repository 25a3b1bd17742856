// Tensor-core (tcgen05, BF16 in / FP32 accumulate in TMEM) certified assignment for sm_103a.
//
// Replaces the x.c contraction of the reference's assignment (main/cuda/ClosestCenters.cu:46-83,
// cuBLAS option kmeans.cpp:918-955) with 5th-generation tensor cores; the N x K matrix is never
// written. Per CTA (persistent, one per SM, 320 threads):
//   warp 0      TMA producer: the unit's 256 points (two 128-row BF16 tiles, all k-blocks) once,
//               then 128-center x 64-dim BF16 stages of C through a shared-memory ring
//               (128-byte swizzle, mbarrier complete_tx);
//   warp 1      TMEM owner + MMA issuer: tcgen05.mma.cta_group::1.kind::f16, M=128 N=128 K=16,
//               one accumulator per point tile per chunk, two chunk buffers (4 x 128 of the 512
//               TMEM columns) so the epilogue of chunk g overlaps the MMAs of chunk g+1;
//   warps 2-9   epilogue: each thread owns one point (its TMEM lane) of one tile. Before a chunk
//               is multiplied its accumulator is pre-loaded (tcgen05.st) with -||c_j||^2/2, so
//               the MMA yields acc_j = x.c_j - ||c_j||^2/2 and arg-min distance = arg-max acc.
//               The epilogue reads 32 columns at a time (tcgen05.ld), packs the column within
//               the 32-column block into the 5 low mantissa bits and keeps the two largest keys
//               per point with 3.5 ALU ops per element; the block of the best key is remembered.
// A point is certified when best - second > 2E, E the rigorous bound of the BF16 evaluation
// (operand rounding, FP32 accumulation, norm rounding, key packing, FP64 reference error);
// other points go to the exact re-rank list, so labels equal the FP64 arg-min.
// Every mbarrier wait is bounded (error word + CTA abort flag); TMEM is freed on every path.
#include <cfloat>

#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

constexpr int BM = 128;                  // rows per M tile
constexpr int TILES = 2;                 // M tiles per unit
constexpr int UNIT = BM * TILES;         // points per unit
constexpr int BN = 128;                  // centers per chunk (UMMA N)
constexpr int BK = 64;                   // BF16 per k-block (one 128-byte swizzle row)
constexpr int NUM_EPI_WARPS = 8;
constexpr int NTHREADS = 64 + NUM_EPI_WARPS * 32;
constexpr uint32_t KB_BYTES = BM * BK * 2;  // 16 KB: one tile k-block == one C stage
constexpr int MAX_STAGES = 8;
constexpr int MAX_D = 256;
constexpr uint32_t TMEM_COLS = 512;
constexpr size_t SMEM_CAP = 227 * 1024;  // upper bound; the device's opt-in limit is queried
constexpr float kUnusable = -3.0e38f;    // start value of padding / unusable centers
static_assert(BN / 32 >= 2, "the epilogue releases a buffer while its last block is in flight");

// UMMA instruction descriptor, kind::f16: D=F32, A=B=BF16, both K-major, N>>3, M>>4.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31, %32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),
      "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Rigorous bound (in accumulator units) of |key - (x.c - ||c||^2/2)| for any usable center.
__device__ __forceinline__ float bound_acc(float xn, float cm, int d, int planes) {
  const float u = 5.9604645e-8f;            // 2^-24, FP32 rounding
  const float ub = 1.953125e-3f;            // 2^-9, BF16 rounding
  // operand error: plain (2ub + ub^2) |x||c|; split x = xh + xl + ex, c = ch + cl + ec with
  // |xl| <= ub|x|, |ex| <= ub^2|x|: dropping xl.cl and the residues leaves <= 3.03 ub^2 |x||c|
  const float op = planes > 1 ? 3.03f * ub * ub : 2.0f * ub + ub * ub;
  // FP32 accumulation in TMEM (from zero): at most one rounding per 16-product MMA step,
  // modelled with margin as (terms/16 + 2) 2^-21 relative to |start| + sum |products|. The
  // measured worst case on GB300 is >= 6x below this (tests/test_gpu_tensor_numerics.py
  // enforces >= 4x on the keys, start value included).
  const int terms = planes > 1 ? 3 * d : d;
  const float gacc = (float)(terms / 16 + 2) * 4.76837158e-7f;
  const float pack = 3.81469727e-6f;        // 2^-18: 5 column bits in the mantissa
  const float cc = 0.5f * cm * cm;
  const float xc = xn * cm * 1.01f;
  const float s64 = (float)(d + 2) * 1.2e-16f * (xn + cm) * (xn + cm);
  // the start value -||c||^2/2 is added to the accumulator with one more FP32 rounding
  const float e = 0.5f * u * cm * cm + op * xc + (gacc + pack + u) * (cc + xc) + s64;
  return e * 1.02f + 1e-30f;
}

struct Bars {
  uint64_t x_full[2], x_empty[2], done;
  uint64_t c_full[MAX_STAGES], c_empty[MAX_STAGES];
  uint64_t acc_full[2], acc_empty[2];
};

__global__ void __launch_bounds__(NTHREADS, 1)
assign_bf16_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmXl,
                   const __grid_constant__ CUtensorMap tmC, const __grid_constant__ CUtensorMap tmCl,
                   AssignArgs p, int stages, int xbufs, int planes) {
  if (stopped(p.stop)) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                             ~static_cast<uintptr_t>(1023));
  __shared__ __align__(8) Bars bars;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkb = (p.d + BK - 1) / BK;
  const int nchunks = (p.k + BN - 1) / BN;
  // Each CTA visits the center chunks in its own rotated order, so that at any moment the CTAs
  // stream different chunks of C from L2 (all CTAs requesting the same lines at once queues
  // the loads on the same L2 slices and starves the C ring).
  const int rot = (int)(blockIdx.x % (unsigned)nchunks);
  auto chunk_of = [&](int c) { return c + rot < nchunks ? c + rot : c + rot - nchunks; };
  // rows of this launch: [row0, row0 + n_rows); a device count bounds them in candidate mode
  long long n_rows = p.n;
  if (p.n_dev) {
    const long long c = (long long)*p.n_dev - p.row0;
    n_rows = c < 0 ? 0 : (c < p.n ? c : p.n);
  }
  const long long n_units = (n_rows + UNIT - 1) / UNIT;
  const bool cand_mode = p.thr_in != nullptr;
  long long my_units = 0;
  if ((long long)blockIdx.x < n_units)
    my_units = (n_units - 1 - blockIdx.x) / gridDim.x + 1;
  const long long total_chunks = my_units * nchunks;
  // X buffer: [plane][tile][k-block] 16 KB boxes; C stage: [plane] 16 KB boxes of one
  // (chunk, k-block). plane 0 = BF16 value, plane 1 = BF16 residual (split tier).
  const size_t xbuf_bytes = (size_t)planes * TILES * nkb * KB_BYTES;
  const uint32_t stage_bytes = (uint32_t)planes * KB_BYTES;
  uint8_t* xs0 = smem;                       // X buffer b at xs0 + b * xbuf_bytes
  uint8_t* cs = smem + (size_t)xbufs * xbuf_bytes;

  if (tid == 0) {
    abort_flag = 0;
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bars.x_full[b]), 1);
      mbar_init(smem_u32(&bars.x_empty[b]), 1);
    }
    mbar_init(smem_u32(&bars.done), 1);
    for (int s = 0; s < stages; ++s) {
      mbar_init(smem_u32(&bars.c_full[s]), 1);
      mbar_init(smem_u32(&bars.c_empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bars.acc_full[b]), 1);
      mbar_init(smem_u32(&bars.acc_empty[b]), NUM_EPI_WARPS);
    }
    fence_mbar_init();
    prefetch_tmap(&tmX);
    prefetch_tmap(&tmC);
    if (planes > 1) {
      prefetch_tmap(&tmXl);
      prefetch_tmap(&tmCl);
    }
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = tmem_base_sh;

  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    if (lane == 0 && total_chunks > 0) {
      long long s = 0;
      long long lu = 0;
      bool ok = true;
      for (long long u = blockIdx.x; u < n_units && ok; u += gridDim.x, ++lu) {
        // X buffer xi is used for the (use)-th time by this unit; wait until the MMAs of its
        // previous user have completed
        const int xi = (int)(lu % xbufs);
        const long long use = lu / xbufs;
        if (use > 0 && !mbar_wait(smem_u32(&bars.x_empty[xi]), (uint32_t)((use - 1) & 1),
                                  &abort_flag, p.err, KMGB_DEV_TIMEOUT_EMPTY))
          break;
        const uint32_t xb = smem_u32(&bars.x_full[xi]);
        uint8_t* xs = xs0 + (size_t)xi * xbuf_bytes;
        mbar_arrive_expect_tx(xb, (uint32_t)xbuf_bytes);
        for (int pl = 0; pl < planes; ++pl)
          for (int t = 0; t < TILES; ++t)
            for (int kb = 0; kb < nkb; ++kb)
              tma_load_2d(smem_u32(xs + (size_t)((pl * TILES + t) * nkb + kb) * KB_BYTES),
                          pl ? &tmXl : &tmX, xb, kb * BK, (int)(p.row0 + u * UNIT + t * BM));
        for (int c = 0; c < nchunks && ok; ++c) {
          for (int kb = 0; kb < nkb; ++kb, ++s) {
            const int stage = (int)(s % stages);
            if (s >= stages &&
                !mbar_wait(smem_u32(&bars.c_empty[stage]), (uint32_t)(((s / stages) - 1) & 1),
                           &abort_flag, p.err, KMGB_DEV_TIMEOUT_EMPTY)) {
              ok = false;
              break;
            }
            const uint32_t cb = smem_u32(&bars.c_full[stage]);
            mbar_arrive_expect_tx(cb, stage_bytes);
            for (int pl = 0; pl < planes; ++pl)
              tma_load_2d(smem_u32(cs + (size_t)stage * stage_bytes + pl * KB_BYTES),
                          pl ? &tmCl : &tmC, cb, kb * BK, chunk_of(c) * BN);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer ------------------------------
    if (lane == 0 && total_chunks > 0) {
      long long s = 0, g = 0, lu = 0;
      bool ok = true;
      for (long long u = blockIdx.x; u < n_units && ok; u += gridDim.x, ++lu) {
        const int xi = (int)(lu % xbufs);
        const long long use = lu / xbufs;
        if (!mbar_wait(smem_u32(&bars.x_full[xi]), (uint32_t)(use & 1), &abort_flag, p.err,
                       KMGB_DEV_TIMEOUT_FULL))
          break;
        tc_fence_after();
        const uint8_t* xs = xs0 + (size_t)xi * xbuf_bytes;
        for (int c = 0; c < nchunks && ok; ++c, ++g) {
          const int b = (int)(g & 1);
          if (!mbar_wait(smem_u32(&bars.acc_empty[b]), (uint32_t)((g >> 1) & 1), &abort_flag,
                         p.err, KMGB_DEV_TIMEOUT_ACC)) {
            ok = false;
            break;
          }
          tc_fence_after();
          for (int kb = 0; kb < nkb; ++kb, ++s) {
            const int stage = (int)(s % stages);
            if (!mbar_wait(smem_u32(&bars.c_full[stage]), (uint32_t)((s / stages) & 1),
                           &abort_flag, p.err, KMGB_DEV_TIMEOUT_FULL)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t cbase = smem_u32(cs + (size_t)stage * stage_bytes);
#pragma unroll
            for (int t = 0; t < TILES; ++t) {
              const uint32_t xhi = smem_u32(xs + (size_t)(t * nkb + kb) * KB_BYTES);
              const uint32_t dcol = tmem_base + (uint32_t)(b * (TILES * BN) + t * BN);
              // plain: x_hi.c_hi; split: + x_hi.c_lo + x_lo.c_hi (x_lo.c_lo is below the bound)
              for (int term = 0; term < (planes > 1 ? 3 : 1); ++term) {
                const uint32_t abase =
                    term == 2 ? smem_u32(xs + (size_t)((TILES + t) * nkb + kb) * KB_BYTES) : xhi;
                const uint32_t bbase = term == 1 ? cbase + KB_BYTES : cbase;
#pragma unroll
                for (int k16 = 0; k16 < BK / 16; ++k16)
                  umma_bf16(dcol, sdesc_sw128(abase + k16 * 32), sdesc_sw128(bbase + k16 * 32),
                            (kb | term | k16) ? 1u : 0u);  // the chunk's first product starts at 0
              }
            }
            umma_commit(smem_u32(&bars.c_empty[stage]));
          }
          if (ok) umma_commit(smem_u32(&bars.acc_full[b]));
        }
        if (ok) umma_commit(smem_u32(&bars.x_empty[xi]));
      }
      // all MMAs issued by this thread have completed once `done` flips
      umma_commit(smem_u32(&bars.done));
      mbar_wait(smem_u32(&bars.done), 0u, &abort_flag, p.err, KMGB_DEV_TIMEOUT_ACC);
    }
  } else {
    // ------------------------------ epilogue ------------------------------
    const int e = warp - 2;
    const int q = warp & 3;       // TMEM lane quadrant this warp may access
    const int t = e >> 2;         // point tile
    const uint32_t lane_addr = tmem_base + ((uint32_t)(q * 32) << 16);
    const float cm = p.certify ? __ldg(p.cmax) : 0.0f;

    bool alive = true;
    for (long long g0 = 0; g0 < 2 && g0 < total_chunks; ++g0)  // both buffers start free
      if (lane == 0) mbar_arrive(smem_u32(&bars.acc_empty[g0 & 1]));
    long long g = 0;
    for (long long u = blockIdx.x; u < n_units && alive; u += gridDim.x) {
      float b1 = -INFINITY, b2 = -INFINITY;
      int bblk = -1;  // global 32-column block holding the best key
      const long long prow = u * UNIT + t * BM + q * 32 + lane;  // row within the launch
      float floor_key = INFINITY;  // candidate mode: record keys >= floor_key
      int ncand = 0;
      if (cand_mode && prow < n_rows) floor_key = __ldg(p.thr_in + p.row0 + prow);
      for (int c = 0; c < nchunks; ++c, ++g) {
        const int b = (int)(g & 1);
        bool ok = mbar_wait(smem_u32(&bars.acc_full[b]), (uint32_t)((g >> 1) & 1), &abort_flag,
                            p.err, KMGB_DEV_TIMEOUT_ACC);
        if (!__all_sync(0xffffffffu, ok)) {
          alive = false;
          break;
        }
        tc_fence_after();
        const uint32_t base = lane_addr + (uint32_t)(b * (TILES * BN) + t * BN);
        // two 32-column register buffers: the load of block cb+1 is in flight while block cb
        // is folded into (b1, b2)
        uint32_t ra[32], rb[32];
        tmem_ld32(base, ra);
        tmem_ld_wait();
#pragma unroll
        for (int cb = 0; cb < BN / 32; ++cb) {
          uint32_t (&cur)[32] = (cb & 1) ? rb : ra;
          uint32_t (&nxt)[32] = (cb & 1) ? ra : rb;
          if (cb + 1 < BN / 32) tmem_ld32(base + (cb + 1) * 32, nxt);
          // key = x.c - ||c||^2/2: the accumulator plus the column's start value (FMA pipe);
          // padding and unusable centers carry a huge negative start value
          {
            const float4* hs =
                reinterpret_cast<const float4*>(p.cinit + (size_t)chunk_of(c) * BN + cb * 32);
#pragma unroll
            for (int j4 = 0; j4 < 8; ++j4) {
              const float4 h = __ldg(hs + j4);
              cur[4 * j4 + 0] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 0]), h.x));
              cur[4 * j4 + 1] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 1]), h.y));
              cur[4 * j4 + 2] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 2]), h.z));
              cur[4 * j4 + 3] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 3]), h.w));
            }
          }
          if (cb + 2 == BN / 32) {
            // the last block's load is in flight: wait for it and hand the buffer back to the
            // MMA issuer before folding the last two blocks
            tmem_ld_wait();
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&bars.acc_empty[b]));
          }
          if (p.dump) {  // diagnostic: keys of this point before the column bits are packed
            const long long pt = u * UNIT + t * BM + q * 32 + lane;
            if (pt < n_rows) {
              float* dst = p.dump + (size_t)pt * (size_t)nchunks * BN + (size_t)chunk_of(c) * BN + cb * 32;
#pragma unroll
              for (int j = 0; j < 32; ++j) dst[j] = __uint_as_float(cur[j]);
            }
          }
          if (cand_mode) {
            // second pass over flagged points: every key at or above the floor is a candidate
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float key = __uint_as_float((cur[j] & ~0x1Fu) | (uint32_t)j);
              if (key >= floor_key) {
                if (ncand < kMaxCand)
                  p.cand[(size_t)(p.row0 + prow) * kMaxCand + ncand] = chunk_of(c) * BN + cb * 32 + j;
                ++ncand;
              }
            }
            if (cb + 1 < BN / 32 && cb + 2 != BN / 32) tmem_ld_wait();
            continue;
          }
          const float blk_before = b1;
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            const float k0 = __uint_as_float((cur[j] & ~0x1Fu) | (uint32_t)j);
            const float k1 = __uint_as_float((cur[j + 1] & ~0x1Fu) | (uint32_t)(j + 1));
            const float hi = fmaxf(k0, k1);
            const float lo = fminf(k0, k1);
            b2 = fmax3(b2, lo, fminf(b1, hi));
            b1 = fmaxf(b1, hi);
          }
          if (b1 != blk_before) bblk = chunk_of(c) * (BN / 32) + cb;  // 32-column block of the best
          if (cb + 1 < BN / 32 && cb + 2 != BN / 32) tmem_ld_wait();
        }
      }
      if (!alive) break;
      if (cand_mode) {
        if (prow < n_rows) p.cand_cnt[p.row0 + prow] = ncand > kMaxCand ? -1 : ncand;
        continue;
      }
      const long long pt = prow;
      if (pt < n_rows) {
        const bool none = !(b1 > -1.0e38f);  // no usable center at all
        const int label = (bblk < 0 || none) ? 0 : bblk * 32 + (int)(__float_as_uint(b1) & 0x1Fu);
        p.labels[pt] = label;
        if (p.certify) {
          const float eb = bound_acc(__ldg(p.xnorm + pt), cm, p.d, planes);
          if (none || !(b1 - b2 > 2.0f * eb)) {
            const int slot = atomicAdd(p.rerank_count, 1);
            p.rerank_list[slot] = (int)pt;
            // the FP64 arg-min's key is >= b1 - 2E (E bounds every key's error)
            if (p.thr_out) p.thr_out[pt] = none ? -INFINITY : __fsub_rd(b1, 2.0f * eb);
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

int g_num_sms = 0;
size_t g_smem_budget = 0;  // dynamic shared memory a CTA of this kernel may use

}  // namespace

// Shared memory of one X buffer for a dimension: planes x TILES x k-blocks x 16 KB.
static size_t xbuf_bytes_for(int d, int planes) {
  return (size_t)planes * TILES * ((d + BK - 1) / BK) * KB_BYTES;
}

bool bf16_tc_supported(int d, int planes) {
  if (d <= 0 || d > MAX_D) return false;
  // one X buffer and two C stages must fit the 227 KB a CTA can use
  return xbuf_bytes_for(d, planes) + 2 * (size_t)planes * KB_BYTES + 1024 + 1024 <= SMEM_CAP;
}

float assign_bf16_gamma(int d) {
  return (float)(2.0 * 1.953125e-3 + (d + 32) * 4.76837158e-7);
}

cudaError_t launch_assign_bf16(const void* Xb, const void* Xl, long long ldxb, const void* Cb,
                               const void* Cl, long long ldcb, const AssignArgs& a,
                               cudaStream_t s) {
  if (a.n <= 0 || a.k <= 0 || a.d <= 0) return cudaSuccess;
  const int planes = (Xl && Cl) ? 2 : 1;
  if (!bf16_tc_supported(a.d, planes) || (ldxb % 8) || (ldcb % 8) ||
      (reinterpret_cast<uintptr_t>(Xb) & 15) || (reinterpret_cast<uintptr_t>(Cb) & 15) ||
      (reinterpret_cast<uintptr_t>(Xl) & 15) || (reinterpret_cast<uintptr_t>(Cl) & 15))
    return cudaErrorInvalidValue;
  if (g_num_sms == 0) {
    int dev = 0, optin = 0;
    KMGB_CUDA_TRY(cudaGetDevice(&dev));
    KMGB_CUDA_TRY(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
    KMGB_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    KMGB_CUDA_TRY(cudaFuncGetAttributes(&fa, assign_bf16_kernel));
    size_t budget = (size_t)optin - fa.sharedSizeBytes;
    if (budget > SMEM_CAP) budget = SMEM_CAP;
    KMGB_CUDA_TRY(cudaFuncSetAttribute(assign_bf16_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget));
    g_smem_budget = budget;
  }
  const size_t xbytes = xbuf_bytes_for(a.d, planes);
  const size_t stage_bytes = (size_t)planes * KB_BYTES;
  const size_t lim = g_smem_budget;
  // double-buffer the unit's points when that still leaves a 4-stage ring for C
  const int xbufs = (2 * xbytes + 4 * stage_bytes + 1024 <= lim) ? 2 : 1;
  if (lim < xbufs * xbytes + 1024 + 2 * stage_bytes) return cudaErrorInvalidValue;
  int stages = (int)((lim - 1024 - xbufs * xbytes) / stage_bytes);
  if (stages > MAX_STAGES) stages = MAX_STAGES;
  const size_t smem = xbufs * xbytes + (size_t)stages * stage_bytes + 1024;
  CUtensorMap tmX, tmC, tmXl, tmCl;
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmX, Xb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)a.d,
                                  (uint64_t)a.n, (uint64_t)ldxb * 2, BK, BM));
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmC, Cb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)a.d,
                                  (uint64_t)a.k, (uint64_t)ldcb * 2, BK, BN));
  tmXl = tmX;
  tmCl = tmC;
  if (planes > 1) {
    KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmXl, Xl, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                    (uint64_t)a.d, (uint64_t)a.n, (uint64_t)ldxb * 2, BK, BM));
    KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmCl, Cl, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                    (uint64_t)a.d, (uint64_t)a.k, (uint64_t)ldcb * 2, BK, BN));
  }
  const long long n_units = (a.n + UNIT - 1) / UNIT;
  const int grid = (int)(n_units < g_num_sms ? n_units : g_num_sms);
  if (grid <= 0) return cudaSuccess;
  assign_bf16_kernel<<<grid, NTHREADS, smem, s>>>(tmX, tmXl, tmC, tmCl, a, stages, xbufs, planes);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace kmgb
