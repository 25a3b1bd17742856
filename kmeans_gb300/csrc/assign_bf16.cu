// Tensor-core (tcgen05, BF16 in / FP32 accumulate in TMEM) certified assignment for sm_103a.
//
// Replaces the x.c contraction of the reference's assignment (main/cuda/ClosestCenters.cu:46-83,
// cuBLAS option kmeans.cpp:918-955) with 5th-generation tensor cores; the N x K matrix is never
// written. The grid is persistent: one CTA per SM, CTAs paired in clusters of two that share one
// tensor-core instruction stream (tcgen05 cta_group::2). A pair works on units of 256 points and
// chunks of 256 centers:
//   * CTA rank r holds points r*128 .. r*128+127 of the unit (the A rows of its half of the
//     M=256 MMA) and centers r*128 .. r*128+127 of the chunk (its half of N=256), both in shared
//     memory, so each SM streams only half of every center chunk and every MMA reads 8 KB of
//     operands per SM per 128 cycles; measured on GB300, M=256 N=256 K=16 pair MMAs run at the
//     full BF16 rate while the 128x128 single-CTA form is held to ~66% by its per-instruction cost.
//   * warp 0 (both CTAs) TMA producer: the unit's points (double-buffered) and 64-dim k-blocks of
//     the centers (both planes per stage) through a ring; every load completes on the leader's
//     mbarrier (cta_group::2),
//     the leader's producer posts the expected bytes of both CTAs.
//   * warp 1 of the leader (rank 0) issues tcgen05.mma.cta_group::2.kind::f16 M=256 N=256 K=16
//     into TMEM (two 256-column accumulator buffers: the epilogue of chunk g overlaps the MMAs of
//     chunk g+1) and multicasts its commits (stage free, accumulator ready, points free) to both
//     CTAs. Warp 1 of both CTAs allocates the 512 TMEM columns collectively.
//   * warps 2.. (both CTAs) epilogue: EPQ warps per TMEM lane quadrant (2 in the split tier, 4 in
//     the plain tier), each owning 32 points and 256/EPQ of the chunk's 256 columns. A thread
//     reads 32 columns at a time (tcgen05.ld), adds -||c_j||^2/2 (FP32, FMA pipe) so that arg-min
//     distance = arg-max key, packs the column within the 32-column block into the 5 low
//     mantissa bits (one lop3) and keeps the two largest keys with 2.5 more ALU ops per element
//     (measured with ncu counters: 4.3 ALU instructions per element in all). Accumulator
//     buffers are handed back to the leader by remote mbarrier arrivals. At the end of a unit the
//     column slices of a point are merged through shared memory (bounded mbarrier handshake).
// A point is certified when best - second > 2E, E the rigorous bound of the BF16 evaluation
// (operand rounding, FP32 accumulation, norm rounding, key packing, FP64 reference error);
// other points go to the exact re-rank list, so labels equal the FP64 arg-min.
// Every mbarrier wait is bounded (error word + CTA abort flag); TMEM is freed on every path.
#include <cfloat>
#include <utility>

#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

constexpr int BM = 128;                  // points per CTA per unit (A rows of one CTA)
constexpr int UNIT = 2 * BM;             // points per pair unit (MMA M)
constexpr int BN = 256;                  // centers per chunk (MMA N)
constexpr int BNH = BN / 2;              // centers per CTA per chunk
constexpr int BK = 64;                   // BF16 per k-block (one 128-byte swizzle row)
// The epilogue has EPQ warps per TMEM lane quadrant (a template parameter): 2 for the split tier,
// whose three products per element leave the tensor pipe the longer task (more epilogue warps
// only take issue slots from the MMA and TMA threads), 4 for the plain tier, whose epilogue is
// the longer task.
constexpr int threads_for(int epq) { return 64 + 4 * epq * 32; }
constexpr uint32_t XKB_BYTES = BM * BK * 2;   // 16 KB: one k-block of one plane of the points
constexpr uint32_t CKB_BYTES = BNH * BK * 2;  // 16 KB: one k-block of one plane of the centers
constexpr int MAX_STAGES = 8;
constexpr int MAX_D = 512;  // one plane; the shared-memory check limits two planes to 320
constexpr uint32_t TMEM_COLS = 512;           // two 256-column accumulator buffers
constexpr size_t SMEM_CAP = 227 * 1024;       // upper bound; the device's opt-in limit is queried

static_assert(2 * BN <= (int)TMEM_COLS, "two accumulator buffers");
static_assert(kCenterPad % BN == 0, "start values are padded to whole chunks");

// UMMA instruction descriptor, kind::f16: D=F32, A=B=BF16, both K-major, N>>3, M>>4.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(UNIT >> 4) << 24);

// kind::f8f6f4: D=F32, A=B=E4M3 (format 0), both K-major; K = 32 elements (32 bytes) per MMA, so
// the shared-memory layout and the per-MMA byte advance are those of the BF16 path.
constexpr uint32_t IDESC8 = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(UNIT >> 4) << 24);
constexpr int BK8 = 128;  // E4M3 elements per k-block (one 128-byte swizzle row)
// Start-value MMA (AssignArgs::cbias): per chunk and CTA a 128-center x 16-column BF16 box of
// the bias matrix (32-byte rows, 32-byte swizzle) next to the center planes of the chunk's first
// stage, and one 128-row x 16-column tile of ones (A) written once per CTA.
constexpr uint32_t BIAS_BYTES = BNH * kBiasCols * 2;  // 4 KB
constexpr uint32_t ONES_BYTES = BM * kBiasCols * 2;   // 4 KB

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

// The same for a K-major tile of 32-byte rows with the 32-byte swizzle (one K=16 BF16 step).
__device__ __forceinline__ uint64_t sdesc_sw32(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(256 >> 4) << 32;   // stride byte offset: 8 rows x 32 B
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)6 << 61;            // 32-byte swizzle
  return d;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
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

__device__ __forceinline__ void tmem_ld_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Packed key of column J of a 32-column block: the key's bits with the 5 low mantissa bits
// replaced by J, (x & msk) | J with msk = ~31 held in a register, so that one lop3 with J as its
// immediate does it (written as C, the two constants took two ALU instructions per element).
template <int J>
__device__ __forceinline__ float packed_key(uint32_t x, uint32_t msk) {
  uint32_t r;
  asm("lop3.b32 %0, %1, %2, %3, 0xEC;" : "=r"(r) : "r"(x), "n"(J), "r"(msk));
  return __uint_as_float(r);
}

// Running top-2 of the packed keys over one pair of columns (J, J + 1).
template <int J>
__device__ __forceinline__ void top2_pair(const uint32_t (&cur)[32], uint32_t msk, float& b1,
                                          float& b2) {
  const float k0 = packed_key<J>(cur[J], msk);
  const float k1 = packed_key<J + 1>(cur[J + 1], msk);
  const float hi = fmaxf(k0, k1);
  const float lo = fminf(k0, k1);
  b2 = fmax3(b2, lo, fminf(b1, hi));
  b1 = fmaxf(b1, hi);
}

template <int... P>
__device__ __forceinline__ void top2_block(const uint32_t (&cur)[32], uint32_t msk, float& b1,
                                           float& b2, std::integer_sequence<int, P...>) {
  (top2_pair<2 * P>(cur, msk, b1, b2), ...);
}

// Rigorous bound (in accumulator units) of |key - (x.c - ||c||^2/2)| for any usable center.
// mode: 1 plain BF16 (x_hi.c_hi), 2 split (x_hi.c_hi + x_hi.c_lo + x_lo.c_hi), 3 split with every x
// a BF16 number (x.c_hi + x.c_lo).
__device__ __forceinline__ float bound_acc(float xn, float cm, int d, int mode, bool bias) {
  const float u = 5.9604645e-8f;            // 2^-24, FP32 rounding
  const float ub = 1.953125e-3f;            // 2^-9, BF16 rounding
  // operand error: plain (2ub + ub^2) |x||c|; split x = xh + xl + ex, c = ch + cl + ec with
  // |xl| <= ub|x|, |ex| <= ub^2|x|: dropping xl.cl and the residues leaves <= 3.03 ub^2 |x||c|;
  // x exact: only x.ec is dropped, <= ub^2 |x||c| (1.01 with margin)
  const float op = mode == 1 ? 2.0f * ub + ub * ub : (mode == 2 ? 3.03f : 1.01f) * ub * ub;
  // FP32 accumulation in TMEM (from zero): at most one rounding per 16-product MMA step,
  // modelled with margin as (terms/16 + 2) 2^-21 relative to |start| + sum |products|. The
  // measured worst case on GB300 is >= 6x below this (tests/test_gpu_tensor_numerics.py
  // enforces >= 4x on the keys, start value included).
  // products per element; the start-value MMA adds one 16-product step
  const int terms = (mode == 1 ? 1 : (mode == 2 ? 3 : 2)) * d + (bias ? 16 : 0);
  const float gacc = (float)(terms / 16 + 2) * 4.76837158e-7f;
  const float pack = 3.81469727e-6f;        // 2^-18: 5 column bits in the mantissa
  const float cc = 0.5f * cm * cm;
  const float xc = xn * cm * 1.01f;
  const float s64 = (float)(d + 2) * 1.2e-16f * (xn + cm) * (xn + cm);
  // the start value -||c||^2/2 is added to the accumulator with one more FP32 rounding
  const float e = 0.5f * u * cm * cm + op * xc + (gacc + pack + u) * (cc + xc) + s64;
  return e * 1.02f + 1e-30f;
}

// The FP8 tier's bound (accumulator units) of |key - (x.c - ||c||^2/2)|. x = sx x8 + ex with
// |ex_i| <= u8 |x_i| + ax (u8 = 2^-4: E4M3 keeps 3 mantissa bits; ax = sx 2^-10: half the spacing
// of the subnormals), likewise c with sc: dropping ex.c + x.ec + ex.ec leaves at most
// (2 u8 + u8^2)|x||c| + (1 + u8) sqrt(d) (ax |c| + ac |x|) + d ax ac. The products of E4M3 numbers
// are exact in FP32; their accumulation in TMEM takes the BF16 path's model with the magnitude
// sum|products| <= 1.2 |x||c| + that slack, and acc * (sx sc) is exact (powers of two) before
// the FMA with the start value rounds once.
__device__ __forceinline__ float bound_fp8(float xn, float cm, int d, float sx, float sc) {
  const float u = 5.9604645e-8f;
  const float u8 = 0.0625f;
  const float ax = sx * 9.765625e-4f, ac = sc * 9.765625e-4f;  // 2^-10
  const float rd = sqrtf((float)d);
  const float xc = xn * cm * 1.01f;
  const float slack = (1.0f + u8) * rd * (ax * cm + ac * xn) + (float)d * ax * ac;
  const float op = (2.0f * u8 + u8 * u8) * xc + slack;
  const float gacc = (float)(d / 16 + 2) * 4.76837158e-7f;
  const float pack = 3.81469727e-6f;
  const float cc = 0.5f * cm * cm;
  const float s64 = (float)(d + 2) * 1.2e-16f * (xn + cm) * (xn + cm);
  const float e = 0.5f * u * cm * cm + op + (gacc + pack + u) * (cc + 1.2f * xc + slack) + s64;
  return e * 1.02f + 1e-30f;
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_to_rank(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}

// Arrive on an mbarrier of either CTA of the pair. Used only to hand an accumulator buffer back
// to the leader's MMA issuer: no generic-memory data travels with it (the TMEM reads before it
// are ordered by tcgen05.fence::before_thread_sync), so the default CTA-scope release suffices;
// a cluster-scope release made every epilogue warp wait for its earlier global stores.
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}

// 2-D TMA load into this CTA's shared memory, completing on an mbarrier of either CTA of the pair.
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map,
                                                 uint32_t bar_cluster, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes.cta_group::2"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cluster), "r"(c0), "r"(c1)
      : "memory");
}

// Pull a 2-D box of a tensor into L2 ahead of its TMA load.
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap* map, int c0, int c1) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(c0), "r"(c1)
               : "memory");
}

// Pair MMA: D[tmem, both CTAs] (+)= A[smem, 128 rows per CTA] . B[smem, 128 rows per CTA]^T.
__device__ __forceinline__ void umma_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
      : "memory");
}

// Pair MMA on E4M3 operands (the FP8 tier).
__device__ __forceinline__ void umma_pair8(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                           uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(IDESC8), "r"(accumulate)
      : "memory");
}

// The same with the A operand kept in the tensor core's collector for the next MMA (fill) and
// taken from it (lastuse): one shared-memory read of A serves two products.
__device__ __forceinline__ void umma_pair_a_fill(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                                 uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16.collector::a::fill [%0], %1, %2, %3, p;\n\t}" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_pair_a_lastuse(uint32_t tmem_d, uint64_t adesc,
                                                    uint64_t bdesc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, 1, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16.collector::a::lastuse [%0], %1, %2, %3, p;\n\t}" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(IDESC)
      : "memory");
}

// Arrive on the mbarrier at this offset in both CTAs once all prior pair MMAs have completed.
__device__ __forceinline__ void umma_commit_pair(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(bar),
      "h"((uint16_t)3)
      : "memory");
}

struct Bars {
  uint64_t x_full[2], x_empty[2], done;
  uint64_t c_full[MAX_STAGES], c_empty[MAX_STAGES];
  uint64_t acc_full[2], acc_empty[2];
  uint64_t merge_full[4], merge_empty[4];
};

// the column slices handed from warps (q, 1..EPQ-1) to warp (q, 0) at the end of a unit
template <int EPQ>
struct MergeSlot {
  float b1[EPQ - 1][4][32], b2[EPQ - 1][4][32];
  int bblk[EPQ - 1][4][32], ncand[EPQ - 1][4][32];
};

// EPQ: epilogue warps per lane quadrant; F8: the FP8 tier's instantiation (mode 4 only); BIAS:
// the start values enter by MMA (AssignArgs::cbias) and the epilogue adds nothing. One CTA per
// SM: each SM sub-partition's 16K registers hold ceil(warps / 4) warps, so a thread may use 168
// registers with EPQ 2 (10 warps) and 96 with EPQ 4 (18 warps).
template <int EPQ, bool F8, bool BIAS, bool XMAX = false>
__global__ void __launch_bounds__(threads_for(EPQ), 1)
assign_bf16_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmXl,
                   const __grid_constant__ CUtensorMap tmC, const __grid_constant__ CUtensorMap tmCl,
                   const __grid_constant__ CUtensorMap tmB,
                   AssignArgs p, int stages, int xbufs, int mode) {
  constexpr int NUM_EPI_WARPS = 4 * EPQ;
  constexpr int EPI_PER_QUAD = EPQ;
  constexpr int COLS_PER_WARP = BN / EPQ;           // columns of a chunk per epilogue warp
  constexpr int CAND_PER_WARP = kMaxCand / EPQ;     // candidate slots per column slice
  static_assert(EPQ >= 2 && COLS_PER_WARP % 32 == 0 && CAND_PER_WARP >= 1, "epilogue split");
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) Bars bars;
  __shared__ MergeSlot<EPQ> merge;
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = cluster_rank();
  // the TMA boxes use the 128-byte swizzle: the dynamic area must start on a 1 KB boundary. The
  // check is uniform over the grid, so every CTA of every pair returns together.
  if ((smem_u32(smem) & 1023u) != 0) {
    if (tid == 0 && blockIdx.x == 0) set_error(p.err, KMGB_DEV_BAD_SHAPE);
    return;
  }
  const bool stop_now = stopped(p.stop);  // uniform: every CTA of the grid sees the same flag
  if (stop_now) return;
  // The two-plane variant (EPQ 2) runs the split modes 2 and 3 only; the plain BF16 tier, the FP8
  // tier and the store mode run with EPQ 4, so their code is compiled out of the split variant
  // (it kept the split epilogue from spilling).
  constexpr bool kOnePlane = EPQ > 2;
  constexpr bool fp8 = F8;
  const int bk = fp8 ? BK8 : BK;  // elements per k-block (128 bytes per row either way)
  const int nkb = (p.d + bk - 1) / bk;
  const int nchunks = (p.k + BN - 1) / BN;
  const long long pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;
  // rows of this launch: [row0, row0 + n_rows); a device count bounds them in candidate mode
  long long n_rows = p.n;
  if (p.n_dev) {
    const long long c = (long long)*p.n_dev - p.row0;
    n_rows = c < 0 ? 0 : (c < p.n ? c : p.n);
  }
  const long long n_units = (n_rows + UNIT - 1) / UNIT;
  const bool cand_mode = p.thr_in != nullptr;
  const bool grouped = p.u_prob != nullptr;
  const bool store_mode = kOnePlane && p.store_out != nullptr;
  // A unit's chunks: how many, the first center, the rows that exist, and a rotation -- each pair
  // visits the chunks in its own rotated order so that at any moment the pairs stream different
  // chunks of C from L2. Every role of both CTAs derives the same sequence (false: skipped unit).
  struct UnitInfo {
    int nch, rot, cbase;
    int cend;  // end of the unit's problem's centers (its chunks are padded to 256 past it)
    long long rend;
  };
  auto unit_info = [&](long long u, UnitInfo& ui) -> bool {
    if (!grouped) {
      ui.nch = nchunks;
      ui.cbase = 0;
      ui.rend = n_rows;
      ui.cend = p.k;
    } else {
      const int pr = p.u_prob[u];
      if (p.g_done && p.g_done[pr]) return false;
      ui.nch = (p.g_k[pr] + BN - 1) / BN;
      ui.cbase = p.g_coff[pr];
      ui.rend = p.g_rend[pr];
      ui.cend = ui.cbase + p.g_k[pr];
    }
    ui.rot = (int)(pair % ui.nch);
    return true;
  };
  auto chunk_of = [](const UnitInfo& ui, int c) {
    return c + ui.rot < ui.nch ? c + ui.rot : c + ui.rot - ui.nch;
  };
  long long total_chunks = 0;
  for (long long u = pair; u < n_units; u += npairs) {
    UnitInfo ui;
    if (unit_info(u, ui)) total_chunks += ui.nch;
  }
  // points: [buffer][plane][k-block] 16 KB boxes; C stage: [plane] 16 KB boxes of one
  // (chunk, k-block). plane 0 = BF16 value, plane 1 = BF16 residual (split tier).
  const int xplanes = mode == 2 ? 2 : 1;                // BF16 planes of the points
  const int cplanes = (mode == 2 || mode == 3) ? 2 : 1;  // and of the centers
  const size_t xbuf_bytes = (size_t)xplanes * nkb * XKB_BYTES;
  // start values by MMA (the launcher picks this variant only where the extra 4 + 4 KB fit)
  constexpr bool bias = BIAS && !F8;
  const uint32_t stage_bytes = (uint32_t)cplanes * CKB_BYTES + (bias ? BIAS_BYTES : 0u);
  uint8_t* cs = smem + (size_t)xbufs * xbuf_bytes;
  uint8_t* ones = cs + (size_t)stages * stage_bytes;  // bias: the A tile of ones
  if (bias) {
    // all ones, so that the swizzle of the tile does not matter; made visible to the tensor
    // core (async proxy) before the barrier below
    for (int i = tid; i < (int)(ONES_BYTES / 4); i += blockDim.x)
      reinterpret_cast<uint32_t*>(ones)[i] = 0x3F803F80u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }

  if (tid == 0) {
    abort_flag = 0;
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bars.x_full[b]), 1);
      mbar_init(smem_u32(&bars.x_empty[b]), 1);
      mbar_init(smem_u32(&bars.acc_full[b]), 1);
      mbar_init(smem_u32(&bars.acc_empty[b]), 2 * NUM_EPI_WARPS);  // both CTAs' epilogue warps
    }
    mbar_init(smem_u32(&bars.done), 1);
    for (int s = 0; s < stages; ++s) {
      mbar_init(smem_u32(&bars.c_full[s]), 1);
      mbar_init(smem_u32(&bars.c_empty[s]), 1);
    }
    for (int q = 0; q < 4; ++q) {
      mbar_init(smem_u32(&bars.merge_full[q]), (EPI_PER_QUAD - 1) * 32);
      mbar_init(smem_u32(&bars.merge_empty[q]), 32);
    }
    fence_mbar_init();
    prefetch_tmap(&tmX);
    prefetch_tmap(&tmC);
    if (xplanes > 1) prefetch_tmap(&tmXl);
    if (cplanes > 1) prefetch_tmap(&tmCl);
    if (bias) prefetch_tmap(&tmB);
  }
  if (warp == 1) {  // both CTAs: one collective allocation of the pair's TMEM
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // the peer's barriers are initialised before any remote arrival
  tc_fence_after();
  const uint32_t tmem_base = tmem_base_sh;

  if (warp == 0) {
    // ------------------------------ TMA producer (both CTAs) ------------------------------
    if (lane == 0 && total_chunks > 0) {
      long long s = 0, lu = 0;
      bool ok = true;
      for (long long u = pair; u < n_units && ok; u += npairs) {
        UnitInfo ui;
        if (!unit_info(u, ui)) continue;
        const int xi = (int)(lu % xbufs);
        const long long use = lu / xbufs;
        ++lu;
        // wait until the MMAs of the previous user of this buffer have completed
        if (use > 0 && !mbar_wait(smem_u32(&bars.x_empty[xi]), (uint32_t)((use - 1) & 1),
                                  &abort_flag, p.err, KMGB_DEV_TIMEOUT_EMPTY))
          break;
        const uint32_t xb_local = smem_u32(&bars.x_full[xi]);
        if (rank == 0) mbar_arrive_expect_tx(xb_local, (uint32_t)(2 * xbuf_bytes));
        const uint32_t xb = map_to_rank(xb_local, 0);
        uint8_t* xs = smem + (size_t)xi * xbuf_bytes;
        const int xrow = (int)(p.row0 + u * UNIT + rank * BM);
        for (int pl = 0; pl < xplanes; ++pl)
          for (int kb = 0; kb < nkb; ++kb)
            tma_load_2d_pair(smem_u32(xs + (size_t)(pl * nkb + kb) * XKB_BYTES), pl ? &tmXl : &tmX,
                             xb, kb * bk, xrow);
        // the next unit's points come from HBM: start them towards L2 now, so that their TMA
        // load (queued behind the center stages) is an L2 hit
        if (u + npairs < n_units) {
          const int nrow = (int)(p.row0 + (u + npairs) * UNIT + rank * BM);
          for (int pl = 0; pl < xplanes; ++pl)
            for (int kb = 0; kb < nkb; ++kb) tma_prefetch_2d(pl ? &tmXl : &tmX, kb * bk, nrow);
        }
        for (int c = 0; c < ui.nch && ok; ++c) {
          const int crow = ui.cbase + chunk_of(ui, c) * BN + (int)rank * BNH;
          for (int kb = 0; kb < nkb; ++kb, ++s) {
            const int stage = (int)(s % stages);
            if (s >= stages &&
                !mbar_wait(smem_u32(&bars.c_empty[stage]), (uint32_t)(((s / stages) - 1) & 1),
                           &abort_flag, p.err, KMGB_DEV_TIMEOUT_EMPTY)) {
              ok = false;
              break;
            }
            const uint32_t cb_local = smem_u32(&bars.c_full[stage]);
            const bool with_bias = bias && kb == 0;  // the chunk's start values ride along
            if (rank == 0)
              mbar_arrive_expect_tx(cb_local,
                                    2 * ((uint32_t)cplanes * CKB_BYTES + (with_bias ? BIAS_BYTES : 0u)));
            const uint32_t cb = map_to_rank(cb_local, 0);
            for (int pl = 0; pl < cplanes; ++pl)
              tma_load_2d_pair(smem_u32(cs + (size_t)stage * stage_bytes + pl * CKB_BYTES),
                               pl ? &tmCl : &tmC, cb, kb * bk, crow);
            if (with_bias)
              tma_load_2d_pair(smem_u32(cs + (size_t)stage * stage_bytes + cplanes * CKB_BYTES),
                               &tmB, cb, 0, crow);
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer (leader) ------------------------------
    if (lane == 0 && rank == 0 && total_chunks > 0) {
      long long s = 0, g = 0, lu = 0;
      bool ok = true;
      for (long long u = pair; u < n_units && ok; u += npairs) {
        UnitInfo ui;
        if (!unit_info(u, ui)) continue;
        const int xi = (int)(lu % xbufs);
        const long long use = lu / xbufs;
        ++lu;
        if (!mbar_wait(smem_u32(&bars.x_full[xi]), (uint32_t)(use & 1), &abort_flag, p.err,
                       KMGB_DEV_TIMEOUT_FULL))
          break;
        tc_fence_after();
        const uint8_t* xs = smem + (size_t)xi * xbuf_bytes;
        for (int c = 0; c < ui.nch && ok; ++c, ++g) {
          const int b = (int)(g & 1);
          if (!mbar_wait(smem_u32(&bars.acc_empty[b]), (uint32_t)((g >> 1) & 1), &abort_flag,
                         p.err, KMGB_DEV_TIMEOUT_ACC)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t dcol = tmem_base + (uint32_t)(b * BN);
          for (int kb = 0; kb < nkb; ++kb, ++s) {
            const int stage = (int)(s % stages);
            if (!mbar_wait(smem_u32(&bars.c_full[stage]), (uint32_t)((s / stages) & 1),
                           &abort_flag, p.err, KMGB_DEV_TIMEOUT_FULL)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t chi = smem_u32(cs + (size_t)stage * stage_bytes);
            const uint32_t xhi = smem_u32(xs + (size_t)kb * XKB_BYTES);
            // the start values -||c||^2/2 first: ones x (hi, mid, lo) pieces set the accumulator
            if (bias && kb == 0)
              umma_pair(dcol, sdesc_sw32(smem_u32(ones)),
                        sdesc_sw32(chi + (uint32_t)cplanes * CKB_BYTES), 0u);
#pragma unroll
            for (int k16 = 0; k16 < BK / 16; ++k16) {
              // the chunk's first product starts at 0 unless the start values are in
              const uint32_t acc = (bias || kb | k16) ? 1u : 0u;
              const uint64_t ahi = sdesc_sw128(xhi + k16 * 32);
              const uint64_t bhi = sdesc_sw128(chi + k16 * 32);
              if (kOnePlane && !F8 && mode == 1) {
                umma_pair(dcol, ahi, bhi, acc);
              } else if (fp8) {
                umma_pair8(dcol, ahi, bhi, acc);
              } else {
                // x_hi.c_hi, x_hi.c_lo (x_hi read once into the A collector), then x_lo.c_hi
                // unless every x is a BF16 number; x_lo.c_lo is below the bound
                umma_pair_a_fill(dcol, ahi, bhi, acc);
                umma_pair_a_lastuse(dcol, ahi, sdesc_sw128(chi + CKB_BYTES + k16 * 32));
                if (mode == 2)
                  umma_pair(dcol, sdesc_sw128(xhi + (size_t)nkb * XKB_BYTES + k16 * 32), bhi, 1u);
              }
            }
            umma_commit_pair(smem_u32(&bars.c_empty[stage]));
          }
          if (ok) umma_commit_pair(smem_u32(&bars.acc_full[b]));
        }
        if (ok) umma_commit_pair(smem_u32(&bars.x_empty[xi]));
      }
      // both CTAs learn that every MMA issued here has completed once `done` flips
      umma_commit_pair(smem_u32(&bars.done));
    }
    if (lane == 0 && total_chunks > 0)
      mbar_wait(smem_u32(&bars.done), 0u, &abort_flag, p.err, KMGB_DEV_TIMEOUT_ACC);
  } else {
    // ------------------------------ epilogue (both CTAs) ------------------------------
    const int e = warp - 2;
    const int q = warp & 3;       // TMEM lane quadrant this warp may access
    const int h = e >> 2;         // column slice of the chunk (0 .. EPI_PER_QUAD-1)
    const uint32_t lane_addr = tmem_base + ((uint32_t)(q * 32) << 16);
    const float cm = (p.certify || XMAX) ? __ldg(p.cmax) : 0.0f;
    const uint32_t acc_empty_leader0 = map_to_rank(smem_u32(&bars.acc_empty[0]), 0);
    const uint32_t acc_empty_leader1 = map_to_rank(smem_u32(&bars.acc_empty[1]), 0);

    bool alive = true;
    for (long long g0 = 0; g0 < 2 && g0 < total_chunks; ++g0)  // both buffers start free
      if (lane == 0) mbar_arrive_remote(g0 ? acc_empty_leader1 : acc_empty_leader0);
    long long g = 0, lu_next = 0;
    for (long long u = pair; u < n_units && alive; u += npairs) {
      UnitInfo ui;
      if (!unit_info(u, ui)) continue;
      const long long lu = lu_next++;    // units this warp has processed before this one
      const long long n_rows = ui.rend;  // rows of this unit that exist end here
      float b1 = -INFINITY, b2 = -INFINITY;
      int bblk = -1;  // global 32-column block holding the best key
      const long long prow = u * UNIT + rank * BM + q * 32 + lane;  // row within the launch
      float floor_key = INFINITY;  // candidate mode: record keys >= floor_key
      int ncand = 0;
      if (cand_mode && prow < n_rows) floor_key = __ldg(p.thr_in + p.row0 + prow);
      // the point's norm bound is needed only after the last chunk: load it now so that its
      // HBM latency hides behind the unit's chunks
      const float xn_pt = ((p.certify || XMAX) && !cand_mode && h == 0 && prow < n_rows)
                              ? __ldg(p.xnorm + p.out0 + prow) : 0.0f;
      // separation mode: the unit's rows (one group: groups fill whole 256-row units) skip the
      // chunks of their own group
      const int unit_group = XMAX ? __ldg(p.slot_group + u * UNIT) : 0;
      // FP8 tier: the row's scale and the accumulator multiplier sx * sc (a power of two)
      const float sx_pt = (fp8 && prow < n_rows)
                              ? __ldg(p.xscale + (cand_mode ? p.row0 : p.out0) + prow) : 0.0f;
      const float sc_all = fp8 ? __ldg(p.cscale) : 0.0f;
      const float mrow = sx_pt * sc_all;
      for (int c = 0; c < ui.nch; ++c, ++g) {
        const int b = (int)(g & 1);
        bool ok = mbar_wait(smem_u32(&bars.acc_full[b]), (uint32_t)((g >> 1) & 1), &abort_flag,
                            p.err, KMGB_DEV_TIMEOUT_ACC);
        if (!__all_sync(0xffffffffu, ok)) {
          alive = false;
          break;
        }
        tc_fence_after();
        // the chunk's 32-column blocks are dealt to the EPQ column slices in turn (block cb of
        // slice h is block cb * EPQ + h), so that a problem's last, partly padded chunk spreads
        // its real blocks over all slices
        const int chunk0 = ui.cbase + chunk_of(ui, c) * BN;  // first center of the chunk
        const uint32_t base = lane_addr + (uint32_t)(b * BN);
        // all of this warp's columns into registers at once, then the buffer goes straight back
        // to the leader's MMA issuer and the folding below overlaps the next MMAs
        uint32_t v[COLS_PER_WARP / 32][32];
#pragma unroll
        for (int cb = 0; cb < COLS_PER_WARP / 32; ++cb)
          tmem_ld32(base + (uint32_t)((cb * EPQ + h) * 32), v[cb]);
        tmem_ld_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_remote(b ? acc_empty_leader1 : acc_empty_leader0);
        if (XMAX && __ldg(p.slot_group + chunk0) == unit_group) continue;
#pragma unroll
        for (int cb = 0; cb < COLS_PER_WARP / 32; ++cb) {
          // a 32-column block wholly past the problem's centers holds padding only (unusable
          // start values): nothing to fold (the MMAs ran over it all the same)
          const int bcol = chunk0 + (cb * EPQ + h) * 32;  // first center of the block
          if (BIAS && bcol >= ui.cend) continue;
          uint32_t (&cur)[32] = v[cb];
          // key = x.c - ||c||^2/2: the accumulator plus the column's start value (FMA pipe);
          // padding and unusable centers carry a huge negative start value
          {
            const float4* hs = reinterpret_cast<const float4*>(p.cinit + (size_t)bcol);
            if (fp8) {
#pragma unroll
              for (int j4 = 0; j4 < 8; ++j4) {
                const float4 hv = __ldg(hs + j4);
                cur[4 * j4 + 0] = __float_as_uint(__fmaf_rn(__uint_as_float(cur[4 * j4 + 0]), mrow, hv.x));
                cur[4 * j4 + 1] = __float_as_uint(__fmaf_rn(__uint_as_float(cur[4 * j4 + 1]), mrow, hv.y));
                cur[4 * j4 + 2] = __float_as_uint(__fmaf_rn(__uint_as_float(cur[4 * j4 + 2]), mrow, hv.z));
                cur[4 * j4 + 3] = __float_as_uint(__fmaf_rn(__uint_as_float(cur[4 * j4 + 3]), mrow, hv.w));
              }
            } else if (!bias) {
#pragma unroll
              for (int j4 = 0; j4 < 8; ++j4) {
                const float4 hv = __ldg(hs + j4);
                cur[4 * j4 + 0] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 0]), hv.x));
                cur[4 * j4 + 1] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 1]), hv.y));
                cur[4 * j4 + 2] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 2]), hv.z));
                cur[4 * j4 + 3] = __float_as_uint(__fadd_rn(__uint_as_float(cur[4 * j4 + 3]), hv.w));
              }
            }
          }
          if (store_mode) {
            // router hidden layer: BF16 of the key (bias included), ReLU when asked; 64 bytes
            // per thread per 32-column block, as four 16-byte stores
            if (prow < n_rows) {
              uint4* dst = reinterpret_cast<uint4*>(
                  static_cast<__nv_bfloat16*>(p.store_out) +
                  (size_t)(p.out0 + prow) * (size_t)p.store_ld + bcol);
#pragma unroll
              for (int q4 = 0; q4 < 4; ++q4) {
                uint32_t w[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                  float lo = __uint_as_float(cur[q4 * 8 + 2 * t]);
                  float hi = __uint_as_float(cur[q4 * 8 + 2 * t + 1]);
                  if (p.store_relu) {
                    lo = fmaxf(lo, 0.0f);
                    hi = fmaxf(hi, 0.0f);
                  }
                  const __nv_bfloat162 b2v = __floats2bfloat162_rn(lo, hi);
                  w[t] = *reinterpret_cast<const uint32_t*>(&b2v);
                }
                dst[q4] = make_uint4(w[0], w[1], w[2], w[3]);
              }
            }
            continue;
          }
          if (p.dump) {  // diagnostic: keys of this point before the column bits are packed
            if (prow < n_rows) {
              float* dst = p.dump + (size_t)prow * (size_t)((p.k + kCenterPad - 1) / kCenterPad * kCenterPad) + bcol;
#pragma unroll
              for (int j = 0; j < 32; ++j) dst[j] = __uint_as_float(cur[j]);
            }
          }
          if (cand_mode) {
            // second pass over flagged points: every key at or above the floor is a candidate;
            // each column slice records up to CAND_PER_WARP in its own part of the point's list
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float key = __uint_as_float((cur[j] & ~0x1Fu) | (uint32_t)j);
              if (key >= floor_key) {
                if (ncand < CAND_PER_WARP && prow < n_rows)
                  p.cand[(size_t)(p.row0 + prow) * kMaxCand + h * CAND_PER_WARP + ncand] =
                      bcol + j;
                ++ncand;
              }
            }
          } else if (XMAX) {
#pragma unroll
            for (int j = 0; j < 32; ++j) b1 = fmaxf(b1, __uint_as_float(cur[j]));
          } else {
            const float blk_before = b1;
            uint32_t msk;  // ~31 in a register (see packed_key)
            asm volatile("mov.b32 %0, 0xFFFFFFE0;" : "=r"(msk));
            top2_block(cur, msk, b1, b2, std::make_integer_sequence<int, 16>{});
            if (b1 != blk_before) bblk = bcol >> 5;  // 32-column block of the best
          }
        }
      }
      if (!alive) break;
      if (store_mode) continue;  // every key was stored; no arg-max to merge
      // ---- merge the column slices of each point: warps (q, 1..) -> warp (q, 0) ----
      const uint32_t mfull = smem_u32(&bars.merge_full[q]);
      const uint32_t mempty = smem_u32(&bars.merge_empty[q]);
      if (h > 0) {
        bool ok = lu == 0 || mbar_wait(mempty, (uint32_t)((lu - 1) & 1), &abort_flag, p.err,
                                       KMGB_DEV_TIMEOUT_ACC);
        if (!__all_sync(0xffffffffu, ok)) break;
        merge.b1[h - 1][q][lane] = b1;
        merge.b2[h - 1][q][lane] = b2;
        merge.bblk[h - 1][q][lane] = bblk;
        merge.ncand[h - 1][q][lane] = ncand;
        mbar_arrive(mfull);  // release: the writes above (and the candidate list) are visible
        continue;
      }
      bool ok = mbar_wait(mfull, (uint32_t)(lu & 1), &abort_flag, p.err, KMGB_DEV_TIMEOUT_ACC);
      if (!__all_sync(0xffffffffu, ok)) break;
      float ob1[EPI_PER_QUAD - 1], ob2[EPI_PER_QUAD - 1];
      int obblk[EPI_PER_QUAD - 1], oncand[EPI_PER_QUAD - 1];
#pragma unroll
      for (int o = 0; o < EPI_PER_QUAD - 1; ++o) {
        ob1[o] = merge.b1[o][q][lane];
        ob2[o] = merge.b2[o][q][lane];
        obblk[o] = merge.bblk[o][q][lane];
        oncand[o] = merge.ncand[o][q][lane];
      }
      mbar_arrive(mempty);
      if (cand_mode) {
        if (prow < n_rows) {
          int* lst = p.cand + (size_t)(p.row0 + prow) * kMaxCand;
          bool over = ncand > CAND_PER_WARP;
          int total = over ? 0 : ncand;
#pragma unroll
          for (int o = 0; o < EPI_PER_QUAD - 1; ++o) {
            over = over || oncand[o] > CAND_PER_WARP;
            if (!over) {  // move slice o+1's candidates behind the earlier slices' (dst <= src)
              for (int i = 0; i < oncand[o]; ++i) lst[total + i] = lst[(o + 1) * CAND_PER_WARP + i];
              total += oncand[o];
            }
          }
          p.cand_cnt[p.row0 + prow] = over ? -1 : total;
        }
        continue;
      }
      // top-2 of the union, slices in order; on equal best keys the earlier slice's block is
      // kept (such a point has a zero margin and is never certified)
#pragma unroll
      for (int o = 0; o < EPI_PER_QUAD - 1; ++o) {
        const float nb2 = fmaxf(fminf(b1, ob1[o]), fmaxf(b2, ob2[o]));
        if (ob1[o] > b1) bblk = obblk[o];
        b1 = fmaxf(b1, ob1[o]);
        b2 = nb2;
      }
      const long long pt = p.out0 + prow;  // row of the data set
      if (XMAX) {  // an upper bound of the largest exact key over the other groups' centers
        if (prow < n_rows)
          p.xmax_out[pt] = b1 > -1.0e38f ? __fadd_ru(b1, bound_acc(xn_pt, cm, p.d, mode, bias))
                                          : -INFINITY;
        continue;
      }
      if (prow < n_rows) {
        const bool none = !(b1 > -1.0e38f);  // no usable center at all
        // no usable center at all: the first center of the point's problem
        const int label =
            (bblk < 0 || none) ? ui.cbase : bblk * 32 + (int)(__float_as_uint(b1) & 0x1Fu);
        p.labels[pt] = label;
        if (p.certify) {
          const float eb = (fp8 ? bound_fp8(xn_pt, cm, p.d, sx_pt, sc_all)
                                      : bound_acc(xn_pt, cm, p.d, mode, bias)) +
                           1.02f * p.pert * (xn_pt * cm * 1.01f + 0.5f * cm * cm);
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

  // every pair MMA has completed (done waited above); both CTAs free the pair's TMEM together
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

// per kernel variant: co-resident clusters of two CTAs and the dynamic shared memory a CTA may use
struct VariantInfo {
  bool ready = false;
  int max_pairs = 0;
  size_t smem_budget = 0;  // 1 KB aligned
  size_t static_bytes = 0;
};
VariantInfo g_variant[8];  // [0] FP8, [2] split BF16, [4] plain BF16, [3] / [5]: with start-value MMA,
                           // [6] / [7]: separation mode (split / plain)
int g_num_sms = 0;

template <int EPQ, bool F8, bool BIAS, bool XMAX = false>
cudaError_t prepare_variant(VariantInfo& vi) {
  if (vi.ready) return cudaSuccess;
  int dev = 0, optin = 0;
  KMGB_CUDA_TRY(cudaGetDevice(&dev));
  KMGB_CUDA_TRY(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
  KMGB_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  KMGB_CUDA_TRY(cudaFuncGetAttributes(&fa, assign_bf16_kernel<EPQ, F8, BIAS, XMAX>));
  // the dynamic area starts on the next 1 KB boundary after the static variables
  vi.static_bytes = (fa.sharedSizeBytes + 1023) / 1024 * 1024;
  size_t budget = (size_t)optin > vi.static_bytes ? (size_t)optin - vi.static_bytes : 0;
  if (budget > SMEM_CAP) budget = SMEM_CAP;
  KMGB_CUDA_TRY(cudaFuncSetAttribute(assign_bf16_kernel<EPQ, F8, BIAS, XMAX>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)budget));
  vi.smem_budget = budget;
  cudaLaunchConfig_t qc = {};
  qc.gridDim = dim3((unsigned)(g_num_sms / 2 * 2));
  qc.blockDim = dim3(threads_for(EPQ));
  qc.dynamicSmemBytes = budget;
  cudaLaunchAttribute qa[1];
  qa[0].id = cudaLaunchAttributeClusterDimension;
  qa[0].val.clusterDim.x = 2;
  qa[0].val.clusterDim.y = 1;
  qa[0].val.clusterDim.z = 1;
  qc.attrs = qa;
  qc.numAttrs = 1;
  KMGB_CUDA_TRY(cudaOccupancyMaxActiveClusters(&vi.max_pairs, assign_bf16_kernel<EPQ, F8, BIAS, XMAX>, &qc));
  if (vi.max_pairs <= 0) return cudaErrorInvalidConfiguration;
  vi.ready = true;
  return cudaSuccess;
}

// epilogue warps per lane quadrant for a tier
constexpr int epq_for(int planes) { return planes > 1 ? 2 : 4; }
// static shared memory of a variant: barriers + merge slots (+ slack), 1 KB aligned
constexpr size_t static_smem_for(int epq) { return epq > 2 ? 7168 : 3072; }

}  // namespace

// Shared memory of one point buffer for a dimension: planes x k-blocks x 16 KB.
static size_t xbuf_bytes_for(int d, int planes) {
  return (size_t)planes * ((d + BK - 1) / BK) * XKB_BYTES;
}

bool bf16_tc_supported(int d, int planes) {
  if (d <= 0 || d > MAX_D) return false;
  // one point buffer (two when they fit) and a C ring of at least two stages must fit the shared
  // memory of a CTA next to the static variables (barriers, merge slots): D <= 256 in both tiers
  return xbuf_bytes_for(d, planes) + 2 * (size_t)planes * CKB_BYTES +
             static_smem_for(epq_for(planes)) <= SMEM_CAP;
}

float assign_bf16_gamma(int d) {
  return (float)(2.0 * 1.953125e-3 + (d + 32) * 4.76837158e-7);
}

bool fp8_tc_supported(int d) {
  return d > 0 && d <= MAX_D &&
         (size_t)((d + BK8 - 1) / BK8) * XKB_BYTES + 2 * (size_t)CKB_BYTES +
                 static_smem_for(4) <= SMEM_CAP;
}

// The FP8 tier (mode 4): E4M3 rows of ld8x / ld8c bytes; one product per k-step.
static cudaError_t launch_assign_fp8(const void* X8, long long ld8x, const void* C8,
                                     long long ld8c, const AssignArgs& a, cudaStream_t s) {
  if (!fp8_tc_supported(a.d) || (ld8x % 16) || (ld8c % 16) || !a.xscale || !a.cscale ||
      (reinterpret_cast<uintptr_t>(X8) & 15) || (reinterpret_cast<uintptr_t>(C8) & 15) ||
      a.store_out || a.u_prob)
    return cudaErrorInvalidValue;
  VariantInfo& vi = g_variant[0];
  KMGB_CUDA_TRY((prepare_variant<4, true, false>(vi)));
  const size_t xbytes = (size_t)((a.d + BK8 - 1) / BK8) * XKB_BYTES;
  const size_t stage_bytes = CKB_BYTES;
  const size_t lim = vi.smem_budget;
  const int xbufs = (2 * xbytes + 3 * stage_bytes <= lim) ? 2 : 1;
  if (lim < xbufs * xbytes + 2 * stage_bytes) return cudaErrorInvalidValue;
  int stages = (int)((lim - xbufs * xbytes) / stage_bytes);
  if (stages > MAX_STAGES) stages = MAX_STAGES;
  const size_t smem = xbufs * xbytes + (size_t)stages * stage_bytes;
  CUtensorMap tmX, tmC;
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmX, X8, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, (uint64_t)a.d,
                                  (uint64_t)a.n, (uint64_t)ld8x, BK8, BM));
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmC, C8, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, (uint64_t)a.d,
                                  (uint64_t)a.k, (uint64_t)ld8c, BK8, BNH));
  const long long n_units = (a.n + UNIT - 1) / UNIT;
  const long long pairs = n_units < vi.max_pairs ? n_units : vi.max_pairs;
  if (pairs <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(2 * pairs));
  cfg.blockDim = dim3(threads_for(4));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<4, true, false>, tmX, tmX, tmC, tmC, tmC, a,
                                   stages, xbufs, 4));
  count_launches(1);
  return cudaSuccess;
}

cudaError_t launch_assign_bf16(const void* Xb, const void* Xl, long long ldxb, const void* Cb,
                               const void* Cl, long long ldcb, const AssignArgs& a,
                               cudaStream_t s) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (a.n <= 0 || a.k <= 0 || a.d <= 0) return cudaSuccess;
  if (a.fp8) return launch_assign_fp8(Xb, ldxb, Cb, ldcb, a, s);
  const int planes = (Xl && Cl) ? 2 : 1;  // planes of the split tier's point buffer
  const int mode = Cl ? (Xl ? 2 : 3) : 1;  // see bound_acc
  if (a.store_out && ((a.store_ld % 8) || (reinterpret_cast<uintptr_t>(a.store_out) & 15)))
    return cudaErrorInvalidValue;
  if (!bf16_tc_supported(a.d, planes) || (ldxb % 8) || (ldcb % 8) ||
      (reinterpret_cast<uintptr_t>(Xb) & 15) || (reinterpret_cast<uintptr_t>(Cb) & 15) ||
      (reinterpret_cast<uintptr_t>(Xl) & 15) || (reinterpret_cast<uintptr_t>(Cl) & 15))
    return cudaErrorInvalidValue;
  const int epq = epq_for(mode > 1 ? 2 : 1);
  // the budget of the variant without bias tiles decides; the variants' static shared memory
  // is the same
  VariantInfo& vi = g_variant[epq];
  if (epq == 2) KMGB_CUDA_TRY((prepare_variant<2, false, false>(vi)));
  else KMGB_CUDA_TRY((prepare_variant<4, false, false>(vi)));
  const size_t xbytes = xbuf_bytes_for(a.d, mode == 2 ? 2 : 1);
  const size_t lim = vi.smem_budget;
  // The start values by MMA (a.cbias) need 4 KB more per stage and the 4 KB tile of ones; they
  // are used where two point buffers and a 2-stage ring still fit (on GB300 the 4M x 128, K=1024
  // split tier ran as fast with 2 stages as with 3), otherwise the epilogue adds cinit.
  AssignArgs ab = a;
  if (ab.store_out) ab.cbias = nullptr;
  const size_t planes_bytes = (size_t)(mode > 1 ? 2 : 1) * CKB_BYTES;
  // (the separation mode needs them: one point buffer is enough there)
  if (ab.cbias && (ab.xmax_out ? 1 : 2) * xbytes + 2 * (planes_bytes + BIAS_BYTES) + ONES_BYTES > lim)
    ab.cbias = nullptr;
  const bool bias = ab.cbias != nullptr;
  const size_t stage_bytes = planes_bytes + (bias ? BIAS_BYTES : 0);
  const size_t extra = bias ? ONES_BYTES : 0;
  // double-buffer the unit's points when that still leaves a 3-stage ring (2 with the bias
  // tiles; a single point buffer measured ~7% slower on GB300)
  const int xbufs = (2 * xbytes + (bias ? 2 : 3) * stage_bytes + extra <= lim) ? 2 : 1;
  if (lim < xbufs * xbytes + 2 * stage_bytes + extra) return cudaErrorInvalidValue;
  int stages = (int)((lim - xbufs * xbytes - extra) / stage_bytes);
  if (stages > MAX_STAGES) stages = MAX_STAGES;
  const size_t smem = xbufs * xbytes + (size_t)stages * stage_bytes + extra;
  CUtensorMap tmX, tmC, tmXl, tmCl;
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmX, Xb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)a.d,
                                  (uint64_t)a.n, (uint64_t)ldxb * 2, BK, BM));
  KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmC, Cb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)a.d,
                                  (uint64_t)a.k, (uint64_t)ldcb * 2, BK, BNH));
  tmXl = tmX;
  tmCl = tmC;
  CUtensorMap tmB = tmC;
  if (bias) {
    // rows: the bias matrix covers round_up(k, kCenterPad) centers, like cinit
    const uint64_t brows = (uint64_t)((a.k + kCenterPad - 1) / kCenterPad) * kCenterPad;
    if (reinterpret_cast<uintptr_t>(ab.cbias) & 15) return cudaErrorInvalidValue;
    KMGB_CUDA_TRY(kmgb_make_tmap_2d_swz(&tmB, ab.cbias, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                        kBiasCols, brows, kBiasCols * 2, kBiasCols, BNH,
                                        CU_TENSOR_MAP_SWIZZLE_32B));
  }
  if (mode == 2)
    KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmXl, Xl, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                    (uint64_t)a.d, (uint64_t)a.n, (uint64_t)ldxb * 2, BK, BM));
  if (mode > 1)
    KMGB_CUDA_TRY(kmgb_make_tmap_2d(&tmCl, Cl, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                    (uint64_t)a.d, (uint64_t)a.k, (uint64_t)ldcb * 2, BK, BNH));
  const long long n_units = (a.n + UNIT - 1) / UNIT;
  const long long pairs = n_units < vi.max_pairs ? n_units : vi.max_pairs;
  if (pairs <= 0) return cudaSuccess;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(2 * pairs));
  cfg.blockDim = dim3(threads_for(epq));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (ab.xmax_out) {  // separation mode: start values by MMA, rows and chunks of whole groups
    if (!bias || !ab.slot_group || ab.u_prob || ab.thr_in || ab.certify)
      return cudaErrorInvalidValue;
    VariantInfo& vx = g_variant[epq == 2 ? 6 : 7];
    if (epq == 2) KMGB_CUDA_TRY((prepare_variant<2, false, true, true>(vx)));
    else KMGB_CUDA_TRY((prepare_variant<4, false, true, true>(vx)));
    if (vx.smem_budget < smem || vx.max_pairs < pairs) return cudaErrorInvalidConfiguration;
    if (epq == 2)
      KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<2, false, true, true>, tmX, tmXl,
                                       tmC, tmCl, tmB, ab, stages, xbufs, mode));
    else
      KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<4, false, true, true>, tmX, tmXl,
                                       tmC, tmCl, tmB, ab, stages, xbufs, mode));
    count_launches(1);
    return cudaSuccess;
  }
  if (bias) {  // the bias variants' launch limits (occupancy, shared memory) are set up too
    VariantInfo& vb = g_variant[epq + 1];
    if (epq == 2) KMGB_CUDA_TRY((prepare_variant<2, false, true>(vb)));
    else KMGB_CUDA_TRY((prepare_variant<4, false, true>(vb)));
    if (vb.smem_budget < smem || vb.max_pairs < pairs) return cudaErrorInvalidConfiguration;
  }
  if (epq == 2 && bias)
    KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<2, false, true>, tmX, tmXl, tmC, tmCl,
                                     tmB, ab, stages, xbufs, mode));
  else if (epq == 2)
    KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<2, false, false>, tmX, tmXl, tmC,
                                     tmCl, tmB, ab, stages, xbufs, mode));
  else if (bias)
    KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<4, false, true>, tmX, tmXl, tmC, tmCl,
                                     tmB, ab, stages, xbufs, mode));
  else
    KMGB_CUDA_TRY(cudaLaunchKernelEx(&cfg, assign_bf16_kernel<4, false, false>, tmX, tmXl, tmC,
                                     tmCl, tmB, ab, stages, xbufs, mode));
  count_launches(1);
  return cudaSuccess;
}

}  // namespace kmgb
