// Deterministic center update and SSE for sm_103a.
//
// Replaces the reference's privatised accumulation (main/cuda/ClusterCenters.cu:3-23, one
// G x K x D partial buffer), its per-center reduce and divide (ClusterCenters.cu:47-87), and the
// compactness reduction (main/cuda/Compactness.cu:3-59). Instead of G*K*D partials:
//   1. hist     per-tile label histogram (tile = `tile_pts` >= 4096 consecutive points),
//               K x T int32, counted in shared memory (global atomics per peer group when K
//               does not fit);
//   2. scan     exclusive scan of the K-major histogram = start of every (label, tile) run;
//   3. scatter  eight warps share a tile: each counts its slice, a scan across the warps gives
//               each its first positions, and each walks its points in order writing every
//               point id to start + rank (rank among equal labels of a 32-point step, from
//               ballot peer groups), so the sort by label is stable (ascending point id);
//   4. pieces   every label's run is cut into pieces of kSumPiece points; one lane group per
//               piece (a warp, or 32/L pieces per warp when D <= 64) sums its rows in point
//               order (FP32 data: error-free float-float sum turned into FP64 once per piece;
//               FP64 data: FP64) and the warp the rows' FP64 ||x||^2;
//   5. finalize one warp per center adds its pieces in order, divides by the count in FP64,
//               rounds once to FP32 (empty cluster: NaN as in ClusterCenters.cu:81, or keep the
//               previous center), and evaluates the cluster's SSE against the new center with
//               Q - 2 mu.S + n ||mu||^2 in FP64;
//   6. sse      one block adds the K cluster SSEs in a fixed order.
// No floating-point atomics: the result is bit-identical run to run and equals the oracle's
// canonical FP64 order.
#include <cfloat>

#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

constexpr int SCAN_T = 1024;
constexpr int SCAN_V = 8;
constexpr long long SCAN_SEG = SCAN_T * SCAN_V;

__device__ __forceinline__ int warp_incl_scan(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one int per thread (blockDim.x == SCAN_T).
__device__ int block_excl_scan(int v) {
  __shared__ int warp_tot[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int inc = warp_incl_scan(v, lane);
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    const int t = warp_tot[lane];
    const int ti = warp_incl_scan(t, lane);
    warp_tot[lane] = ti - t;
  }
  __syncthreads();
  const int res = warp_tot[w] + inc - v;
  __syncthreads();
  return res;
}

__global__ void scan_reduce_kernel(const int* __restrict__ in, long long n, int* __restrict__ sums,
                                   const int* stop) {
  if (stopped(stop)) return;
  const long long base = (long long)blockIdx.x * SCAN_SEG + (long long)threadIdx.x * SCAN_V;
  int s = 0;
#pragma unroll
  for (int v = 0; v < SCAN_V; ++v)
    if (base + v < n) s += in[base + v];
  __shared__ int red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    int t = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = t;
  }
}

// In-place exclusive scan of segment blockIdx.x, plus offset (*offsets)[blockIdx.x] if given.
__global__ void scan_seg_kernel(int* __restrict__ data, long long n, const int* __restrict__ offsets,
                                const int* stop) {
  if (stopped(stop)) return;
  const long long base = (long long)blockIdx.x * SCAN_SEG + (long long)threadIdx.x * SCAN_V;
  int vals[SCAN_V];
  int s = 0;
#pragma unroll
  for (int v = 0; v < SCAN_V; ++v) {
    vals[v] = (base + v < n) ? data[base + v] : 0;
    s += vals[v];
  }
  int pre = block_excl_scan(s);
  if (offsets) pre += offsets[blockIdx.x];
#pragma unroll
  for (int v = 0; v < SCAN_V; ++v) {
    if (base + v < n) data[base + v] = pre;
    pre += vals[v];
  }
}

// hist[l * ntiles + tile] = members of label l in the tile. SMEM: the tile counts in shared
// memory (k ints) and writes each nonzero count once; otherwise global atomics per warp group.
template <bool SMEM>
__global__ void hist_kernel(const int* __restrict__ labels, long long n, int k, int tile_pts,
                            int ntiles, int* __restrict__ hist, int* err, const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ int cnt_s[];
  const int tile = blockIdx.x;
  const long long i0 = (long long)tile * tile_pts;
  const long long i1 = min(n, i0 + tile_pts);
  const int lane = threadIdx.x & 31;
  if (SMEM) {
    for (int j = threadIdx.x; j < k; j += blockDim.x) cnt_s[j] = 0;
    __syncthreads();
  }
  const int nbits = label_bits(k);
  constexpr int U = 8;  // labels loaded ahead per thread: one memory round trip per U steps
  for (long long b = i0; b < i1; b += (long long)blockDim.x * U) {
    int lv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long i = b + (long long)u * blockDim.x + threadIdx.x;
      lv[u] = i < i1 ? __ldg(labels + i) : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      int l = lv[u];
      const long long i = b + (long long)u * blockDim.x + threadIdx.x;
      if (i < i1 && (l < 0 || l >= k)) {
        set_error(err, KMGB_DEV_BAD_LABEL);
        l = -1;
      }
      if (SMEM) {
        if (l >= 0) atomicAdd(&cnt_s[l], 1);
      } else {
        const unsigned peers = warp_peers(l, nbits);
        if (l >= 0 && lane == __ffs(peers) - 1)
          atomicAdd(&hist[(size_t)l * ntiles + tile], __popc(peers));
      }
    }
  }
  if (SMEM) {
    __syncthreads();
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
      const int c = cnt_s[j];
      if (c) hist[(size_t)j * ntiles + tile] = c;
    }
  }
}

// label_off[j] = start of label j in the sorted order, label_off[k] = n; piece_cnt[j] = pieces
// of label j (piece_cnt[k] = 0, the scan turns it into the total); counts[j] = members.
__global__ void label_offsets_kernel(const int* __restrict__ hist, long long n, int k, int ntiles,
                                     int* __restrict__ label_off, int* __restrict__ piece_cnt,
                                     long long* __restrict__ counts, const int* stop) {
  if (stopped(stop)) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > k) return;
  if (j == k) {
    label_off[k] = (int)n;
    piece_cnt[k] = 0;
    return;
  }
  const int a = hist[(size_t)j * ntiles];
  const int b = (j + 1 < k) ? hist[(size_t)(j + 1) * ntiles] : (int)n;
  label_off[j] = a;
  piece_cnt[j] = (b - a + kSumPiece - 1) / kSumPiece;
  if (counts) counts[j] = b - a;
}

template <bool SMEM>
__global__ void scatter_kernel(const int* __restrict__ labels, long long n, int k, int tile_pts,
                               int ntiles, int* pos, int* __restrict__ sorted, const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ int cnt_s[];
  const int tile = blockIdx.x;
  const int lane = threadIdx.x;
  if (tile >= ntiles) return;
  if (SMEM) {
    for (int j = lane; j < k; j += 32) cnt_s[j] = pos[(size_t)j * ntiles + tile];
    __syncwarp();
  }
  volatile int* vpos = pos;
  const long long i0 = (long long)tile * tile_pts;
  const long long i1 = min(n, i0 + tile_pts);
  const int nbits = label_bits(k);
  constexpr int U = 8;  // labels loaded ahead: one memory round trip per U steps of 32 points
  for (long long b = i0; b < i1; b += 32 * U) {
    int lv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long i = b + 32 * u + lane;
      lv[u] = i < i1 ? __ldg(labels + i) : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const long long i = b + 32 * u + lane;
      int l = lv[u];
      if (l < 0 || l >= k) l = -1;
      const unsigned peers = warp_peers(l, nbits);
      const int leader = __ffs(peers) - 1;
      const int rank = __popc(peers & lanemask_lt());
      int base = 0;
      if (l >= 0 && lane == leader)
        base = SMEM ? cnt_s[l] : vpos[(size_t)l * ntiles + tile];
      base = __shfl_sync(0xffffffffu, base, leader);
      if (l >= 0) sorted[base + rank] = (int)i;
      if (l >= 0 && lane == leader) {
        const int nv = base + __popc(peers);
        if (SMEM) cnt_s[l] = nv;
        else vpos[(size_t)l * ntiles + tile] = nv;
      }
      __syncwarp();
    }
  }
}

// Stable scatter of one tile by kScatterWarps warps: warp w takes the w-th slice of the tile's
// rows, counts its labels in shared memory, an exclusive scan over the warps (label by label,
// from the tile's start positions) gives every warp its own first positions, and the warps then
// place their rows in parallel. Same positions as one warp walking the tile in order.
constexpr int kScatterWarps = 8;

__global__ void scatter_multi_kernel(const int* __restrict__ labels, long long n, int k,
                                     int tile_pts, int ntiles, const int* __restrict__ pos,
                                     int* __restrict__ sorted, const int* stop) {
  if (stopped(stop)) return;
  extern __shared__ int wcnt[];  // [kScatterWarps][k]
  const int tile = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long i0 = (long long)tile * tile_pts;
  const long long i1 = min(n, i0 + tile_pts);
  const long long span = ((i1 - i0 + kScatterWarps - 1) / kScatterWarps + 31) / 32 * 32;
  const long long s0 = min(i1, i0 + w * span), s1 = min(i1, s0 + span);
  int* mine = wcnt + (size_t)w * k;
  for (int j = threadIdx.x; j < kScatterWarps * k; j += blockDim.x) wcnt[j] = 0;
  __syncthreads();
  for (long long i = s0 + lane; i < s1; i += 32) {
    const int l = __ldg(labels + i);
    if (l >= 0 && l < k) atomicAdd(&mine[l], 1);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < k; j += blockDim.x) {
    int run = pos[(size_t)j * ntiles + tile];
    for (int v = 0; v < kScatterWarps; ++v) {
      const int c = wcnt[(size_t)v * k + j];
      wcnt[(size_t)v * k + j] = run;
      run += c;
    }
  }
  __syncthreads();
  const int nbits = label_bits(k);
  for (long long b = s0; b < s1; b += 32) {
    const long long i = b + lane;
    int l = i < s1 ? __ldg(labels + i) : -1;
    if (l < 0 || l >= k) l = -1;
    const unsigned peers = warp_peers(l, nbits);
    const int leader = __ffs(peers) - 1;
    const int rank = __popc(peers & lanemask_lt());
    int base = 0;
    if (l >= 0 && lane == leader) base = mine[l];
    base = __shfl_sync(0xffffffffu, base, leader);
    if (l >= 0) sorted[base + rank] = (int)i;
    if (l >= 0 && lane == leader) mine[l] = base + __popc(peers);
    __syncwarp();
  }
}

// Piece accumulator. FP32 data: an error-free float-float sum (Knuth's TwoSum on the FP32
// pipe: hi + lo carries ~48 significant bits), turned into one FP64 value per piece; FP64 data:
// a plain FP64 sum. GB300 issues FP64 (and FP32->FP64 conversions) at a small fraction of the
// FP32 rate, so converting every element would bound the update.
template <typename T>
struct PieceAcc;

template <>
struct PieceAcc<float> {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(hi, x);
    const float bp = __fsub_rn(t, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    hi = t;
    lo = __fadd_rn(lo, err);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <>
struct PieceAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};

__device__ __forceinline__ int find_label(const int* __restrict__ pstart, int k, int p) {
  int lo = 0, hi = k - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(pstart + mid) <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One warp per piece; dims lane + 32 r in chunks of 256.
template <typename T>
__global__ void piece_sums_kernel(const T* __restrict__ X, long long ldx,
                                  const double* __restrict__ qn, const int* __restrict__ sorted,
                                  const int* __restrict__ label_off, const int* __restrict__ pstart,
                                  int k, int d, double* __restrict__ part,
                                  double* __restrict__ partq, const int* stop) {
  if (stopped(stop)) return;
  const int ptot = pstart[k];
  const int lane = threadIdx.x & 31;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p = gw; p < ptot; p += nw) {
    const int j = find_label(pstart, k, (int)p);
    const int q = (int)p - pstart[j];
    const int b = label_off[j] + q * kSumPiece;
    const int e = min(b + kSumPiece, label_off[j + 1]);
    for (int d0 = 0; d0 < d; d0 += 256) {
      PieceAcc<T> acc[8];
      double qs = 0.0;
#pragma unroll 4
      for (int t = b; t < e; ++t) {
        const int i = __ldg(sorted + t);
        const T* x = X + (size_t)i * ldx + d0;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const int c = lane + 32 * r;
          if (d0 + c < d) acc[r].add(__ldg(x + c));
        }
        if (qn && d0 == 0) qs += __ldg(qn + i);
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int c = d0 + lane + 32 * r;
        if (c < d) part[(size_t)p * d + c] = acc[r].value();
      }
      if (d0 == 0 && lane == 0 && partq) partq[p] = qs;
    }
  }
}

// FP32 rows with D > 64 whose width and stride are multiples of 4 (16-byte aligned). One warp per
// piece; lane l owns dimensions d0 + 4l .. d0 + 4l + 3 of each 128-dimension chunk d0 of a row.
// The rows travel by cp.async (16 bytes per lane and row) into a per-warp ring of kRingStages
// stages of kRingRows rows in shared memory, so the loads in flight hold no registers: the issuing
// side runs kRingStages - 1 stages ahead of the summing side along the warp's sequence of
// (piece, chunk, 8-row stage), across piece boundaries. A lane reads back only the 16 bytes it
// copied itself, so cp.async.wait_group alone orders its data. Every (piece, dimension) adds the
// piece's points in sorted order with the same float-float TwoSum as the generic kernel, so the
// sums are identical; the piece's sum of ||x||^2 (SSE only) is added as a tree over 32 rows at a
// time.
constexpr int kRingStages = 3;
constexpr int kRingRows = 8;
constexpr int kRingWarps = 4;
static_assert(32 % kRingRows == 0, "a stage never straddles a 32-row id window");
static_assert(kRingWarps * kRingStages * kRingRows * 32 * 16 <= 48 * 1024, "static shared memory");

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Issuing side of piece_sums_ring_kernel: the cursor over the warp's (piece, chunk, stage)
// sequence. Pieces gw, gw + nw, ...; rows b..e-1 of the current piece, chunk d0, next row t; the
// ids of the 32-row window starting at row wt in `id` (lane l: row wt + l) and, prefetched, of the
// window after it in the same chunk in `id_nx`.
struct RingCursor {
  long long p;
  int b, e, d0, t, wt, id, id_nx;
  double qs;
};

__device__ __forceinline__ int ring_window_id(const int* __restrict__ sorted, int t0, int e,
                                              int lane) {
  return t0 + lane < e ? __ldg(sorted + t0 + lane) : 0;
}

__device__ __forceinline__ void ring_start_piece(RingCursor& q, long long ptot,
                                                 const int* __restrict__ sorted,
                                                 const int* __restrict__ label_off,
                                                 const int* __restrict__ pstart, int k, int lane) {
  q.d0 = 0;
  q.qs = 0.0;
  if (q.p >= ptot) return;
  const int j = find_label(pstart, k, (int)q.p);
  q.b = label_off[j] + ((int)q.p - pstart[j]) * kSumPiece;
  q.e = min(q.b + kSumPiece, label_off[j + 1]);
  q.t = q.b;
  q.id_nx = ring_window_id(sorted, q.b, q.e, lane);
}

// Issues the next stage into ring slot `slot` (one cp.async group, empty once the warp's pieces
// are done) and describes it in `desc`: bit 0 valid, bit 1 last stage of its (piece, chunk),
// bits 2-5 rows, bits 8+ chunk; `dp` = its piece.
__device__ __forceinline__ void ring_issue(RingCursor& q, long long ptot, long long nw,
                                           const float* __restrict__ X, long long ldx,
                                           const double* __restrict__ qn,
                                           const int* __restrict__ sorted,
                                           const int* __restrict__ label_off,
                                           const int* __restrict__ pstart, int k, int d,
                                           double* __restrict__ partq, uint32_t slot_addr, int lane,
                                           int& dp, int& desc) {
  if (q.p >= ptot) {
    cp_async_commit();
    dp = 0;
    desc = 0;
    return;
  }
  const bool window = ((q.t - q.b) & 31) == 0;
  double qv = 0.0;
  if (window) {  // a new window: its ids were prefetched; prefetch the next one of the chunk
    q.wt = q.t;
    q.id = q.id_nx;
    q.id_nx = ring_window_id(sorted, q.t + 32, q.e, lane);
    if (qn && q.d0 == 0 && q.t + lane < q.e) qv = __ldg(qn + q.id);
  }
  const int nr = min(kRingRows, q.e - q.t);
  const int c = q.d0 + 4 * lane;
#pragma unroll
  for (int r = 0; r < kRingRows; ++r) {
    const int i = __shfl_sync(0xffffffffu, q.id, (q.t - q.wt + r) & 31);
    if (r < nr && c < d) cp_async16(slot_addr + r * 512, X + (size_t)i * ldx + c);
  }
  cp_async_commit();
  if (window && qn && q.d0 == 0) {  // ||x||^2 of the window's rows: tree sum (FP64)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) qv += __shfl_xor_sync(0xffffffffu, qv, o);
    q.qs += qv;
  }
  const bool last = q.t + nr >= q.e;
  dp = (int)q.p;
  desc = (q.d0 << 8) | (nr << 2) | (last ? 2 : 0) | 1;
  q.t += nr;
  if (last) {
    if (q.d0 == 0 && partq && lane == 0) partq[q.p] = q.qs;
    q.d0 += 128;
    if (q.d0 < d) {  // the piece's next chunk: rows from the start again
      q.t = q.b;
      q.id_nx = ring_window_id(sorted, q.b, q.e, lane);
    } else {
      q.p += nw;
      ring_start_piece(q, ptot, sorted, label_off, pstart, k, lane);
    }
  }
}

__global__ void __launch_bounds__(kRingWarps * 32, 4)
piece_sums_ring_kernel(const float* __restrict__ X, long long ldx, const double* __restrict__ qn,
                       const int* __restrict__ sorted, const int* __restrict__ label_off,
                       const int* __restrict__ pstart, int k, int d, double* __restrict__ part,
                       double* __restrict__ partq, const int* stop) {
  if (stopped(stop)) return;
  __shared__ __align__(16) float4 ring[kRingWarps][kRingStages][kRingRows][32];
  const long long ptot = pstart[k];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long nw = (long long)gridDim.x * kRingWarps;
  const uint32_t ring0 = (uint32_t)__cvta_generic_to_shared(&ring[w][0][0][lane]);
  constexpr uint32_t kSlotBytes = kRingRows * 32 * 16;
  static_assert(kRingStages == 3, "the descriptor queue below holds two stages");
  RingCursor q;
  q.p = (long long)blockIdx.x * kRingWarps + w;
  q.b = q.e = q.t = q.wt = q.id = q.id_nx = 0;
  ring_start_piece(q, ptot, sorted, label_off, pstart, k, lane);
  // descriptors of the two stages in flight ahead of the one being issued
  int p0, f0, p1, f1;
  ring_issue(q, ptot, nw, X, ldx, qn, sorted, label_off, pstart, k, d, partq, ring0, lane, p0, f0);
  ring_issue(q, ptot, nw, X, ldx, qn, sorted, label_off, pstart, k, d, partq, ring0 + kSlotBytes,
             lane, p1, f1);
  PieceAcc<float> a0, a1, a2, a3;
  int slot_sum = 0, slot_issue = 2;
  for (;;) {
    int p2, f2;
    ring_issue(q, ptot, nw, X, ldx, qn, sorted, label_off, pstart, k, d, partq,
               ring0 + slot_issue * kSlotBytes, lane, p2, f2);
    cp_async_wait<kRingStages - 1>();  // this lane's copies of stage slot_sum have landed
    if (!(f0 & 1)) break;
    const int c = (f0 >> 8) + 4 * lane;
    const int nr = (f0 >> 2) & 15;
    if (c < d) {
      const float4* src = &ring[w][slot_sum][0][lane];
#pragma unroll
      for (int r = 0; r < kRingRows; ++r) {
        if (r < nr) {
          const float4 v = src[r * 32];
          a0.add(v.x);
          a1.add(v.y);
          a2.add(v.z);
          a3.add(v.w);
        }
      }
      if (f0 & 2) {
        double* o = part + (size_t)p0 * d + c;
        o[0] = a0.value();
        o[1] = a1.value();
        o[2] = a2.value();
        o[3] = a3.value();
      }
    }
    if (f0 & 2) a0 = a1 = a2 = a3 = PieceAcc<float>{};
    p0 = p1;
    f0 = f1;
    p1 = p2;
    f1 = f2;
    slot_sum = slot_sum == kRingStages - 1 ? 0 : slot_sum + 1;
    slot_issue = slot_issue == kRingStages - 1 ? 0 : slot_issue + 1;
  }
  cp_async_wait<0>();
}

// Small D (a multiple of 4, at most 64): L lanes per piece, each owning 4 consecutive
// dimensions, 32/L pieces per warp. Each lane group walks its own piece's rows in order, so every
// (piece, dimension) float-float sum is the same sequence of additions as in the
// one-piece-per-warp kernel, and the whole warp computes each piece's sum of ||x||^2 with that
// kernel's 32-lane tree; the results are identical, with 32/L times the rows in flight.
template <int L>
__global__ void piece_sums_small_kernel(const float* __restrict__ X, long long ldx,
                                        const double* __restrict__ qn, const int* __restrict__ sorted,
                                        const int* __restrict__ label_off,
                                        const int* __restrict__ pstart, int k, int d,
                                        double* __restrict__ part, double* __restrict__ partq,
                                        const int* stop) {
  if (stopped(stop)) return;
  constexpr int G = 32 / L;
  const int ptot = pstart[k];
  const int lane = threadIdx.x & 31, grp = lane / L, sub = lane % L;
  const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long p0 = gw * G; p0 < ptot; p0 += nw * G) {
    const long long p = p0 + grp;
    const bool live = p < ptot;
    int b = 0, e = 0;
    if (live) {
      const int j = find_label(pstart, k, (int)p);
      b = label_off[j] + ((int)p - pstart[j]) * kSumPiece;
      e = min(b + kSumPiece, label_off[j + 1]);
    }
    if (qn) {  // the members' sum of ||x||^2, piece by piece, as the one-piece-per-warp kernel
      for (int g = 0; g < G; ++g) {
        const int bg = __shfl_sync(0xffffffffu, b, g * L);
        const int eg = __shfl_sync(0xffffffffu, e, g * L);
        if (p0 + g >= ptot) break;
        double qs = 0.0;
        for (int t0 = bg; t0 < eg; t0 += 32) {
          const int nt = min(32, eg - t0);
          double qv = lane < nt ? __ldg(qn + __ldg(sorted + t0 + lane)) : 0.0;
          for (int o = 16; o > 0; o >>= 1) qv += __shfl_xor_sync(0xffffffffu, qv, o);
          qs += qv;
        }
        if (lane == 0 && partq) partq[p0 + g] = qs;
      }
    } else if (partq && lane < G && p0 + lane < ptot) {
      partq[p0 + lane] = 0.0;
    }
    const int c = 4 * sub;
    const bool on = live && c < d;
    const int n = e - b;
    PieceAcc<float> a0, a1, a2, a3;
    for (int t = 0; t < n; t += 8) {  // eight rows in flight per lane group
      int idx[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) idx[r] = t + r < n ? __ldg(sorted + b + t + r) : -1;
      float4 v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r)
        v[r] = (on && idx[r] >= 0)
                   ? __ldg(reinterpret_cast<const float4*>(X + (size_t)idx[r] * ldx + c))
                   : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (t + r < n) {
          a0.add(v[r].x);
          a1.add(v[r].y);
          a2.add(v[r].z);
          a3.add(v[r].w);
        }
      }
    }
    if (on) {
      double* o = part + (size_t)p * d + c;
      o[0] = a0.value();
      o[1] = a1.value();
      o[2] = a2.value();
      o[3] = a3.value();
    }
  }
}

// Canonical piece sums of FP32 rows: the small-D kernel where D <= 64, the cp.async ring kernel
// for other 16-byte-aligned rows, the scalar kernel otherwise.
cudaError_t launch_piece_sums_f32(const float* X, long long ldx, const double* qn,
                                  const int* sorted, const int* label_off, const int* pstart, int k,
                                  int d, double* part, double* partq, const int* stop,
                                  long long max_pieces, cudaStream_t s) {
  // (the ring kernel's stage descriptor holds the chunk offset in 23 bits)
  const bool vec = ldx % 4 == 0 && d % 4 == 0 && d < (1 << 23) &&
                   (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  const int lanes = !vec || d > 64 ? 32 : (d <= 16 ? 4 : (d <= 32 ? 8 : 16));
  long long warps = (max_pieces + 32 / lanes - 1) / (32 / lanes);
  if (warps > kmgb::num_sms() * 64LL) warps = kmgb::num_sms() * 64LL;
  const unsigned blocks = (unsigned)((warps * 32 + 255) / 256);
  if (vec && lanes == 4)
    piece_sums_small_kernel<4><<<blocks, 256, 0, s>>>(X, ldx, qn, sorted, label_off, pstart, k, d,
                                                      part, partq, stop);
  else if (vec && lanes == 8)
    piece_sums_small_kernel<8><<<blocks, 256, 0, s>>>(X, ldx, qn, sorted, label_off, pstart, k, d,
                                                      part, partq, stop);
  else if (vec && lanes == 16)
    piece_sums_small_kernel<16><<<blocks, 256, 0, s>>>(X, ldx, qn, sorted, label_off, pstart, k,
                                                       d, part, partq, stop);
  else if (vec) {
    // four 4-warp blocks (48 KB of ring each) per SM
    const long long cap = kmgb::num_sms() * 4LL * kRingWarps;
    const long long rw = max_pieces < cap ? max_pieces : cap;
    piece_sums_ring_kernel<<<(unsigned)((rw + kRingWarps - 1) / kRingWarps), kRingWarps * 32, 0,
                             s>>>(X, ldx, qn, sorted, label_off, pstart, k, d, part, partq, stop);
  } else
    piece_sums_kernel<float><<<blocks, 256, 0, s>>>(X, ldx, qn, sorted, label_off, pstart, k, d,
                                                    part, partq, stop);
  kmgb::count_launches(1);
  return cudaGetLastError();
}

// One warp per (center j, group g of 32 dimensions): lane c of group g owns dimension
// g*32 + c, adds the center's piece sums in piece order (the canonical order: centers are
// unchanged by the split), divides in FP64 and rounds once. The group's SSE term
// sum_c (n mu^2 - 2 mu s) lands in sse_k[j * G + g]; group 0 adds the members' sum of ||x||^2.
__global__ void finalize_kernel(const double* __restrict__ part, const double* __restrict__ partq,
                                const int* __restrict__ label_off, const int* __restrict__ pstart,
                                int k, int d, float* __restrict__ C, long long ldc,
                                int empty_policy, double* __restrict__ sse_k, const int* stop) {
  if (stopped(stop)) return;
  const int groups = (d + 31) / 32;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= (long long)k * groups) return;
  const int j = (int)(wid / groups), g = (int)(wid - (long long)j * groups);
  const int c = g * 32 + lane;
  const long long n = (long long)label_off[j + 1] - label_off[j];
  const int p0 = pstart[j], p1 = pstart[j + 1];
  double sse = 0.0;
  if (c < d) {
    double s = 0.0;
    int p = p0;
    for (; p + 8 <= p1; p += 8) {  // eight loads in flight, additions in piece order
      double v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = __ldg(part + (size_t)(p + i) * d + c);
#pragma unroll
      for (int i = 0; i < 8; ++i) s += v[i];
    }
    for (; p < p1; ++p) s += __ldg(part + (size_t)p * d + c);
    float mu;
    if (n > 0) {
      mu = __double2float_rn(__ddiv_rn(s, (double)n));
      const double m = (double)mu;
      sse = fma((double)n * m, m, -2.0 * m * s);
    } else if (empty_policy == 1) {
      mu = C[(size_t)j * ldc + c];
    } else {
      mu = __int_as_float(0x7fc00000);
    }
    C[(size_t)j * ldc + c] = mu;
  }
  for (int o = 16; o > 0; o >>= 1) sse += __shfl_xor_sync(0xffffffffu, sse, o);
  // the members' sum of ||x||^2, in piece order: the warp loads 32 pieces at a time, every
  // lane adds them in order from shuffles
  double q = 0.0;
  if (g == 0 && partq && n > 0 && sse_k) {
    for (int b = p0; b < p1; b += 32) {
      const int cnt = min(32, p1 - b);
      const double v = lane < cnt ? __ldg(partq + b + lane) : 0.0;
      for (int i = 0; i < cnt; ++i) q += __shfl_sync(0xffffffffu, v, i);
    }
  }
  if (lane == 0 && sse_k) sse_k[(size_t)j * groups + g] = (n > 0) ? sse + q : 0.0;
}

// Clusters whose identity SSE (Q - 2 mu.S + n |mu|^2, summed over the groups) is within
// 1e-9 Q of zero -- singletons, duplicates, variance far below the magnitude of the points --
// get their SSE again in the direct form sum_i sum_d ((double)x - (double)mu)^2 over the
// members (exactly 0 when every member equals the center, as the reference's compactness,
// Compactness.cu:3-59, gives); the identity's cancellation error is of the order of 1e-15 Q.
// One warp per center; the direct sum only runs for flagged clusters.
__global__ void sse_fixup_kernel(double* __restrict__ sse_k, int groups,
                                 const double* __restrict__ partq, const int* __restrict__ label_off,
                                 const int* __restrict__ pstart, int k, int d,
                                 const float* __restrict__ X, long long ldx,
                                 const int* __restrict__ sorted, const float* __restrict__ C,
                                 long long ldc, const int* stop) {
  if (stopped(stop)) return;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= k) return;
  const int j = (int)wid;
  const int m0 = label_off[j], m1 = label_off[j + 1];
  if (m1 <= m0) return;
  double t = 0.0, q = 0.0;
  for (int g = lane; g < groups; g += 32) t += sse_k[(size_t)j * groups + g];
  for (int p = pstart[j] + lane; p < pstart[j + 1]; p += 32) q += partq[p];
  for (int o = 16; o > 0; o >>= 1) {
    t += __shfl_xor_sync(0xffffffffu, t, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
  }
  if (!(fabs(t) <= 1e-9 * q)) return;
  const float* mu = C + (size_t)j * ldc;
  double s = 0.0;
  for (int m = m0; m < m1; ++m) {
    const float* x = X + (size_t)sorted[m] * ldx;
    for (int c = lane; c < d; c += 32) {
      const double u = (double)x[c] - (double)mu[c];
      s = fma(u, u, s);
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  for (int g = lane; g < groups; g += 32) sse_k[(size_t)j * groups + g] = (g == 0) ? s : 0.0;
}

// Second level of the SSE reduction plus the loop's stop rule (kmeans.cpp:1234-1237,1194):
// relErr = |SSE - SSE_old| / |SSE|; the run stops once !(relErr > criterion), NaN included.
__global__ void sse_reduce_kernel(const double* __restrict__ sse_k, int k, double* __restrict__ out,
                                  int* stop, double criterion, double* sse_prev, double* rel_out,
                                  int* iters_done, int indexed) {
  if (stopped(stop)) return;
  __shared__ double red[1024];
  const int per = (k + blockDim.x - 1) / blockDim.x;
  double s = 0.0;
  for (int j = threadIdx.x * per; j < min(k, (int)(threadIdx.x + 1) * per); ++j) s += sse_k[j];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double sse = red[0];
    if (indexed && iters_done) out[*iters_done] = sse;
    else *out = sse;
    if (sse_prev) {
      const double rel = fabs(sse - *sse_prev) / fabs(sse);
      *sse_prev = sse;
      *rel_out = rel;
      *iters_done += 1;
      if (stop && !(rel > criterion)) *stop = 1;
    }
  }
}

cudaError_t excl_scan(int* data, long long n, int* tmp, cudaStream_t s, const int* stop) {
  if (n <= 0) return cudaSuccess;
  const long long nb = (n + SCAN_SEG - 1) / SCAN_SEG;
  if (nb > SCAN_SEG) return cudaErrorInvalidValue;
  if (nb == 1) {
    scan_seg_kernel<<<1, SCAN_T, 0, s>>>(data, n, nullptr, stop); kmgb::count_launches(1);
    return cudaGetLastError();
  }
  scan_reduce_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(data, n, tmp, stop); kmgb::count_launches(1);
  scan_seg_kernel<<<1, SCAN_T, 0, s>>>(tmp, nb, nullptr, stop); kmgb::count_launches(1);
  scan_seg_kernel<<<(unsigned)nb, SCAN_T, 0, s>>>(data, n, tmp, stop); kmgb::count_launches(1);
  return cudaGetLastError();
}

}  // namespace

// Tile size of the label histogram: at least 4096 points (the histogram, its scan and the
// scatter's strided counter loads scale with K x T), and K x T below ~16M entries (one scan of
// <= 64 MB).
void plan_update_tiles(long long n, int k, int* tile_pts, int* ntiles) {
  const long long per = (n * (long long)k + (16LL << 20) - 1) / (16LL << 20);
  long long tp = per < 4096 ? 4096 : (per + 31) / 32 * 32;
  if (tp > (1LL << 30)) tp = 1LL << 30;
  *tile_pts = (int)tp;
  *ntiles = (int)((n + tp - 1) / tp);
}

size_t update_scan_tmp_elems(long long elems) {
  return (size_t)((elems + SCAN_SEG - 1) / SCAN_SEG) + 1;
}

// Stable sort of the point ids by label + per-label offsets and piece starts.
static cudaError_t sort_by_label(const int* labels, const UpdateWork& w, cudaStream_t s) {
  const long long n = w.n;
  const int k = w.k;
  const long long hist_elems = (long long)k * w.ntiles;
  KMGB_CUDA_TRY(cudaMemsetAsync(w.hist, 0, sizeof(int) * hist_elems, s));
  const size_t smem = sizeof(int) * (size_t)k;
  if (smem <= 96 * 1024) {
    static int hist_attr_k = -1;
    if (smem > 48 * 1024 && hist_attr_k < k) {
      KMGB_CUDA_TRY(cudaFuncSetAttribute(hist_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
      hist_attr_k = k;
    }
    hist_kernel<true><<<w.ntiles, 256, smem, s>>>(labels, n, k, w.tile_pts, w.ntiles, w.hist, w.err,
                                                  w.stop);
  } else {
    hist_kernel<false><<<w.ntiles, 256, 0, s>>>(labels, n, k, w.tile_pts, w.ntiles, w.hist, w.err,
                                                w.stop);
  }
  kmgb::count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  KMGB_CUDA_TRY(excl_scan(w.hist, hist_elems, w.scan_tmp, s, w.stop));
  label_offsets_kernel<<<(k + 1 + 255) / 256, 256, 0, s>>>(w.hist, n, k, w.ntiles, w.label_off,
                                                          w.piece_cnt, w.counts, w.stop); kmgb::count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  KMGB_CUDA_TRY(excl_scan(w.piece_cnt, k + 1, w.scan_tmp, s, w.stop));
  const size_t msmem = sizeof(int) * (size_t)k * kScatterWarps;
  if (msmem <= 96 * 1024) {
    static int multi_attr_k = -1;
    if (msmem > 48 * 1024 && multi_attr_k < k) {
      KMGB_CUDA_TRY(cudaFuncSetAttribute(scatter_multi_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
      multi_attr_k = k;
    }
    scatter_multi_kernel<<<w.ntiles, 32 * kScatterWarps, msmem, s>>>(
        labels, n, k, w.tile_pts, w.ntiles, w.hist, w.sorted, w.stop);
    kmgb::count_launches(1);
  } else if (smem <= 96 * 1024) {
    static int attr_k = -1;
    if (smem > 48 * 1024 && attr_k < k) {
      KMGB_CUDA_TRY(cudaFuncSetAttribute(scatter_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
      attr_k = k;
    }
    scatter_kernel<true><<<w.ntiles, 32, smem, s>>>(labels, n, k, w.tile_pts, w.ntiles, w.hist,
                                                    w.sorted, w.stop); kmgb::count_launches(1);
  } else {
    scatter_kernel<false><<<w.ntiles, 32, 0, s>>>(labels, n, k, w.tile_pts, w.ntiles, w.hist,
                                                  w.sorted, w.stop); kmgb::count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t launch_update(const float* X, const double* qn, const int* labels, float* C,
                          long long ldc, int empty_policy, const UpdateWork& w, double* sse_out,
                          cudaStream_t s) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  const int k = w.k;
  if (w.n <= 0 || k <= 0) return cudaSuccess;
  KMGB_CUDA_TRY(sort_by_label(labels, w, s));
  KMGB_CUDA_TRY(launch_piece_sums_f32(X, w.ldx, qn, w.sorted, w.label_off, w.piece_cnt, k, w.d,
                                     w.part, w.partq, w.stop, w.max_pieces, s));
  const long long fin_warps = (long long)k * ((w.d + 31) / 32);
  finalize_kernel<<<(unsigned)((fin_warps * 32 + 255) / 256), 256, 0, s>>>(
      w.part, qn ? w.partq : nullptr, w.label_off, w.piece_cnt, k, w.d, C, ldc, empty_policy,
      w.sse_k, w.stop); kmgb::count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  if (qn) {
    sse_fixup_kernel<<<(unsigned)((k * 32LL + 255) / 256), 256, 0, s>>>(
        w.sse_k, (w.d + 31) / 32, w.partq, w.label_off, w.piece_cnt, k, w.d, X, w.ldx, w.sorted, C,
        ldc, w.stop);
    kmgb::count_launches(1);
    KMGB_CUDA_TRY(cudaGetLastError());
  }
  if (sse_out) {
    sse_reduce_kernel<<<1, 1024, 0, s>>>(w.sse_k, (int)fin_warps, sse_out, w.stop, w.criterion,
                                         w.sse_prev, w.rel_out, w.iters_done, w.sse_indexed); kmgb::count_launches(1);
    KMGB_CUDA_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

namespace {

// Per-kernel ABI: add this tile's canonical per-center sums to FP64 accumulators.
__global__ void accumulate_kernel(const double* __restrict__ part, const int* __restrict__ label_off,
                                  const int* __restrict__ pstart, int k, int d,
                                  double* __restrict__ acc, int* __restrict__ acc_counts) {
  const int j = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= k) return;
  const int p0 = pstart[j], p1 = pstart[j + 1];
  for (int c = lane; c < d; c += 32) {
    double s = 0.0;
    for (int p = p0; p < p1; ++p) s += part[(size_t)p * d + c];
    acc[(size_t)j * d + c] += s;
  }
  if (lane == 0) acc_counts[j] += label_off[j + 1] - label_off[j];
}

// Host-streamed tiles: add this tile's canonical per-center sums, member counts and sum of
// ||x||^2 to the run's FP64 accumulators (the tile's pieces in piece order, then one addition per
// tile, tiles in order).
__global__ void accumulate_stream_kernel(const double* __restrict__ part,
                                         const double* __restrict__ partq,
                                         const int* __restrict__ label_off,
                                         const int* __restrict__ pstart, int k, int d,
                                         double* __restrict__ accS, int* __restrict__ accN,
                                         double* __restrict__ accQ, const int* stop) {
  if (stopped(stop)) return;
  const int j = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= k) return;
  const int p0 = pstart[j], p1 = pstart[j + 1];
  for (int c = lane; c < d; c += 32) {
    double s = 0.0;
    for (int p = p0; p < p1; ++p) s += part[(size_t)p * d + c];
    accS[(size_t)j * d + c] += s;
  }
  if (lane == 0) {
    double q = 0.0;
    for (int p = p0; p < p1; ++p) q += partq[p];
    accQ[j] += q;
    accN[j] += label_off[j + 1] - label_off[j];
  }
}

// Host-streamed tiles: centers and SSE terms from the run's accumulators, one warp per (center,
// group of 32 dimensions) as finalize_kernel.
__global__ void finalize_stream_kernel(const double* __restrict__ accS, const int* __restrict__ accN,
                                       const double* __restrict__ accQ, int k, int d,
                                       float* __restrict__ C, long long ldc, int empty_policy,
                                       double* __restrict__ sse_k, const int* stop) {
  if (stopped(stop)) return;
  const int groups = (d + 31) / 32;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= (long long)k * groups) return;
  const int j = (int)(wid / groups), g = (int)(wid - (long long)j * groups);
  const int c = g * 32 + lane;
  const long long n = accN[j];
  double sse = 0.0;
  if (c < d) {
    const double s = accS[(size_t)j * d + c];
    float mu;
    if (n > 0) {
      mu = __double2float_rn(__ddiv_rn(s, (double)n));
      const double m = (double)mu;
      sse = fma((double)n * m, m, -2.0 * m * s);
    } else if (empty_policy == 1) {
      mu = C[(size_t)j * ldc + c];
    } else {
      mu = __int_as_float(0x7fc00000);
    }
    C[(size_t)j * ldc + c] = mu;
  }
  for (int o = 16; o > 0; o >>= 1) sse += __shfl_xor_sync(0xffffffffu, sse, o);
  if (lane == 0) sse_k[(size_t)j * groups + g] = (n > 0) ? sse + (g == 0 ? accQ[j] : 0.0) : 0.0;
}

template <typename T>
__global__ void finalize_acc_kernel(const double* __restrict__ acc, const int* __restrict__ acc_counts,
                                    int k, int d, T* __restrict__ centers, int* __restrict__ counts) {
  const long long total = (long long)k * d;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / d);
    const int n = acc_counts[j];
    T v;
    if (n > 0) {
      const double q = __ddiv_rn(acc[e], (double)n);
      v = (T)q;
    } else {
      v = (T)__longlong_as_double(0x7ff8000000000000LL);
    }
    centers[e] = v;
    if (counts && e % d == 0) counts[j] = n;
  }
}

}  // namespace

template <typename T>
cudaError_t launch_tile_accumulate(const T* X, long long ldx, const int* labels, const UpdateWork& w,
                                   double* acc, int* acc_counts, cudaStream_t s) {
  if (w.n <= 0 || w.k <= 0) return cudaSuccess;
  KMGB_CUDA_TRY(sort_by_label(labels, w, s));
  long long warps = w.max_pieces < kmgb::num_sms() * 64LL ? w.max_pieces : kmgb::num_sms() * 64LL;
  piece_sums_kernel<T><<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(
      X, ldx, nullptr, w.sorted, w.label_off, w.piece_cnt, w.k, w.d, w.part, nullptr, w.stop); kmgb::count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  accumulate_kernel<<<(unsigned)(((long long)w.k * 32 + 255) / 256), 256, 0, s>>>(
      w.part, w.label_off, w.piece_cnt, w.k, w.d, acc, acc_counts); kmgb::count_launches(1);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_finalize_acc(const double* acc, const int* acc_counts, int k, int d, T* centers,
                                int* counts, cudaStream_t s) {
  finalize_acc_kernel<T><<<kmgb::num_sms() * 4, 256, 0, s>>>(acc, acc_counts, k, d, centers, counts); kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_stream_accumulate(const float* X, long long ldx, const double* qn,
                                     const int* labels, const UpdateWork& w, double* accS,
                                     int* accN, double* accQ, cudaStream_t s) {
  if (w.n <= 0 || w.k <= 0) return cudaSuccess;
  KMGB_CUDA_TRY(sort_by_label(labels, w, s));
  KMGB_CUDA_TRY(launch_piece_sums_f32(X, w.ldx, qn, w.sorted, w.label_off, w.piece_cnt, w.k, w.d,
                                     w.part, w.partq, w.stop, w.max_pieces, s));
  accumulate_stream_kernel<<<(unsigned)(((long long)w.k * 32 + 255) / 256), 256, 0, s>>>(
      w.part, w.partq, w.label_off, w.piece_cnt, w.k, w.d, accS, accN, accQ, w.stop);
  kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_stream_finalize(const double* accS, const int* accN, const double* accQ,
                                   float* C, long long ldc, int empty_policy, const UpdateWork& w,
                                   double* sse_out, cudaStream_t s) {
  const int k = w.k;
  const long long fin_warps = (long long)k * ((w.d + 31) / 32);
  finalize_stream_kernel<<<(unsigned)((fin_warps * 32 + 255) / 256), 256, 0, s>>>(
      accS, accN, accQ, k, w.d, C, ldc, empty_policy, w.sse_k, w.stop);
  kmgb::count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  sse_reduce_kernel<<<1, 1024, 0, s>>>(w.sse_k, (int)fin_warps, sse_out, w.stop, w.criterion,
                                       w.sse_prev, w.rel_out, w.iters_done, w.sse_indexed);
  kmgb::count_launches(1);
  return cudaGetLastError();
}

template cudaError_t launch_tile_accumulate<float>(const float*, long long, const int*,
                                                   const UpdateWork&, double*, int*, cudaStream_t);
template cudaError_t launch_tile_accumulate<double>(const double*, long long, const int*,
                                                    const UpdateWork&, double*, int*, cudaStream_t);
template cudaError_t launch_finalize_acc<float>(const double*, const int*, int, int, float*, int*,
                                                cudaStream_t);
template cudaError_t launch_finalize_acc<double>(const double*, const int*, int, int, double*, int*,
                                                 cudaStream_t);

// ---------------------------------------------------------------------------------------
// Batched Lloyd: many problems of one dimension share X (problem p: rows row_beg[p] ..
// row_end[p]-1) and one center matrix (problem p: centers c_off[p] .. c_off[p]+k[p]-1), labels
// being global center indices. The counting sort uses tiles of tile_pts rows that never cross a
// problem; problem p's counters are hist[hoff[p] + j * ntiles[p] + t] (center j, tile t), so the
// exclusive scan of hist in memory order is the stable order by global label, i.e. problem by
// problem, each sorted exactly as a single problem would be. Piece sums and the finalize step
// are the single-problem kernels over all K centers.
namespace {

__global__ void hist_batched_kernel(const int* __restrict__ labels, BatchUpdate b,
                                    int* __restrict__ hist, int* err) {
  const long long st = blockIdx.x;
  const int prob = b.stile_prob[st];
  const int tl = b.stile_local[st];
  const long long i0 = b.row_beg[prob] + (long long)tl * b.tile_pts;
  const long long i1 = min(b.row_end[prob], i0 + b.tile_pts);
  const int cb = b.c_off[prob], kp = b.k[prob], nt = b.ntiles[prob];
  int* h = hist + b.hoff[prob];
  const int lane = threadIdx.x & 31;
  const int nbits = label_bits(kp);
  for (long long base = i0; base < i1; base += blockDim.x) {
    const long long i = base + threadIdx.x;
    int l = -1;
    if (i < i1) {
      l = labels[i] - cb;
      if (l < 0 || l >= kp) {
        set_error(err, KMGB_DEV_BAD_LABEL);
        l = -1;
      }
    }
    const unsigned peers = warp_peers(l, nbits);
    const int leader = __ffs(peers) - 1;
    if (l >= 0 && lane == leader) atomicAdd(&h[(size_t)l * nt + tl], __popc(peers));
  }
}

// label_off[g] = first sorted position of global center g (label_off[K] = rows), piece counts
// and member counts, from the scanned counters.
__global__ void label_offsets_batched_kernel(const int* __restrict__ hist, BatchUpdate b,
                                             int* __restrict__ label_off, int* __restrict__ piece_cnt,
                                             long long* __restrict__ counts) {
  const int gc = blockIdx.x * blockDim.x + threadIdx.x;
  if (gc > b.K) return;
  auto start = [&](int c) -> int {
    if (c >= b.K) return (int)b.n_valid;
    const int prob = b.cprob[c];
    return hist[b.hoff[prob] + (size_t)(c - b.c_off[prob]) * b.ntiles[prob]];
  };
  if (gc == b.K) {
    label_off[b.K] = (int)b.n_valid;
    piece_cnt[b.K] = 0;
    return;
  }
  const int a0 = start(gc), a1 = start(gc + 1);
  label_off[gc] = a0;
  piece_cnt[gc] = (a1 - a0 + kSumPiece - 1) / kSumPiece;
  if (counts) counts[gc] = a1 - a0;
}

// One warp per sort tile. SMEM: the tile's k counters live in shared memory (k <= smem_k).
template <bool SMEM>
__global__ void scatter_batched_kernel(const int* __restrict__ labels, BatchUpdate b, int* pos,
                                       int* __restrict__ sorted) {
  extern __shared__ int cnt_s[];
  const long long st = blockIdx.x;
  const int prob = b.stile_prob[st];
  const int tl = b.stile_local[st];
  const long long i0 = b.row_beg[prob] + (long long)tl * b.tile_pts;
  const long long i1 = min(b.row_end[prob], i0 + b.tile_pts);
  const int cb = b.c_off[prob], kp = b.k[prob], nt = b.ntiles[prob];
  volatile int* vpos = pos + b.hoff[prob];
  const int lane = threadIdx.x;
  if (SMEM) {
    for (int j = lane; j < kp; j += 32) cnt_s[j] = vpos[(size_t)j * nt + tl];
    __syncwarp();
  }
  const int nbits = label_bits(kp);
  int lnext = (i0 + lane < i1) ? labels[i0 + lane] : 0;
  for (long long base = i0; base < i1; base += 32) {
    const long long i = base + lane;
    int l = -1;
    if (i < i1) {
      l = lnext - cb;
      if (l < 0 || l >= kp) l = -1;
    }
    if (base + 32 + lane < i1) lnext = labels[base + 32 + lane];  // next batch in flight
    const unsigned peers = warp_peers(l, nbits);
    const int leader = __ffs(peers) - 1;
    const int rank = __popc(peers & lanemask_lt());
    int bs = 0;
    if (l >= 0 && lane == leader) bs = SMEM ? cnt_s[l] : vpos[(size_t)l * nt + tl];
    bs = __shfl_sync(0xffffffffu, bs, leader);
    if (l >= 0) sorted[bs + rank] = (int)i;
    if (l >= 0 && lane == leader) {
      if (SMEM) cnt_s[l] = bs + __popc(peers);
      else vpos[(size_t)l * nt + tl] = bs + __popc(peers);
    }
    __syncwarp();
  }
}

// One warp per problem: SSE = sum of its centers' terms; the reference's stop rule per problem
// (kmeans.cpp:1194-1237). A problem that has stopped keeps its history; its centers are
// recomputed from unchanged labels, which reproduces them bit for bit.
// The problem's SSE history slot is its own count of recorded iterations (a stopped problem
// records nothing more), so every iteration issues the same launch: a CUDA graph replays it.
__global__ void sse_batched_kernel(const double* __restrict__ sse_k, int groups, BatchUpdate b) {
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= b.P) return;
  const int prob = (int)wid;
  if (b.done[prob]) return;
  const long long e0 = (long long)b.c_off[prob] * groups;
  const long long e1 = e0 + (long long)b.k[prob] * groups;
  double s = 0.0;
  for (long long e = e0 + lane; e < e1; e += 32) s += sse_k[e];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    const double rel = fabs(s - b.sse_prev[prob]) / fabs(s);
    b.sse_prev[prob] = s;
    b.rel[prob] = rel;
    const int iter = b.iters[prob];
    if (iter < b.max_iters) b.sse_hist[(size_t)prob * b.max_iters + iter] = s;
    b.iters[prob] = iter + 1;
    if (!(rel > b.criterion)) b.done[prob] = 1;
  }
}

}  // namespace

cudaError_t launch_update_batched(const float* X, long long ldx, int d, const double* qn,
                                  const int* labels, float* C, long long ldc, int empty_policy,
                                  const UpdateWork& w, const BatchUpdate& b, cudaStream_t s) {
  if (b.P <= 0 || b.K <= 0 || b.n_valid <= 0) return cudaSuccess;
  KMGB_CUDA_TRY(cudaMemsetAsync(w.hist, 0, sizeof(int) * b.hist_elems, s));
  hist_batched_kernel<<<(unsigned)b.stiles, 256, 0, s>>>(labels, b, w.hist, w.err);
  count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  KMGB_CUDA_TRY(excl_scan(w.hist, b.hist_elems, w.scan_tmp, s, nullptr));
  label_offsets_batched_kernel<<<(b.K + 1 + 255) / 256, 256, 0, s>>>(w.hist, b, w.label_off,
                                                                    w.piece_cnt, w.counts);
  count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  KMGB_CUDA_TRY(excl_scan(w.piece_cnt, b.K + 1, w.scan_tmp, s, nullptr));
  if (b.kmax <= 12288)
    scatter_batched_kernel<true><<<(unsigned)b.stiles, 32, sizeof(int) * (size_t)b.kmax, s>>>(
        labels, b, w.hist, w.sorted);
  else
    scatter_batched_kernel<false><<<(unsigned)b.stiles, 32, 0, s>>>(labels, b, w.hist, w.sorted);
  count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  KMGB_CUDA_TRY(launch_piece_sums_f32(X, ldx, qn, w.sorted, w.label_off, w.piece_cnt, b.K, d,
                                     w.part, w.partq, nullptr, w.max_pieces, s));
  const int groups = (d + 31) / 32;
  const long long fin_warps = (long long)b.K * groups;
  finalize_kernel<<<(unsigned)((fin_warps * 32 + 255) / 256), 256, 0, s>>>(
      w.part, w.partq, w.label_off, w.piece_cnt, b.K, d, C, ldc, empty_policy, w.sse_k, nullptr);
  count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  sse_fixup_kernel<<<(unsigned)((b.K * 32LL + 255) / 256), 256, 0, s>>>(
      w.sse_k, groups, w.partq, w.label_off, w.piece_cnt, b.K, d, X, ldx, w.sorted, C, ldc,
      nullptr);
  count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  sse_batched_kernel<<<(unsigned)((b.P * 32LL + 255) / 256), 256, 0, s>>>(w.sse_k, groups, b);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace kmgb
