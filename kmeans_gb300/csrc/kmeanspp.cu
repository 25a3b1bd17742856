// k-means++ initialisation (the reference declares initAlgorithm and numRetries,
// main/cpp/kmeans.hpp:94-95, kmeans.cpp:29, but implements only its shuffle-and-pick init).
//
// Centers are drawn one at a time, each with probability proportional to D^2, the squared
// distance of a point to its nearest already-chosen center. The draws are reproducible bit for
// bit on the data type T (float or double):
//   * D^2 is computed in T: lane l of a warp accumulates dimensions l, l+32, ... with
//     fma((x-c), (x-c), s) in increasing order, then an xor butterfly over the 32 lanes
//     (s += shfl_xor(s, o), o = 16, 8, 4, 2, 1; every lane ends with the same sum);
//     D^2 = fmin(D^2, distance to the newest center).
//   * The sampling weight of a point is q = uint32 truncation (saturating, NaN -> 0) of
//     D^2 * (2^31 / M) in T, M the largest D^2 after the update (so q <= 2^31). Sums of q are
//     exact 64-bit integers: the order of the parallel sums does not matter.
//   * Draw r takes u = splitmix64(splitmix64(seed) + r) >> 11 (53 bits) and picks the point whose
//     interval [prefix, prefix + q) of the running sum of q holds (u * total) >> 53 (128-bit
//     product). Draw 0, and any draw whose total weight is 0, picks point (u * n) >> 53.
// Per draw: one pass over X (D^2 update and maximum), one over D^2 (weights and their sums per
// 1024 points) and one single-block pass (scan of the block sums, the draw, the pick). D^2 is
// n elements of T; X is read once per draw, which bounds the whole initialisation by HBM.
#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

constexpr int KPP_BLOCK = 1024;  // points per weight-sum block (= threads of the pick kernel)
constexpr int KPP_THREADS = 256;

__host__ __device__ inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ inline uint64_t draw53(uint64_t seed, uint64_t round) {
  return splitmix64(splitmix64(seed) + round) >> 11;
}

__device__ __forceinline__ float kpp_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double kpp_fma(double a, double b, double c) { return __fma_rn(a, b, c); }

// Largest D^2 as an order-preserving unsigned key (D^2 >= 0 or NaN; NaN never raises it).
__device__ __forceinline__ unsigned long long kpp_key(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned long long kpp_key(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
template <typename T>
__device__ __forceinline__ T kpp_unkey(unsigned long long k);
template <>
__device__ __forceinline__ float kpp_unkey<float>(unsigned long long k) {
  return __uint_as_float((unsigned int)k);
}
template <>
__device__ __forceinline__ double kpp_unkey<double>(unsigned long long k) {
  return __longlong_as_double((long long)k);
}

template <typename T>
__device__ __forceinline__ T kpp_scale(unsigned long long mkey) {
  const T m = kpp_unkey<T>(mkey);
  return m > T(0) ? T(2147483648.0) / m : T(0);  // IEEE division in T
}

// Saturating truncation to uint32 (cvt.rzi.u32: NaN and negatives -> 0).
__device__ __forceinline__ unsigned int kpp_weight(float v, float scale) {
  return __float2uint_rz(__fmul_rn(v, scale));
}
__device__ __forceinline__ unsigned int kpp_weight(double v, double scale) {
  return __double2uint_rz(__dmul_rn(v, scale));
}

// Exclusive scan of one value per thread over a 1024-thread block; *total gets the sum.
__device__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long* warp_sh,
                                                   unsigned long long* total_sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sh[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = warp_sh[lane];
    unsigned long long wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    warp_sh[lane] = wi - w;
    if (lane == 31) *total_sh = wi;
  }
  __syncthreads();
  const unsigned long long r = warp_sh[warp] + incl - v;
  __syncthreads();  // warp_sh may be reused by the caller's next scan
  return r;
}

// D^2 of the points of one 1024-point block against the newest center (row *pick); the block's
// largest D^2 raises *max_key. A warp takes KPP_ROWS rows at a time, their loads interleaved so
// that each lane keeps 4 x KPP_ROWS loads in flight; every row keeps its own lane-partial fma
// chain in increasing dimension order, so the sums are those of one row at a time.
constexpr int KPP_ROWS = 4;

template <typename T>
__global__ void __launch_bounds__(KPP_THREADS)
kpp_update_kernel(const T* __restrict__ X, long long ldx, long long n, int d,
                  const int* __restrict__ pick, T* __restrict__ d2, int first,
                  unsigned long long* __restrict__ max_key) {
  __shared__ unsigned long long wmax[KPP_THREADS / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const T* c = X + (size_t)(*pick) * ldx;
  T mx = T(0);
  const long long p0 = (long long)blockIdx.x * KPP_BLOCK;
  const long long pend = min(n, p0 + KPP_BLOCK);
  for (long long pr = p0 + (long long)warp * KPP_ROWS; pr < pend;
       pr += (long long)(KPP_THREADS / 32) * KPP_ROWS) {
    const T* x[KPP_ROWS];
    T s[KPP_ROWS];
#pragma unroll
    for (int r = 0; r < KPP_ROWS; ++r) {
      // rows past the end re-read the last valid row (never stored)
      x[r] = X + (size_t)min(pr + r, pend - 1) * ldx;
      s[r] = T(0);
    }
#pragma unroll 4
    for (int t = lane; t < d; t += 32) {
      const T cv = __ldg(c + t);
#pragma unroll
      for (int r = 0; r < KPP_ROWS; ++r) {
        const T u = __ldg(x[r] + t) - cv;
        s[r] = kpp_fma(u, u, s[r]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int r = 0; r < KPP_ROWS; ++r) s[r] = s[r] + __shfl_xor_sync(0xffffffffu, s[r], o);
    }
#pragma unroll
    for (int r = 0; r < KPP_ROWS; ++r) {
      const long long pt = pr + r;
      if (pt < pend) {
        const T v = first ? s[r] : fmin(d2[pt], s[r]);
        if (lane == 0) d2[pt] = v;
        mx = fmax(mx, v);
      }
    }
  }
  if (lane == 0) wmax[warp] = kpp_key(mx);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0;
    for (int w = 0; w < KPP_THREADS / 32; ++w) m = max(m, wmax[w]);
    atomicMax(max_key, m);
  }
}

// The same D^2 update with X staged through shared memory: a producer warp streams chunks of
// `rows_per_stage` contiguous rows (and their old D^2 values) with cp.async.bulk into a ring of
// `stages` buffers, so the bytes in flight per SM are the ring's, not the registers'; 8
// consumer warps compute each row exactly as kpp_update_kernel does (lane l: dims l, l+32, ...
// from shared memory, fma chain, xor butterfly). Needs 16-byte aligned rows (ldx * sizeof(T) a
// multiple of 16, X 16-byte aligned) and d2 padded to a multiple of 4 rows. Every wait is
// bounded; on a timeout the CTA records KMGB_DEV_TIMEOUT_FULL/EMPTY in *err, waits (bounded)
// for its copies in flight and returns.
constexpr int KPP_CONSUMERS = 8;
constexpr int KPP_BULK_THREADS = (KPP_CONSUMERS + 1) * 32;
constexpr int KPP_MAX_STAGES = 8;

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
      : "memory");
}

template <typename T>
__global__ void __launch_bounds__(KPP_BULK_THREADS)
kpp_update_bulk_kernel(const T* __restrict__ X, long long ldx, long long n, int d,
                       const int* __restrict__ pick, T* __restrict__ d2, int first,
                       unsigned long long* __restrict__ max_key, int rows_per_stage, int stages,
                       int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char kpp_smem[];
  __shared__ __align__(8) uint64_t full_bar[KPP_MAX_STAGES], empty_bar[KPP_MAX_STAGES];
  __shared__ unsigned long long wmax[KPP_CONSUMERS];
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long row_elems = ldx;
  const uint32_t row_bytes = (uint32_t)(ldx * (long long)sizeof(T));
  const uint32_t xstage_bytes = row_bytes * (uint32_t)rows_per_stage;
  T* cs = reinterpret_cast<T*>(kpp_smem);                              // the new center
  unsigned char* ring = kpp_smem + ((d * sizeof(T) + 127) / 128) * 128;  // X stages, then D^2
  T* dring = reinterpret_cast<T*>(ring + (size_t)stages * xstage_bytes);
  const long long nchunks = (n + rows_per_stage - 1) / rows_per_stage;

  const T* c = X + (size_t)(*pick) * ldx;
  for (int t = threadIdx.x; t < d; t += blockDim.x) cs[t] = c[t];
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int i = 0; i < stages; ++i) {
      mbar_init(smem_u32(&full_bar[i]), 1);
      mbar_init(smem_u32(&empty_bar[i]), KPP_CONSUMERS);
    }
    fence_mbar_init();
  }
  __syncthreads();

  if (warp == KPP_CONSUMERS) {  // producer
    if (lane == 0) {
      long long it = 0;
      for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x, ++it) {
        const int sidx = (int)(it % stages);
        if (it >= stages &&
            !mbar_wait(smem_u32(&empty_bar[sidx]), (uint32_t)(((it / stages) - 1) & 1),
                       &abort_flag, err, KMGB_DEV_TIMEOUT_EMPTY))
          break;
        const long long r0 = ch * rows_per_stage;
        const int rows = (int)min((long long)rows_per_stage, n - r0);
        const uint32_t xb = row_bytes * (uint32_t)rows;
        // D^2 slice rounded up to 16 bytes (d2 holds a multiple of 4 rows)
        const uint32_t db = first ? 0u : (uint32_t)((((rows + 3) & ~3)) * sizeof(T));
        const uint32_t bar = smem_u32(&full_bar[sidx]);
        mbar_arrive_expect_tx(bar, xb + db);
        bulk_g2s(smem_u32(ring + (size_t)sidx * xstage_bytes), X + (size_t)r0 * row_elems, xb, bar);
        if (db) bulk_g2s(smem_u32(dring + (size_t)sidx * rows_per_stage), d2 + r0, db, bar);
      }
      // copies still in flight (only after an abort) must land before the CTA exits
      const long long issued = it;
      for (long long j = issued - 1; j >= 0 && j >= issued - stages; --j) {
        const uint32_t bar = smem_u32(&full_bar[j % stages]);
        const uint32_t par = (uint32_t)((j / stages) & 1);
        const long long t0 = clock64();
        while (!mbar_try_wait(bar, par) &&
               (unsigned long long)(clock64() - t0) < KMGB_WAIT_CYCLES) {
        }
      }
    }
    __syncwarp();
  } else {  // consumers
    T mx = T(0);
    long long it = 0;
    for (long long ch = blockIdx.x; ch < nchunks; ch += gridDim.x, ++it) {
      const int sidx = (int)(it % stages);
      if (!mbar_wait(smem_u32(&full_bar[sidx]), (uint32_t)((it / stages) & 1), &abort_flag, err,
                     KMGB_DEV_TIMEOUT_FULL))
        break;
      const long long r0 = ch * rows_per_stage;
      const int rows = (int)min((long long)rows_per_stage, n - r0);
      const T* xs = reinterpret_cast<const T*>(ring + (size_t)sidx * xstage_bytes);
      const T* ds = dring + (size_t)sidx * rows_per_stage;
      for (int g = warp * KPP_ROWS; g < rows; g += KPP_CONSUMERS * KPP_ROWS) {
        T sv[KPP_ROWS];
#pragma unroll
        for (int r = 0; r < KPP_ROWS; ++r) sv[r] = T(0);
        const T* xr[KPP_ROWS];
#pragma unroll
        for (int r = 0; r < KPP_ROWS; ++r) xr[r] = xs + (size_t)min(g + r, rows - 1) * row_elems;
#pragma unroll 4
        for (int t = lane; t < d; t += 32) {
          const T cv = cs[t];
#pragma unroll
          for (int r = 0; r < KPP_ROWS; ++r) {
            const T u = xr[r][t] - cv;
            sv[r] = kpp_fma(u, u, sv[r]);
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
          for (int r = 0; r < KPP_ROWS; ++r) sv[r] = sv[r] + __shfl_xor_sync(0xffffffffu, sv[r], o);
        }
#pragma unroll
        for (int r = 0; r < KPP_ROWS; ++r) {
          if (g + r < rows) {
            const T v = first ? sv[r] : fmin(ds[g + r], sv[r]);
            if (lane == 0) d2[r0 + g + r] = v;
            mx = fmax(mx, v);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&empty_bar[sidx]));
    }
    if (lane == 0) wmax[warp] = kpp_key(mx);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = 0;
    for (int w = 0; w < KPP_CONSUMERS; ++w) m = max(m, wmax[w]);
    atomicMax(max_key, m);
  }
}

// Weights q of one 1024-point block and their exact sum.
template <typename T>
__global__ void __launch_bounds__(KPP_THREADS)
kpp_weight_kernel(const T* __restrict__ d2, long long n, const unsigned long long* __restrict__ max_key,
                  unsigned long long* __restrict__ blocksum) {
  __shared__ unsigned long long part[KPP_THREADS / 32];
  const T scale = kpp_scale<T>(*max_key);
  unsigned long long s = 0;
  const long long p0 = (long long)blockIdx.x * KPP_BLOCK;
  for (int i = threadIdx.x; i < KPP_BLOCK; i += KPP_THREADS) {
    const long long pt = p0 + i;
    if (pt < n) s += kpp_weight(d2[pt], scale);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < KPP_THREADS / 32; ++w) t += part[w];
    blocksum[blockIdx.x] = t;
  }
}

// The draw of round `round`: scan of the block sums, the block holding the target, then the
// point inside it (1024 threads, one point each). Writes *pick and picks[round].
template <typename T>
__global__ void __launch_bounds__(KPP_BLOCK)
kpp_pick_kernel(long long n, const T* __restrict__ d2, const unsigned long long* __restrict__ blocksum,
                long long nblocks, const unsigned long long* __restrict__ max_key,
                unsigned long long* __restrict__ next_max_key, unsigned long long seed, int round,
                int* __restrict__ pick, int* __restrict__ picks) {
  __shared__ unsigned long long warp_sh[32];
  __shared__ unsigned long long total_sh, off_sh, tot2_sh;
  __shared__ long long block_sh, chosen_sh;
  const int tid = threadIdx.x;
  if (tid == 0) {
    block_sh = -1;
    chosen_sh = -1;
  }
  // each thread sums a contiguous run of blocks
  const long long per = (nblocks + KPP_BLOCK - 1) / KPP_BLOCK;
  const long long b0 = (long long)tid * per, b1 = min(nblocks, b0 + per);
  unsigned long long s = 0;
  for (long long b = b0; b < b1; ++b) s += blocksum[b];
  unsigned long long off = block_exclusive_scan(s, warp_sh, &total_sh);
  const unsigned long long total = total_sh;
  const uint64_t u = draw53(seed, (uint64_t)round);
  const unsigned long long uniform = __umul64hi(u << 11, (unsigned long long)n);  // (u*n) >> 53
  if (tid == 0) *next_max_key = 0;  // the next draw's maximum (not read by this draw)
  if (total == 0) {
    if (tid == 0) {
      *pick = (int)uniform;
      picks[round] = (int)uniform;
    }
    return;
  }
  const unsigned long long target = __umul64hi(u << 11, total);  // (u * total) >> 53 < total
  if (off <= target && target < off + s) {  // exactly one thread's run holds the target
    for (long long b = b0; b < b1; ++b) {
      const unsigned long long nx = off + blocksum[b];
      if (nx > target) {
        block_sh = b;
        off_sh = off;
        break;
      }
      off = nx;
    }
  }
  __syncthreads();
  const long long b = block_sh;  // >= 0: the runs partition [0, total)
  const T scale = kpp_scale<T>(*max_key);
  const long long pt = b * (long long)KPP_BLOCK + tid;
  const unsigned long long q = (b >= 0 && pt < n) ? kpp_weight(d2[pt], scale) : 0ull;
  const unsigned long long ex = off_sh + block_exclusive_scan(q, warp_sh, &tot2_sh);
  if (q > 0 && ex <= target && target < ex + q) chosen_sh = pt;
  __syncthreads();
  if (tid == 0) {
    const long long c = chosen_sh >= 0 ? chosen_sh : (long long)uniform;
    *pick = (int)c;
    picks[round] = (int)c;
  }
}

template <typename T>
__global__ void kpp_gather_kernel(const T* __restrict__ X, long long ldx, int d,
                                  const int* __restrict__ picks, int k, T* __restrict__ C,
                                  long long ldc) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < (long long)k * d;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / d), t = (int)(e - (long long)j * d);
    C[(size_t)j * ldc + t] = X[(size_t)picks[j] * ldx + t];
  }
}

// Ring geometry of kpp_update_bulk_kernel for rows of `row_bytes`: rows per stage (a multiple
// of 4, about 16 KB of rows) and stages (2..8) within a shared-memory budget that leaves room for
// two CTAs per SM. Returns false when the rows are too wide (the register kernel is used then).
constexpr size_t KPP_SMEM_BUDGET = 100 * 1024;

bool kpp_bulk_plan(long long row_bytes, int elem, int d, int* rows_per_stage, int* stages,
                   size_t* smem) {
  long long rps = (16384 / row_bytes) & ~3LL;
  if (rps < 4) rps = 4;
  const long long center = ((long long)d * elem + 127) / 128 * 128;
  const long long per_stage = rps * row_bytes + rps * elem;
  long long st = ((long long)KPP_SMEM_BUDGET - center) / per_stage;
  if (st > KPP_MAX_STAGES) st = KPP_MAX_STAGES;
  if (st < 2) return false;
  *rows_per_stage = (int)rps;
  *stages = (int)st;
  *smem = (size_t)(center + st * per_stage);
  return true;
}

template <typename T>
cudaError_t kmeanspp_impl(const T* X, long long ldx, long long n, int d, int k,
                          unsigned long long seed, T* C, long long ldc, int* picks, T* d2,
                          unsigned long long* blocksum, unsigned long long* scalars, int* err,
                          cudaStream_t s) {
  if (n <= 0 || d <= 0 || k <= 0 || k > n || n > 0x7fffffffLL || ldx < d || ldc < d)
    return cudaErrorInvalidValue;
  const long long nb = (n + KPP_BLOCK - 1) / KPP_BLOCK;
  const long long row_bytes = ldx * (long long)sizeof(T);
  int rps = 0, stages = 0;
  size_t smem = 0;
  const bool bulk = (row_bytes % 16) == 0 && (reinterpret_cast<uintptr_t>(X) % 16) == 0 &&
                    (reinterpret_cast<uintptr_t>(d2) % 16) == 0 &&
                    kpp_bulk_plan(row_bytes, (int)sizeof(T), d, &rps, &stages, &smem);
  int grid = 0;
  if (bulk) {
    KMGB_CUDA_TRY(cudaFuncSetAttribute(kpp_update_bulk_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, per_sm = 0;
    KMGB_CUDA_TRY(cudaGetDevice(&dev));
    KMGB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    KMGB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, kpp_update_bulk_kernel<T>, KPP_BULK_THREADS, smem));
    const long long chunks = (n + rps - 1) / rps;
    grid = (int)min((long long)sms * max(per_sm, 1), chunks);
  }
  // scalars: [0], [1] the maxima of alternate draws (the pick kernel of draw r clears draw
  // r+1's), [2] the newest center's row
  unsigned long long* mx = scalars;
  int* pick = reinterpret_cast<int*>(scalars + 2);
  // draw 0: zero total weight, so uniform
  KMGB_CUDA_TRY(cudaMemsetAsync(blocksum, 0, sizeof(unsigned long long) * nb, s));
  KMGB_CUDA_TRY(cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s));
  kpp_pick_kernel<T><<<1, KPP_BLOCK, 0, s>>>(n, d2, blocksum, nb, mx, mx + 1, seed, 0, pick, picks);
  count_launches(1);
  for (int r = 1; r < k; ++r) {
    unsigned long long* m = mx + (r & 1);
    if (bulk)
      kpp_update_bulk_kernel<T><<<grid, KPP_BULK_THREADS, smem, s>>>(X, ldx, n, d, pick, d2, r == 1,
                                                                     m, rps, stages, err);
    else
      kpp_update_kernel<T><<<(unsigned)nb, KPP_THREADS, 0, s>>>(X, ldx, n, d, pick, d2, r == 1, m);
    kpp_weight_kernel<T><<<(unsigned)nb, KPP_THREADS, 0, s>>>(d2, n, m, blocksum);
    kpp_pick_kernel<T><<<1, KPP_BLOCK, 0, s>>>(n, d2, blocksum, nb, m, mx + ((r + 1) & 1), seed, r,
                                               pick, picks);
    count_launches(3);
  }
  kpp_gather_kernel<T><<<kmgb::num_sms() * 4, 256, 0, s>>>(X, ldx, d, picks, k, C, ldc);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

long long kmeanspp_blocks(long long n) { return (n + KPP_BLOCK - 1) / KPP_BLOCK; }
long long kmeanspp_d2_elems(long long n) { return (n + 3) / 4 * 4; }

cudaError_t launch_kmeanspp(const float* X, long long ldx, long long n, int d, int k,
                            unsigned long long seed, float* C, long long ldc, int* picks,
                            float* d2, unsigned long long* blocksum, unsigned long long* scalars,
                            int* err, cudaStream_t s) {
  return kmeanspp_impl<float>(X, ldx, n, d, k, seed, C, ldc, picks, d2, blocksum, scalars, err, s);
}

cudaError_t launch_kmeanspp(const double* X, long long ldx, long long n, int d, int k,
                            unsigned long long seed, double* C, long long ldc, int* picks,
                            double* d2, unsigned long long* blocksum, unsigned long long* scalars,
                            int* err, cudaStream_t s) {
  return kmeanspp_impl<double>(X, ldx, n, d, k, seed, C, ldc, picks, d2, blocksum, scalars, err,
                               s);
}

}  // namespace kmgb
