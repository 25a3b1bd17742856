// computeKmeansD: the reference's double-precision driver entry (main/cpp/kmeans.cpp:1364-1409).
//
// The reference's FP64 custom assignment is broken (its partial reduction for double2 is an
// empty function, main/cuda/reduction.hcu:7-11, so every label becomes 0); only its cuBLAS path
// (cublasDgemm + rowTransformMinimumD, kmeans.cpp:958-993) defines FP64 behaviour. This path
// computes what that one intends, exactly: label = FP64 arg-min of sum_d (x_d - c_d)^2 (lowest
// index on ties), centers = canonical FP64 sums / counts, SSE in FP64 against the new centers.
// FP64 throughput on GB300 is low (about 1.25 TFLOP/s), so this is the correctness path, not a
// fast one; every kernel is plain SIMT.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <future>
#include <random>
#include <string>
#include <vector>

#include "../../include/kmeans_gb300.h"
#include "common.cuh"
#include "kernels.h"

using namespace kmgb;

namespace {

// CT[t][j] = C[j][t]
__global__ void transpose_d_kernel(const double* __restrict__ C, int k, int d, double* __restrict__ CT) {
  const long long total = (long long)k * d;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / d), t = (int)(e % d);
    CT[(size_t)t * k + j] = C[e];
  }
}

// One warp per point, lanes over centers (coalesced reads of CT); exact FP64 direct distance.
// list (nullable): only the points list[0 .. *count) (the tensor pass's uncertified points).
__global__ void assign_d_kernel(const double* __restrict__ X, long long n, int d,
                                const double* __restrict__ CT, int k, int* __restrict__ labels,
                                const int* __restrict__ list = nullptr,
                                const int* __restrict__ count = nullptr) {
  extern __shared__ double xs_all[];
  const int warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* xs = xs_all + (size_t)w * d;
  const long long todo = list ? (long long)*count : n;
  for (long long slot = (long long)blockIdx.x * warps + w; slot < todo;
       slot += (long long)gridDim.x * warps) {
    const long long i = list ? (long long)list[slot] : slot;
    for (int t = lane; t < d; t += 32) xs[t] = X[(size_t)i * d + t];
    __syncwarp();
    double best = INFINITY;
    int bi = -1;
    for (int j = lane; j < k; j += 32) {
      double s = 0.0;
      for (int t = 0; t < d; ++t) {
        const double u = xs[t] - CT[(size_t)t * k + j];
        s = fma(u, u, s);
      }
      if (s < best) {
        best = s;
        bi = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      const bool take = (ob < best) || (ob == best && (unsigned)oi < (unsigned)bi);
      best = take ? ob : best;
      bi = take ? oi : bi;
    }
    if (lane == 0) labels[i] = bi < 0 ? 0 : bi;
    __syncwarp();
  }
}

// out[r][c] = (float)in[r][c] (round to nearest) for c < d, 0 for d <= c < ldo.
__global__ void d2f_kernel(const double* __restrict__ in, long long rows, int d,
                           float* __restrict__ out, long long ldo) {
  const long long total = rows * ldo;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long r = e / ldo, c = e - r * ldo;
    out[e] = c < d ? __double2float_rn(in[(size_t)r * d + c]) : 0.0f;
  }
}

__global__ void sse_d_partial_kernel(const double* __restrict__ X, long long n, int d,
                                     const int* __restrict__ lab, const double* __restrict__ C,
                                     double* __restrict__ partial) {
  __shared__ double red[8];
  const int warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double acc = 0.0;
  for (long long i = (long long)blockIdx.x * warps + w; i < n; i += (long long)gridDim.x * warps) {
    const int l = lab[i];
    double s = 0.0;
    for (int t = lane; t < d; t += 32) {
      const double u = X[(size_t)i * d + t] - C[(size_t)l * d + t];
      s = fma(u, u, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    acc += s;
  }
  if (lane == 0) red[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < warps; ++i) t += red[i];
    partial[blockIdx.x] = t;
  }
}

__global__ void sse_d_final_kernel(const double* __restrict__ partial, int nb, double* out) {
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < nb; ++i) t += partial[i];
    *out = t;
  }
}

__global__ void gather_d_kernel(const double* __restrict__ X, int d, const int* __restrict__ perm,
                                long long m, long long start, long long m_mb, double* __restrict__ Xw) {
  const long long total = m_mb * d;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long r = e / d;
    long long pos = start + r;
    if (pos >= m) pos -= m;
    Xw[e] = X[(size_t)perm[pos] * d + (e % d)];
  }
}

struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t count) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

#define KD_TRY(expr, code)                \
  do {                                    \
    if ((expr) != cudaSuccess) return (code); \
  } while (0)

// One FP64 run. kpp_seed < 0: the reference initialisation; else k-means++ with that seed (on the
// device, from the uploaded data). result receives the initial then the final centers (D x K);
// *final_sse the SSE of the last iteration (NaN when none ran).
kmeansErrorStatus run_d(const double* data, int m, int n, int k, double criterion, int maxIters,
                        double* result, double fraction, long long kpp_seed, double* final_sse) {
  *final_sse = std::nan("");
  const bool mini = fraction < 1.0;
  const long long m_mb = mini ? (long long)(int)((float)fraction * (float)m) : m;
  if (m_mb <= 0) return KMEANS_ERROR_TILING;
  // reference initialisation on the host (kmeans.cpp:554-564, 876-888): the shuffle is
  // sequential and independent of the data, so it runs on a host thread while the data set is
  // allocated and uploaded
  struct RefInit {
    std::vector<int> perm, picks;
    bool ok = true;
  };
  auto ref_task = [m, k, kpp_seed] {
    RefInit r;
    reference_perm(m, r.perm);
    if (kpp_seed < 0) r.ok = reference_picks(m, k, r.picks);
    return r;
  };
  std::future<RefInit> ref;
  try {
    ref = std::async(std::launch::async, ref_task);
  } catch (...) {  // no thread to be had: run it when the result is asked for
    ref = std::async(std::launch::deferred, ref_task);
  }

  DevBufs B;
  double *X = nullptr, *Xw = nullptr, *Cd = nullptr, *CT = nullptr, *acc = nullptr, *part = nullptr,
         *sse = nullptr;
  int *lab = nullptr, *cnt = nullptr, *permd = nullptr;
  const cudaStream_t s = 0;
  const kmeansErrorStatus E = KMEANS_ERROR_BUILDDATA;
  KD_TRY(B.alloc(&X, (size_t)m * n), E);
  KD_TRY(cudaMemcpy(X, data, sizeof(double) * (size_t)m * n, cudaMemcpyHostToDevice), E);

  RefInit r;
  try {
    r = ref.get();
  } catch (...) {
    return KMEANS_ERROR_INITIALIZE;
  }
  if (!r.ok) return KMEANS_ERROR_INITIALIZE;
  const std::vector<int>& perm = r.perm;
  const std::vector<int>& picks = r.picks;
  std::vector<double> C((size_t)k * n);
  if (kpp_seed < 0)
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < n; ++j) {
        C[(size_t)i * n + j] = data[(size_t)perm[picks[i]] * n + j];
        result[(size_t)j * k + i] = C[(size_t)i * n + j];
      }
  if (mini) {
    KD_TRY(B.alloc(&Xw, (size_t)m_mb * n), E);
    KD_TRY(B.alloc(&permd, m), E);
    KD_TRY(cudaMemcpy(permd, perm.data(), sizeof(int) * m, cudaMemcpyHostToDevice), E);
  }
  KD_TRY(B.alloc(&Cd, (size_t)k * n), E);
  KD_TRY(B.alloc(&CT, (size_t)k * n), E);
  KD_TRY(B.alloc(&acc, (size_t)k * n), E);
  KD_TRY(B.alloc(&cnt, k), E);
  KD_TRY(B.alloc(&lab, m_mb), E);
  const int sse_blocks = kmgb::num_sms() * 4;
  KD_TRY(B.alloc(&part, sse_blocks), E);
  KD_TRY(B.alloc(&sse, 1), E);
  if (kpp_seed < 0) {
    KD_TRY(cudaMemcpy(Cd, C.data(), sizeof(double) * C.size(), cudaMemcpyHostToDevice), E);
  } else {
    double* d2 = nullptr;
    unsigned long long *blk = nullptr, *sc = nullptr;
    int *kp = nullptr, *err = nullptr;
    const kmeansErrorStatus EI = KMEANS_ERROR_INITIALIZE;
    KD_TRY(B.alloc(&d2, kmeanspp_d2_elems(m)), EI);
    KD_TRY(B.alloc(&blk, kmeanspp_blocks(m)), EI);
    KD_TRY(B.alloc(&sc, 3), EI);
    KD_TRY(B.alloc(&kp, k), EI);
    KD_TRY(B.alloc(&err, 1), EI);
    KD_TRY(cudaMemset(err, 0, sizeof(int)), EI);
    KD_TRY(launch_kmeanspp(X, n, m, n, k, (unsigned long long)kpp_seed, Cd, n, kp, d2, blk, sc, err,
                           s),
           EI);
    KD_TRY(cudaMemcpy(C.data(), Cd, sizeof(double) * C.size(), cudaMemcpyDeviceToHost), EI);
    int e = 0;
    KD_TRY(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost), EI);
    if (e) return EI;
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < n; ++j) result[(size_t)j * k + i] = C[(size_t)i * n + j];
  }
  UpdateWork w{};
  w.n = m_mb;
  w.k = k;
  w.d = n;
  w.ldx = n;
  plan_update_tiles(m_mb, k, &w.tile_pts, &w.ntiles);
  w.max_pieces = m_mb / kSumPiece + k + 1;
  const long long hist_elems = (long long)k * w.ntiles;
  KD_TRY(B.alloc(&w.hist, hist_elems), E);
  KD_TRY(B.alloc(&w.scan_tmp, update_scan_tmp_elems(std::max<long long>(hist_elems, k + 1))), E);
  KD_TRY(B.alloc(&w.label_off, k + 1), E);
  KD_TRY(B.alloc(&w.piece_cnt, k + 1), E);
  KD_TRY(B.alloc(&w.sorted, m_mb), E);
  KD_TRY(B.alloc(&w.part, (size_t)w.max_pieces * n), E);

  // Tensor path (full batches, D within the split tier's limit): X and the centers are rounded
  // to FP32, the split BF16 tier assigns every point under its bound widened by that rounding
  // (|key(x,c) - key(fl(x),fl(c))| <= 2^-23 (|x||c| + |c|^2/2), taken twice), and the points it
  // cannot certify get the exact FP64 scan. KMGB_ASSIGN=fp32 keeps the FP64 scan for every point.
  const char* tier_env = std::getenv("KMGB_ASSIGN");
  const bool tc = !mini && bf16_tc_supported(n, 2) &&
                  !(tier_env && std::strcmp(tier_env, "fp32") == 0);
  const long long ldx = (n + 3) / 4 * 4, ldb = (n + 7) / 8 * 8;
  float *Xf = nullptr, *xn = nullptr, *Cf = nullptr, *Cop = nullptr, *cn = nullptr,
        *cmax = nullptr, *cinit = nullptr;
  double* qn = nullptr;
  uint16_t *Xb = nullptr, *Xl = nullptr, *Cb = nullptr, *Cl = nullptr;
  int *rr_list = nullptr, *rr_count = nullptr, *derr = nullptr;
  if (tc) {
    const kmeansErrorStatus EA = KMEANS_ERROR_CLOSEST_CENTERS;
    KD_TRY(B.alloc(&Xf, (size_t)m * ldx), E);
    KD_TRY(B.alloc(&xn, m), E);
    KD_TRY(B.alloc(&qn, m), E);
    KD_TRY(B.alloc(&Xb, (size_t)m * ldb), E);
    KD_TRY(B.alloc(&Xl, (size_t)m * ldb), E);
    KD_TRY(B.alloc(&Cf, (size_t)k * ldx), E);
    KD_TRY(B.alloc(&Cop, (size_t)k * ldx), E);
    KD_TRY(B.alloc(&Cb, (size_t)k * ldb), E);
    KD_TRY(B.alloc(&Cl, (size_t)k * ldb), E);
    KD_TRY(B.alloc(&cn, k), E);
    KD_TRY(B.alloc(&cmax, 1), E);
    KD_TRY(B.alloc(&cinit, (size_t)((k + kCenterPad - 1) / kCenterPad * kCenterPad)), E);
    KD_TRY(B.alloc(&rr_list, m), E);
    KD_TRY(B.alloc(&rr_count, 3), E);
    KD_TRY(B.alloc(&derr, 1), E);
    KD_TRY(cudaMemsetAsync(derr, 0, sizeof(int), s), E);
    d2f_kernel<<<kmgb::num_sms() * 8, 256, 0, s>>>(X, m, n, Xf, ldx); kmgb::count_launches(1);
    KD_TRY(cudaGetLastError(), E);
    KD_TRY(launch_point_norms(Xf, ldx, m, n, qn, xn, s), E);
    KD_TRY(launch_to_bf16(Xf, ldx, m, n, Xb, ldb, s, nullptr, Xl, nullptr), EA);
  }

  const int threads = 256;
  const size_t smem = sizeof(double) * n * (threads / 32);
  if (smem > 200 * 1024) return KMEANS_ERROR_CLOSEST_CENTERS;
  if (smem > 48 * 1024)
    KD_TRY(cudaFuncSetAttribute(assign_d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem),
           KMEANS_ERROR_CLOSEST_CENTERS);
  double sse_old = 0.0, rel = 1.0;
  int it = 0;
  long long start = 0;
  while (it < maxIters && rel > criterion) {
    const double* Xa = X;
    if (mini) {
      gather_d_kernel<<<kmgb::num_sms() * 8, 256, 0, s>>>(X, n, permd, m, start, m_mb, Xw); kmgb::count_launches(1);
      Xa = Xw;
    }
    transpose_d_kernel<<<kmgb::num_sms() * 4, 256, 0, s>>>(Cd, k, n, CT); kmgb::count_launches(1);
    if (tc) {
      const kmeansErrorStatus EA = KMEANS_ERROR_CLOSEST_CENTERS;
      d2f_kernel<<<kmgb::num_sms() * 4, 256, 0, s>>>(Cd, k, n, Cf, ldx); kmgb::count_launches(1);
      KD_TRY(cudaMemsetAsync(cmax, 0, sizeof(float), s), EA);
      KD_TRY(cudaMemsetAsync(rr_count, 0, 3 * sizeof(int), s), EA);
      KD_TRY(launch_prep_centers(Cf, ldx, k, n, Cop, Cb, ldb, cn, cmax, s, nullptr, cinit, Cl), EA);
      AssignArgs a{};
      a.cn = cn;
      a.xnorm = xn;
      a.cmax = cmax;
      a.cinit = cinit;
      a.labels = lab;
      a.rerank_list = rr_list;
      a.rerank_count = rr_count;
      a.err = derr;
      a.n = m;
      a.k = k;
      a.d = n;
      a.certify = 1;
      a.gamma = assign_bf16_gamma(n);
      a.pert = 0x1p-22f;
      KD_TRY(launch_assign_bf16(Xb, Xl, ldb, Cb, Cl, ldb, a, s), EA);
      assign_d_kernel<<<kmgb::num_sms() * 8, threads, smem, s>>>(X, m, n, CT, k, lab, rr_list, rr_count);
      kmgb::count_launches(1);
    } else {
      assign_d_kernel<<<kmgb::num_sms() * 8, threads, smem, s>>>(Xa, m_mb, n, CT, k, lab);
      kmgb::count_launches(1);
    }
    KD_TRY(cudaGetLastError(), KMEANS_ERROR_CLOSEST_CENTERS);
    KD_TRY(cudaMemsetAsync(acc, 0, sizeof(double) * (size_t)k * n, s), KMEANS_ERROR_RESET);
    KD_TRY(cudaMemsetAsync(cnt, 0, sizeof(int) * k, s), KMEANS_ERROR_RESET);
    KD_TRY(launch_tile_accumulate<double>(Xa, n, lab, w, acc, cnt, s), KMEANS_ERROR_CLUSTER_CENTERS);
    KD_TRY(launch_finalize_acc<double>(acc, cnt, k, n, Cd, nullptr, s), KMEANS_ERROR_CLUSTER_CENTERS);
    sse_d_partial_kernel<<<sse_blocks, 256, 0, s>>>(Xa, m_mb, n, lab, Cd, part); kmgb::count_launches(1);
    sse_d_final_kernel<<<1, 32, 0, s>>>(part, sse_blocks, sse); kmgb::count_launches(1);
    KD_TRY(cudaGetLastError(), KMEANS_ERROR_COMPACTNESS);
    double h = 0.0;
    KD_TRY(cudaMemcpy(&h, sse, sizeof(double), cudaMemcpyDeviceToHost), KMEANS_ERROR_COMPACTNESS);
    rel = std::fabs(h - sse_old) / std::fabs(h);
    sse_old = h;
    *final_sse = h;
    ++it;
    if (mini) {
      start += m_mb;
      if (start > m) start %= m;
      else if (start == m) start = 0;
    }
  }
  KD_TRY(cudaMemcpy(C.data(), Cd, sizeof(double) * C.size(), cudaMemcpyDeviceToHost),
         KMEANS_ERROR_GET_CENTERS);
  if (tc) {  // a bounded wait of the tensor pass gave up: its labels cannot be trusted
    int e = 0;
    KD_TRY(cudaMemcpy(&e, derr, sizeof(int), cudaMemcpyDeviceToHost), KMEANS_ERROR_CLOSEST_CENTERS);
    if (e) {
      set_last_error("computeKmeansD: a bounded wait in the tensor-core assignment gave up");
      return KMEANS_ERROR_CLOSEST_CENTERS;
    }
  }
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < n; ++j) result[(size_t)j * k + i] = C[(size_t)i * n + j];
  return (rel <= criterion) ? KMEANS_SUCCESS : KMEANS_NONCONVERGENCE;
}

}  // namespace

extern "C" kmeansErrorStatus computeKmeansD(const double* data, const int m, const int n,
                                            const int k, const double criterion,
                                            const int maxIters, const int numRetries,
                                            const int initAlgorithm, const int doFullSGEMM,
                                            const int matrixFormat, double* result,
                                            const double miniBatchFraction) {
  if (!data || !result || m <= 0 || n <= 0 || k <= 0) return KMEANS_ERROR_BUILDDATA;
  if (doFullSGEMM < 0 || doFullSGEMM > 2 || matrixFormat < 0 || matrixFormat > 1)
    return KMEANS_ERROR_BUILDDATA;
  if (k > m) return KMEANS_ERROR_INITIALIZE;
  const int iters = maxIters < 0 ? 0 : maxIters;
  double sse = 0.0;
  if (initAlgorithm != KMGB_INIT_KMEANSPP)  // the reference ignores numRetries
    return run_d(data, m, n, k, criterion, iters, result, miniBatchFraction, -1, &sse);
  // k-means++ with seeds 0 .. numRetries-1; the lowest final SSE wins (the first on ties)
  const int retries = numRetries < 1 ? 1 : numRetries;
  double best_sse = std::nan("");
  kmeansErrorStatus best_st = KMEANS_SUCCESS;
  std::vector<double> tmp((size_t)n * k), keep((size_t)n * k);
  for (int r = 0; r < retries; ++r) {
    const kmeansErrorStatus st =
        run_d(data, m, n, k, criterion, iters, tmp.data(), miniBatchFraction, r, &sse);
    if (st != KMEANS_SUCCESS && st != KMEANS_NONCONVERGENCE) return st;
    if (r == 0 || sse < best_sse || (std::isnan(best_sse) && !std::isnan(sse))) {
      best_sse = sse;
      best_st = st;
      keep.swap(tmp);
    }
  }
  std::memcpy(result, keep.data(), sizeof(double) * keep.size());
  return best_st;
}
