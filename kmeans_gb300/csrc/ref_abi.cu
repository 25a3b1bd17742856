// The reference's per-kernel C entry points (main/cuda/KmeansCudaKernels.h:198-474) on the GB300
// kernels. Same names, argument meaning and kmeansCudaErrorStatus codes; asynchronous on the
// default stream like the reference; the reference's scratch arguments (Bpadded, C, Cindices,
// normRowsOfA_squared in ClosestCenters) are accepted and not needed. Temporary buffers are
// stream-ordered (cudaMallocAsync on the default stream).
#include <cfloat>
#include <cmath>

#include "../../include/kmeans_gb300.h"
#include "common.cuh"
#include "kernels.h"

using namespace kmgb;

namespace {

const cudaStream_t kDefault = 0;

template <typename T>
cudaError_t tmp_alloc(T** p, size_t count) {
  return cudaMallocAsync(reinterpret_cast<void**>(p), sizeof(T) * (count ? count : 1), kDefault);
}
void tmp_free(void* p) {
  if (p) cudaFreeAsync(p, kDefault);
}

// Bt[j][t] = B[t * k + j] (t < d), zero padding to ldc.
template <typename T>
__global__ void transpose_centers_kernel(const T* __restrict__ B, int d, int k, float* __restrict__ Bt,
                                         long long ldc) {
  const long long total = (long long)k * ldc;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e / ldc), t = (int)(e % ldc);
    Bt[e] = t < d ? (float)B[(size_t)t * k + j] : 0.0f;
  }
}

__global__ void copy_pad_kernel(const float* __restrict__ A, long long m, int d, float* __restrict__ Ap,
                                long long ld) {
  const long long total = m * ld;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long r = e / ld;
    const int c = (int)(e % ld);
    Ap[e] = c < d ? A[(size_t)r * d + c] : 0.0f;
  }
}

// cmax = max_j max(||Bt_j||, sqrt(|nb_j|)) (upper bound), for the expansion-mode bound.
__global__ void cmax_expansion_kernel(const float* __restrict__ Bt, long long ldc, int k, int d,
                                      const float* __restrict__ nb, float* cmax) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= k) return;
  double s = 0.0;
  for (int t = lane; t < d; t += 32) {
    const double v = Bt[(size_t)warp * ldc + t];
    s = fma(v, v, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    double m = fmax(s, fabs((double)nb[warp]));
    if (!(m < INFINITY)) m = 3.0e38;  // NaN / inf norms: make the bound huge (all re-ranked)
    const float r = __double2float_ru(sqrt(m) * (1.0 + 1e-12));
    atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(r));
  }
}

// FP64 arg-min of nb_j - 2 A_i.B_j (B is d x k, K fastest); one warp per row, lanes over j.
__global__ void closest_fp64_kernel(int m0, int m, int d, const double* __restrict__ A, int k,
                                    const double* __restrict__ B, const double* __restrict__ nb,
                                    int* __restrict__ out) {
  extern __shared__ double xs_all[];
  const int warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* xs = xs_all + (size_t)w * d;
  for (long long i = (long long)blockIdx.x * warps + w; i < m; i += (long long)gridDim.x * warps) {
    for (int t = lane; t < d; t += 32) xs[t] = A[(size_t)i * d + t];
    __syncwarp();
    double best = INFINITY;
    int bi = -1;
    for (int j = lane; j < k; j += 32) {
      double s = 0.0;
      for (int t = 0; t < d; ++t) s = fma(xs[t], B[(size_t)t * k + j], s);
      const double v = fma(-2.0, s, nb[j]);
      if (v < best) {
        best = v;
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
    if (lane == 0) out[m0 + i] = bi < 0 ? 0 : bi;
    __syncwarp();
  }
}

// rowTransformMinimum with the reference's expression (RowTransformMinimum.cu:27-50).
template <typename T>
__global__ void row_transform_min_kernel(int m0, int m, int n, const T* __restrict__ na,
                                         const T* __restrict__ nbv, const T* __restrict__ in,
                                         int* __restrict__ out) {
  const int warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (long long i = (long long)blockIdx.x * warps + w; i < m; i += (long long)gridDim.x * warps) {
    T best = (T)FLT_MAX;
    int bi = -1;
    const T a = na[i];
    for (int j = lane; j < n; j += 32) {
      T v;
      if (sizeof(T) == 4) {
        const float s = (float)a + (float)nbv[j];
        v = (T)(float)((double)s - 2.0 * (double)in[(size_t)i * n + j]);
      } else {
        v = a + nbv[j] - (T)2.0 * in[(size_t)i * n + j];
      }
      if (v < best) {
        best = v;
        bi = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const T ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      const bool take = (ob < best) || (ob == best && (unsigned)oi < (unsigned)bi);
      best = take ? ob : best;
      bi = take ? oi : bi;
    }
    if (lane == 0) out[m0 + i] = bi;
  }
}

// Squared distance of each row to its center, FP64, block partial sums.
template <typename T>
__global__ void compactness_partial_kernel(int m0, int m, int n, const T* __restrict__ data,
                                           const int* __restrict__ idx, const T* __restrict__ centers,
                                           double* __restrict__ partial) {
  __shared__ double red[256];
  double acc = 0.0;
  const int warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (long long i = (long long)blockIdx.x * warps + w; i < m; i += (long long)gridDim.x * warps) {
    const int l = idx[m0 + i];
    double s = 0.0;
    for (int t = lane; t < n; t += 32) {
      const double u = (double)data[(size_t)i * n + t] - (double)centers[(size_t)l * n + t];
      s = fma(u, u, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    acc += s;  // identical in all lanes
  }
  red[threadIdx.x] = (lane == 0) ? acc : 0.0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)blockDim.x; i += 32) t += red[i];
    partial[blockIdx.x] = t;
  }
}

template <typename T>
__global__ void compactness_final_kernel(const double* __restrict__ partial, int nb, double* acc,
                                         T* out, bool last) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < nb; ++i) t += partial[i];
    *acc += t;
    if (last) out[0] = (T)*acc;
  }
}

template <typename T>
__global__ void row_norm_kernel(int m0, int m, int n, const T* __restrict__ in, T* __restrict__ out) {
  const int warps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (long long i = (long long)blockIdx.x * warps + w; i < m; i += (long long)gridDim.x * warps) {
    double s = 0.0;
    for (int t = lane; t < n; t += 32) s = fma((double)in[(size_t)i * n + t], (double)in[(size_t)i * n + t], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[m0 + i] = (T)s;
  }
}

template <typename T>
__global__ void col_norm_kernel(int m, int n, const T* __restrict__ in, T* __restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s = fma((double)in[(size_t)i * n + j], (double)in[(size_t)i * n + j], s);
    out[j] = (T)s;
  }
}

// C = A B for row-major A (ra x ca), B (ca x cb) and C (ra x cb): 64 x 64 outputs per block of
// 256 threads (4 x 4 per thread), k in steps of 16 through shared memory; each output is one FMA
// chain over k in ascending order. Row tiles beyond the grid's y extent are taken in turn.
template <typename T>
__global__ void matmul_kernel(int ra, int ca, int cb, const T* __restrict__ A,
                              const T* __restrict__ B, T* __restrict__ C) {
  constexpr int TM = 64, TN = 64, TK = 16;
  __shared__ T As[TK][TM + 1];
  __shared__ T Bs[TK][TN];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const long long c0 = (long long)blockIdx.x * TN;
  const long long row_tiles = ((long long)ra + TM - 1) / TM;
  for (long long rt = blockIdx.y; rt < row_tiles; rt += gridDim.y) {
    const long long r0 = rt * TM;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    for (int k0 = 0; k0 < ca; k0 += TK) {
      for (int e = threadIdx.x; e < TM * TK; e += blockDim.x) {
        const int rr = e / TK, kk = e % TK;
        const long long r = r0 + rr;
        As[kk][rr] = (r < ra && k0 + kk < ca) ? A[r * ca + k0 + kk] : T(0);
      }
      for (int e = threadIdx.x; e < TK * TN; e += blockDim.x) {
        const int kk = e / TN, cc = e % TN;
        const long long c = c0 + cc;
        Bs[kk][cc] = (k0 + kk < ca && c < cb) ? B[(long long)(k0 + kk) * cb + c] : T(0);
      }
      __syncthreads();
      const int kn = min(TK, ca - k0);
      for (int kk = 0; kk < kn; ++kk) {
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long r = r0 + ty + 16 * i;
      if (r >= ra) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const long long c = c0 + tx + 16 * j;
        if (c < cb) C[r * cb + c] = acc[i][j];
      }
    }
  }
}

template <typename T>
kmeansCudaErrorStatus mat_mat_mult(int ra, int ca, const T* A, int cb, const T* B, T* C) {
  if (ra < 0 || ca < 0 || cb < 0) return ERROR_MATMATMULT;
  if (ra == 0 || cb == 0) return NO_ERROR;
  if (!C || (ca > 0 && (!A || !B))) return ERROR_MATMATMULT;
  const long long col_tiles = ((long long)cb + 63) / 64, row_tiles = ((long long)ra + 63) / 64;
  const dim3 grid((unsigned)col_tiles, (unsigned)(row_tiles < 65535 ? row_tiles : 65535));
  matmul_kernel<T><<<grid, 256, 0, kDefault>>>(ra, ca, cb, A, B, C);
  kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_MATMATMULT : NO_ERROR;
}

template <typename T>
kmeansCudaErrorStatus cluster_centers(int m0, int m, int n, int k, bool lastTile, const T* data,
                                      const int* indices, T* centers_large, int* counts_large,
                                      T* centers, int* counts) {
  if (m < 0 || n <= 0 || k <= 0 || !centers_large || !counts_large) return ERROR_CLUSTERCENTERS;
  double* acc = reinterpret_cast<double*>(centers_large);
  if (reinterpret_cast<uintptr_t>(acc) & 7) return ERROR_CLUSTERCENTERS;
  UpdateWork w{};
  w.n = m;
  w.k = k;
  w.d = n;
  w.ldx = n;
  plan_update_tiles(m, k, &w.tile_pts, &w.ntiles);
  w.max_pieces = m / kSumPiece + k + 1;
  const long long hist_elems = (long long)k * w.ntiles;
  cudaError_t e = cudaSuccess;
  if (m > 0) {
    e = tmp_alloc(&w.hist, hist_elems);
    if (!e) e = tmp_alloc(&w.scan_tmp, update_scan_tmp_elems(hist_elems > k + 1 ? hist_elems : k + 1));
    if (!e) e = tmp_alloc(&w.label_off, k + 1);
    if (!e) e = tmp_alloc(&w.piece_cnt, k + 1);
    if (!e) e = tmp_alloc(&w.sorted, m);
    if (!e) e = tmp_alloc(&w.part, (size_t)w.max_pieces * n);
    if (!e) e = launch_tile_accumulate<T>(data, n, indices + m0, w, acc, counts_large, kDefault);
  }
  if (!e && lastTile) e = launch_finalize_acc<T>(acc, counts_large, k, n, centers, counts, kDefault);
  tmp_free(w.hist);
  tmp_free(w.scan_tmp);
  tmp_free(w.label_off);
  tmp_free(w.piece_cnt);
  tmp_free(w.sorted);
  tmp_free(w.part);
  return e ? ERROR_CLUSTERCENTERS : NO_ERROR;
}

template <typename T>
kmeansCudaErrorStatus compactness(int m0, int m, bool lastTile, int n, int k, const T* data,
                                  const int* indices, const T* centers, T* out) {
  (void)k;
  if (m < 0 || n <= 0 || !out) return ERROR_COMPACTNESS;
  double* acc = (sizeof(T) == 4) ? reinterpret_cast<double*>(out + 2) : reinterpret_cast<double*>(out + 1);
  if (reinterpret_cast<uintptr_t>(acc) & 7) return ERROR_COMPACTNESS;
  const int blocks = kmgb::num_sms() * 4;
  double* part = nullptr;
  cudaError_t e = tmp_alloc(&part, blocks);
  if (!e) {
    compactness_partial_kernel<T><<<blocks, 256, 0, kDefault>>>(m0, m, n, data, indices, centers, part); kmgb::count_launches(1);
    e = cudaGetLastError();
  }
  if (!e) {
    compactness_final_kernel<T><<<1, 32, 0, kDefault>>>(part, blocks, acc, out, lastTile); kmgb::count_launches(1);
    e = cudaGetLastError();
  }
  tmp_free(part);
  return e ? ERROR_COMPACTNESS : NO_ERROR;
}

}  // namespace

extern "C" {

kmeansCudaErrorStatus ClosestCentersF(const int m0, const int nRowsA, const int nColsA,
                                      const float* A, const int nColsB, const float* B,
                                      float* Bpadded, const float* normRowsOfA_squared,
                                      const float* normColsOfB_squared, const int nColsC, float* C,
                                      int* Cindices, int* CindicesFinal) {
  (void)Bpadded;
  (void)normRowsOfA_squared;
  (void)nColsC;
  (void)C;
  (void)Cindices;
  if (nRowsA < 0 || nColsA <= 0 || nColsB <= 0 || !A || !B || !normColsOfB_squared ||
      !CindicesFinal)
    return ERROR_CLOSESTCENTERS;
  if (nRowsA == 0) return NO_ERROR;
  const int d = nColsA, k = nColsB;
  const long long ld = (d + 3) / 4 * 4;
  const bool direct = (ld == d) && !(reinterpret_cast<uintptr_t>(A) & 15);
  float *Ap = nullptr, *Bt = nullptr, *xn = nullptr, *cmax = nullptr;
  int *list = nullptr, *count = nullptr, *err = nullptr;
  cudaError_t e = cudaSuccess;
  if (!direct) e = tmp_alloc(&Ap, (size_t)nRowsA * ld);
  if (!e) e = tmp_alloc(&Bt, (size_t)k * ld);
  if (!e) e = tmp_alloc(&xn, nRowsA);
  if (!e) e = tmp_alloc(&cmax, 1);
  if (!e) e = tmp_alloc(&list, nRowsA);
  if (!e) e = tmp_alloc(&count, 2);
  if (!e) e = tmp_alloc(&err, 1);
  if (!e) e = cudaMemsetAsync(cmax, 0, sizeof(float), kDefault);
  if (!e) e = cudaMemsetAsync(count, 0, 2 * sizeof(int), kDefault);
  if (!e) e = cudaMemsetAsync(err, 0, sizeof(int), kDefault);
  const float* Xa = A;
  if (!e && !direct) {
    copy_pad_kernel<<<kmgb::num_sms() * 8, 256, 0, kDefault>>>(A, nRowsA, d, Ap, ld); kmgb::count_launches(1);
    e = cudaGetLastError();
    Xa = Ap;
  }
  if (!e) {
    transpose_centers_kernel<float><<<kmgb::num_sms() * 4, 256, 0, kDefault>>>(B, d, k, Bt, ld); kmgb::count_launches(1);
    e = cudaGetLastError();
  }
  if (!e) e = launch_point_norms(Xa, ld, nRowsA, d, nullptr, xn, kDefault);
  if (!e) {
    cmax_expansion_kernel<<<(k * 32 + 255) / 256, 256, 0, kDefault>>>(Bt, ld, k, d,
                                                                     normColsOfB_squared, cmax); kmgb::count_launches(1);
    e = cudaGetLastError();
  }
  if (!e) {
    AssignArgs a{};
    a.cn = normColsOfB_squared;
    a.xnorm = xn;
    a.cmax = cmax;
    a.labels = CindicesFinal + m0;
    a.rerank_list = list;
    a.rerank_count = count;
    a.err = err;
    a.n = nRowsA;
    a.k = k;
    a.d = d;
    a.certify = 1;
    a.gamma = assign_fp32_gamma(d);
    e = launch_assign_fp32(Xa, ld, Bt, ld, a, kDefault);
  }
  if (!e) {
    RerankArgs r{};
    r.X = Xa;
    r.ldx = ld;
    r.C = Bt;
    r.ldc = ld;
    r.nb = normColsOfB_squared;
    r.xnorm = xn;
    r.cmax = cmax;
    r.list = list;
    r.count = count;
    r.labels = CindicesFinal + m0;
    r.n = nRowsA;
    r.k = k;
    r.d = d;
    r.mode = 1;
    r.max_list = nRowsA;
    e = launch_rerank(r, kDefault);
  }
  tmp_free(Ap);
  tmp_free(Bt);
  tmp_free(xn);
  tmp_free(cmax);
  tmp_free(list);
  tmp_free(count);
  tmp_free(err);
  return e ? ERROR_CLOSESTCENTERS : NO_ERROR;
}

kmeansCudaErrorStatus ClosestCentersD(const int m0, const int nRowsA, const int nColsA,
                                      const double* A, const int nColsB, const double* B,
                                      double* Bpadded, const double* normRowsOfA_squared,
                                      const double* normColsOfB_squared, const int nColsC,
                                      double* C, int* Cindices, int* CindicesFinal) {
  (void)Bpadded;
  (void)normRowsOfA_squared;
  (void)nColsC;
  (void)C;
  (void)Cindices;
  if (nRowsA < 0 || nColsA <= 0 || nColsB <= 0 || !A || !B || !normColsOfB_squared ||
      !CindicesFinal)
    return ERROR_CLOSESTCENTERS;
  if (nRowsA == 0) return NO_ERROR;
  const int threads = 256;
  const size_t smem = sizeof(double) * nColsA * (threads / 32);
  if (smem > 200 * 1024) return ERROR_CLOSESTCENTERS;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(closest_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return ERROR_CLOSESTCENTERS;
  closest_fp64_kernel<<<kmgb::num_sms() * 8, threads, smem, kDefault>>>(m0, nRowsA, nColsA, A, nColsB, B,
                                                            normColsOfB_squared, CindicesFinal); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_CLOSESTCENTERS : NO_ERROR;
}

kmeansCudaErrorStatus rowTransformMinimumF(const int m0, const int m, const int n,
                                           const float* normRowsOfA_squared,
                                           const float* normColsOfB_squared, const float* input,
                                           int* output) {
  if (m < 0 || n <= 0) return ERROR_ROWTRANSFORMMINIMUM;
  if (m == 0) return NO_ERROR;
  row_transform_min_kernel<float><<<kmgb::num_sms() * 8, 256, 0, kDefault>>>(
      m0, m, n, normRowsOfA_squared, normColsOfB_squared, input, output); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_ROWTRANSFORMMINIMUM : NO_ERROR;
}

kmeansCudaErrorStatus rowTransformMinimumD(const int m0, const int m, const int n,
                                           const double* normRowsOfA_squared,
                                           const double* normColsOfB_squared,
                                           const double* input, int* output) {
  if (m < 0 || n <= 0) return ERROR_ROWTRANSFORMMINIMUM;
  if (m == 0) return NO_ERROR;
  row_transform_min_kernel<double><<<kmgb::num_sms() * 8, 256, 0, kDefault>>>(
      m0, m, n, normRowsOfA_squared, normColsOfB_squared, input, output); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_ROWTRANSFORMMINIMUM : NO_ERROR;
}

kmeansCudaErrorStatus ClusterCentersF(const int m0, const int m, const int n, const int k,
                                      const bool lastTile, const float* data, const int* indices,
                                      float* centers_large, int* counts_large, float* centers,
                                      int* counts) {
  return cluster_centers<float>(m0, m, n, k, lastTile, data, indices, centers_large, counts_large,
                                centers, counts);
}

kmeansCudaErrorStatus ClusterCentersD(const int m0, const int m, const int n, const int k,
                                      const bool lastTile, const double* data, const int* indices,
                                      double* centers_large, int* counts_large, double* centers,
                                      int* counts) {
  return cluster_centers<double>(m0, m, n, k, lastTile, data, indices, centers_large,
                                 counts_large, centers, counts);
}

kmeansCudaErrorStatus CompactnessF(const int m0, const int m, const bool lastTile, const int n,
                                   const int k, const float* data, const int* indices,
                                   const float* centers, float* compactness_out) {
  return compactness<float>(m0, m, lastTile, n, k, data, indices, centers, compactness_out);
}

kmeansCudaErrorStatus CompactnessD(const int m0, const int m, const bool lastTile, const int n,
                                   const int k, const double* data, const int* indices,
                                   const double* centers, double* compactness_out) {
  return compactness<double>(m0, m, lastTile, n, k, data, indices, centers, compactness_out);
}

kmeansCudaErrorStatus MatMatMultF(const int nRowsA, const int nColsA, const float* A,
                                  const int nColsB, const float* B, float* C) {
  return mat_mat_mult<float>(nRowsA, nColsA, A, nColsB, B, C);
}

kmeansCudaErrorStatus MatMatMultD(const int nRowsA, const int nColsA, const double* A,
                                  const int nColsB, const double* B, double* C) {
  return mat_mat_mult<double>(nRowsA, nColsA, A, nColsB, B, C);
}

kmeansCudaErrorStatus rowNormalizeF(const int m0, const int m, const int n, const float* input,
                                    float* output) {
  if (m < 0 || n <= 0) return ERROR_ROWNORMALIZE;
  if (m == 0) return NO_ERROR;
  row_norm_kernel<float><<<kmgb::num_sms() * 8, 256, 0, kDefault>>>(m0, m, n, input, output); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_ROWNORMALIZE : NO_ERROR;
}

kmeansCudaErrorStatus rowNormalizeD(const int m0, const int m, const int n, const double* input,
                                    double* output) {
  if (m < 0 || n <= 0) return ERROR_ROWNORMALIZE;
  if (m == 0) return NO_ERROR;
  row_norm_kernel<double><<<kmgb::num_sms() * 8, 256, 0, kDefault>>>(m0, m, n, input, output); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_ROWNORMALIZE : NO_ERROR;
}

kmeansCudaErrorStatus colNormalizeF(const int m, const int n, const float* input, float* output) {
  if (m < 0 || n <= 0) return ERROR_COLNORMALIZE;
  col_norm_kernel<float><<<(n + 127) / 128, 128, 0, kDefault>>>(m, n, input, output); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_COLNORMALIZE : NO_ERROR;
}

kmeansCudaErrorStatus colNormalizeD(const int m, const int n, const double* input,
                                    double* output) {
  if (m < 0 || n <= 0) return ERROR_COLNORMALIZE;
  col_norm_kernel<double><<<(n + 127) / 128, 128, 0, kDefault>>>(m, n, input, output); kmgb::count_launches(1);
  return cudaGetLastError() ? ERROR_COLNORMALIZE : NO_ERROR;
}

}  // extern "C"
