// Learned router, network part: the MLP D -> H -> G (ReLU hidden layer, softmax over G groups of
// centers) that proposes, for every point, the group of centers its nearest center lies in.
//
// The reference has no counterpart: its assignment scans every center for every point
// (main/cuda/ClosestCenters.cu:46-83, kmeans.cpp:910-1014). The router only decides which
// centers are scanned first; the certificate and the full-scan fallback (router.cu, engine.cu)
// keep every label equal to the FP64 arg-min over all centers, so a wrong proposal costs time,
// never a label.
//
// Training runs in FP32 on the SIMT pipe, deterministically (every sum in a fixed order), so the
// gradients can be checked against an FP64 oracle:
//   forward   Hd = relu(Xs W1^T + b1)              sgemm<NT> with bias + ReLU epilogue
//             Z  = Hd W2^T + b2                      sgemm<NT> with bias epilogue
//   loss      mean over the batch of logsumexp(Z_i) - Z_i[y_i]; dZ = (softmax(Z) - onehot(y)) / B
//   backward  dW2 = dZ^T Hd, db2 = colsum(dZ)        sgemm<TN> (split over the batch into
//                                                    slices added in order), colsum
//             dHd = (dZ W2) * [Hd > 0]               sgemm<NN> with mask epilogue
//             dW1 = dHd^T Xs, db1 = colsum(dHd)      sgemm<TN>, colsum
//   update    Adam (Kingma & Ba, 2015) with bias correction, over the flat parameter vector
//             [W1 | b1 | W2 | b2].
// Inference on all points runs on the tensor cores (the pair kernel of assign_bf16.cu: store mode
// for the hidden layer, arg-max mode for the group), see router.cu.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "../../include/kmeans_gb300.h"
#include "common.cuh"
#include "kernels.h"
#include "router.h"

namespace kmgb {
namespace {

constexpr int GK = 16;  // k-block of the SIMT GEMM

// C[m][n] = epi(sum_k A(m,k) B(k,n)), k ascending for every output (deterministic).
// A(m,k) = TA ? A[k*lda + m] : A[m*lda + k];  B(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n].
// A tile of (16 TM) x (16 TM) outputs per CTA of 256 threads, TM x TM per thread.
template <bool TA, bool TB, int EPI, int TM>
__global__ void __launch_bounds__(256)
sgemm_kernel(int M, int N, int K, const float* __restrict__ A, long long lda,
             const float* __restrict__ B, long long ldb, float* __restrict__ C, long long ldc,
             const float* __restrict__ bias, const float* __restrict__ mask, long long ldm) {
  constexpr int T = 16 * TM;
  constexpr int PER = T * GK / 256;  // elements of each operand tile per thread
  __shared__ float As[GK][T + 4];
  __shared__ float Bs[GK][T + 4];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const long long m0 = (long long)blockIdx.y * T, n0 = (long long)blockIdx.x * T;
  // split over k (gridDim.z > 1): slice z sums k in [kb, ke) into its own output C + z M ldc
  const int kc = (int)(((K + GK - 1) / GK + gridDim.z - 1) / gridDim.z) * GK;
  const int kb = (int)blockIdx.z * kc;
  const int ke = min(K, kb + kc);
  C += (size_t)blockIdx.z * (size_t)M * (size_t)ldc;
  float acc[TM][TM];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TM; ++j) acc[i][j] = 0.0f;
  for (int k0 = kb; k0 < ke; k0 += GK) {
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int e = tid + r * 256;
      int mm, kk;
      if (TA) {
        kk = e / T;
        mm = e % T;
      } else {
        mm = e / GK;
        kk = e % GK;
      }
      const long long gm = m0 + mm;
      const int gk = k0 + kk;
      float v = 0.0f;
      if (gm < M && gk < ke) v = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      As[kk][mm] = v;
    }
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int e = tid + r * 256;
      int nn, kk;
      if (TB) {
        nn = e / GK;
        kk = e % GK;
      } else {
        kk = e / T;
        nn = e % T;
      }
      const long long gn = n0 + nn;
      const int gk = k0 + kk;
      float v = 0.0f;
      if (gn < N && gk < ke) v = TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[TM], b[TM];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TM; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const long long gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < TM; ++j) {
      const long long gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (EPI == kEpiBias || EPI == kEpiBiasRelu) v += bias[gn];
      if (EPI == kEpiBiasRelu) v = fmaxf(v, 0.0f);
      if (EPI == kEpiMask) v = mask[(size_t)gm * ldm + gn] > 0.0f ? v : 0.0f;
      C[(size_t)gm * ldc + gn] = v;
    }
  }
}

// One warp per row of the logits (G <= 1024): loss_row = logsumexp(z) - z[y],
// dZ = (softmax(z) - onehot(y)) * inv_batch. Lanes take columns lane, lane+32, ... and the
// reductions run as a fixed xor butterfly, so the result does not depend on scheduling.
__global__ void softmax_xent_kernel(const float* __restrict__ Z, int rows, int G,
                                    const int* __restrict__ y, float inv_batch,
                                    float* __restrict__ dZ, float* __restrict__ loss_rows) {
  const int lane = threadIdx.x & 31;
  const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= rows) return;
  const float* z = Z + (size_t)row * G;
  float mx = -INFINITY;
  for (int g = lane; g < G; g += 32) mx = fmaxf(mx, z[g]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  float s = 0.0f;
  for (int g = lane; g < G; g += 32) s += expf(z[g] - mx);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const int t = y[row];
  const float inv_s = 1.0f / s;
  for (int g = lane; g < G; g += 32) {
    const float p = expf(z[g] - mx) * inv_s;
    dZ[(size_t)row * G + g] = (p - (g == t ? 1.0f : 0.0f)) * inv_batch;
  }
  if (lane == 0) loss_rows[row] = (mx + logf(s)) - z[t];
}

// out[n] = sum over rows of M[row][n]: per column, 8 row slices summed in order, then the 8
// partial sums added in order (deterministic).
__global__ void colsum_kernel(const float* __restrict__ Mx, int rows, int cols,
                              float* __restrict__ out) {
  __shared__ float part[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + tx;
  float s = 0.0f;
  if (c < cols)
    for (int r = ty; r < rows; r += 8) s += Mx[(size_t)r * cols + c];
  part[ty][tx] = s;
  __syncthreads();
  if (ty == 0 && c < cols) {
    float t = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) t += part[i][tx];
    out[c] = t;
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, long long n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  }
}

// C[i] = part[0][i] + part[1][i] + ... in slice order (deterministic split-k).
__global__ void sum_slices_kernel(const float* __restrict__ part, int slices, long long count,
                                  float* __restrict__ C) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    float v = part[i];
    for (int z = 1; z < slices; ++z) v += part[(size_t)z * count + i];
    C[i] = v;
  }
}

// part (nullable, part_elems floats): scratch for splitting a long k over slices when the output
// has too few tiles to fill the GPU (the weight gradients: k = the batch); without epilogue only.
template <bool TA, bool TB, int EPI>
cudaError_t sgemm(int M, int N, int K, const float* A, long long lda, const float* B,
                  long long ldb, float* C, long long ldc, const float* bias, const float* mask,
                  long long ldm, cudaStream_t s, float* part = nullptr, long long part_elems = 0) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const long long tiles64 = ((long long)(M + 63) / 64) * ((N + 63) / 64);
  if (part && EPI == kEpiNone && ldc == N && tiles64 < num_sms()) {
    long long z = std::min<long long>(8, std::max<long long>(1, 2LL * num_sms() / tiles64));
    z = std::min<long long>(z, (K + GK - 1) / GK);
    if (z > 1 && z * M * N <= part_elems) {
      dim3 grid((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64), (unsigned)z);
      sgemm_kernel<TA, TB, EPI, 4><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, part, N, bias,
                                                       mask, ldm);
      sum_slices_kernel<<<num_sms() * 4, 256, 0, s>>>(part, (int)z, (long long)M * N, C);
      count_launches(2);
      return cudaGetLastError();
    }
  }
  // 128 x 128 tiles when they still give every SM a tile, else 64 x 64
  const long long big = ((long long)(M + 127) / 128) * ((N + 127) / 128);
  if (big >= num_sms()) {
    dim3 grid((unsigned)((N + 127) / 128), (unsigned)((M + 127) / 128));
    sgemm_kernel<TA, TB, EPI, 8><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, mask,
                                                     ldm);
  } else {
    dim3 grid((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64));
    sgemm_kernel<TA, TB, EPI, 4><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, mask,
                                                     ldm);
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t mlp_forward(const MlpShape& sh, const float* params, const float* Xs, int rows,
                        float* Hd, float* Z, cudaStream_t s) {
  const float* W1 = params;
  const float* b1 = W1 + (size_t)sh.hidden * sh.d;
  const float* W2 = b1 + sh.hidden;
  const float* b2 = W2 + (size_t)sh.groups * sh.hidden;
  KMGB_CUDA_TRY((sgemm<false, true, kEpiBiasRelu>(rows, sh.hidden, sh.d, Xs, sh.d, W1, sh.d, Hd,
                                                   sh.hidden, b1, nullptr, 0, s)));
  return sgemm<false, true, kEpiBias>(rows, sh.groups, sh.hidden, Hd, sh.hidden, W2, sh.hidden, Z,
                                      sh.groups, b2, nullptr, 0, s);
}

cudaError_t mlp_backward(const MlpShape& sh, const float* params, const float* Xs, const int* y,
                         int rows, int batch_norm_rows, float* Hd, float* Z, float* dZ,
                         float* dHd, float* grads, float* loss_rows, cudaStream_t s, float* part,
                         long long part_elems) {
  KMGB_CUDA_TRY(mlp_forward(sh, params, Xs, rows, Hd, Z, s));
  const float* W2 = params + (size_t)sh.hidden * sh.d + sh.hidden;
  float* gW1 = grads;
  float* gb1 = gW1 + (size_t)sh.hidden * sh.d;
  float* gW2 = gb1 + sh.hidden;
  float* gb2 = gW2 + (size_t)sh.groups * sh.hidden;
  const int warps_per_block = 8;
  softmax_xent_kernel<<<(rows + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0,
                        s>>>(Z, rows, sh.groups, y, 1.0f / (float)batch_norm_rows, dZ, loss_rows);
  count_launches(1);
  KMGB_CUDA_TRY(cudaGetLastError());
  // dW2[g][h] = sum_b dZ[b][g] Hd[b][h]
  KMGB_CUDA_TRY((sgemm<true, false, kEpiNone>(sh.groups, sh.hidden, rows, dZ, sh.groups, Hd,
                                               sh.hidden, gW2, sh.hidden, nullptr, nullptr, 0, s,
                                               part, part_elems)));
  colsum_kernel<<<(sh.groups + 31) / 32, 256, 0, s>>>(dZ, rows, sh.groups, gb2);
  count_launches(1);
  // dHd[b][h] = (sum_g dZ[b][g] W2[g][h]) [Hd[b][h] > 0]
  KMGB_CUDA_TRY((sgemm<false, false, kEpiMask>(rows, sh.hidden, sh.groups, dZ, sh.groups, W2,
                                                sh.hidden, dHd, sh.hidden, nullptr, Hd, sh.hidden,
                                                s)));
  // dW1[h][j] = sum_b dHd[b][h] Xs[b][j]
  KMGB_CUDA_TRY((sgemm<true, false, kEpiNone>(sh.hidden, sh.d, rows, dHd, sh.hidden, Xs, sh.d, gW1,
                                               sh.d, nullptr, nullptr, 0, s, part, part_elems)));
  colsum_kernel<<<(sh.hidden + 31) / 32, 256, 0, s>>>(dHd, rows, sh.hidden, gb1);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t mlp_adam(float* params, const float* grads, float* m, float* v, long long n,
                     const AdamCfg& c, long long step, cudaStream_t s) {
  const double c1 = 1.0 / (1.0 - std::pow((double)c.beta1, (double)step));
  const double c2 = 1.0 / (1.0 - std::pow((double)c.beta2, (double)step));
  adam_kernel<<<num_sms() * 4, 256, 0, s>>>(params, grads, m, v, n, c.lr, c.beta1, c.beta2, c.eps,
                                            (float)c1, (float)c2);
  count_launches(1);
  return cudaGetLastError();
}

long long mlp_split_scratch(const MlpShape& sh) {
  return 8LL * std::max((long long)sh.groups * sh.hidden, (long long)sh.hidden * sh.d);
}

long long mlp_param_count(const MlpShape& sh) {
  return (long long)sh.hidden * sh.d + sh.hidden + (long long)sh.groups * sh.hidden + sh.groups;
}

}  // namespace kmgb

// ------------------------------------------------------------------------------------------
// C-ABI: the training step and loop on host arrays, for checking them against an oracle
// ------------------------------------------------------------------------------------------
namespace {

struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t get(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return e;
    ptrs.push_back(q);
    *p = static_cast<T*>(q);
    return cudaSuccess;
  }
};

}  // namespace

extern "C" {

int kmgb_router_mlp_train(const float* X, int rows, int d, const int* y, int hidden, int groups,
                          float* params, int batch, int steps, float lr, double* loss,
                          float* grads_out) {
  using namespace kmgb;
  if (!X || !y || !params || rows <= 0 || d <= 0 || hidden <= 0 || groups <= 0 || groups > 1024 ||
      batch <= 0 || steps < 0) {
    set_last_error("kmgb_router_mlp_train: invalid arguments");
    return KMEANS_ERROR_BUILDDATA;
  }
  for (int i = 0; i < rows; ++i)
    if (y[i] < 0 || y[i] >= groups) {
      set_last_error("kmgb_router_mlp_train: a label is outside [0, groups)");
      return KMEANS_ERROR_BUILDDATA;
    }
  const MlpShape sh{d, hidden, groups};
  const long long np = mlp_param_count(sh);
  const int b = batch < rows ? batch : rows;
  DevBufs db;
  float *dX, *dP, *dG, *dm, *dv, *Hd, *Z, *dZ, *dH, *lr_rows, *part;
  int* dy;
  const long long part_elems = mlp_split_scratch(sh);
  cudaError_t e = cudaSuccess;
  if ((e = db.get(&part, part_elems)) ||
      (e = db.get(&dX, (size_t)rows * d)) || (e = db.get(&dy, rows)) || (e = db.get(&dP, np)) ||
      (e = db.get(&dG, np)) || (e = db.get(&dm, np)) || (e = db.get(&dv, np)) ||
      (e = db.get(&Hd, (size_t)b * hidden)) || (e = db.get(&Z, (size_t)b * groups)) ||
      (e = db.get(&dZ, (size_t)b * groups)) || (e = db.get(&dH, (size_t)b * hidden)) ||
      (e = db.get(&lr_rows, b))) {
    set_last_error(cudaGetErrorString(e));
    return KMEANS_ERROR_BUILDDATA;
  }
  const cudaStream_t s = 0;
  cudaMemcpy(dX, X, sizeof(float) * (size_t)rows * d, cudaMemcpyHostToDevice);
  cudaMemcpy(dy, y, sizeof(int) * rows, cudaMemcpyHostToDevice);
  cudaMemcpy(dP, params, sizeof(float) * np, cudaMemcpyHostToDevice);
  cudaMemset(dm, 0, sizeof(float) * np);
  cudaMemset(dv, 0, sizeof(float) * np);
  const AdamCfg cfg{lr, 0.9f, 0.999f, 1e-8f};
  // steps == 0: one forward/backward over the first `batch` rows, gradients out, no update;
  // otherwise `steps` Adam steps over consecutive batches (wrapping around the rows)
  const int todo = steps == 0 ? 1 : steps;
  long long r0 = 0;
  for (int t = 0; t < todo && e == cudaSuccess; ++t) {
    if (r0 + b > rows) r0 = 0;
    e = mlp_backward(sh, dP, dX + (size_t)r0 * d, dy + r0, b, b, Hd, Z, dZ, dH, dG, lr_rows, s,
                     part, part_elems);
    if (e == cudaSuccess && steps > 0) e = mlp_adam(dP, dG, dm, dv, np, cfg, t + 1, s);
    r0 += b;
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return KMEANS_ERROR_COMPUTE;
  }
  if (loss) {
    std::vector<float> lrow(b);
    cudaMemcpy(lrow.data(), lr_rows, sizeof(float) * b, cudaMemcpyDeviceToHost);
    double t = 0.0;
    for (float v : lrow) t += v;
    *loss = t / b;
  }
  if (grads_out) cudaMemcpy(grads_out, dG, sizeof(float) * np, cudaMemcpyDeviceToHost);
  cudaMemcpy(params, dP, sizeof(float) * np, cudaMemcpyDeviceToHost);
  return 0;
}

}  // extern "C"
