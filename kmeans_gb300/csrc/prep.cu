// Per-iteration center preparation and once-per-data-set point preparation.
//
// Replaces the reference's colNormalize (main/cuda/Normalize.cu:33-47, run every iteration from
// kmeans.cpp:1161-1163) and rowNormalize (Normalize.cu:3-31, kmeans.cpp:838-840). Norms are
// accumulated in FP64 and rounded once; an empty-cluster (NaN) center becomes an unusable
// center: zero operand row, +inf norm, so it can never win an arg-min (the reference's
// rowTransformMinimum skips NaN the same way: its val < dataReg is false for NaN,
// RowTransformMinimum.cu:29-31).
#include <cuda_bf16.h>

#include <cuda_fp8.h>

#include "common.cuh"
#include "kernels.h"

namespace kmgb {
namespace {

// Row of the bias matrix (kBiasCols BF16 per center): the start value v split exactly into
// three BF16 numbers, v = hi + mid + lo (v - hi and v - hi - mid are exact in FP32, and what
// is left after two 8-bit pieces of a 24-bit significand fits the third), then zeros.
__device__ __forceinline__ void write_bias_row(__nv_bfloat16* row, float v, int lane) {
  const __nv_bfloat16 hi = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(hi);
  const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
  const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
  if (lane < kBiasCols)
    row[lane] = lane == 0 ? hi : (lane == 1 ? mid : (lane == 2 ? lo : __float2bfloat16_rn(0.0f)));
}

// One warp per center.
__global__ void prep_centers_kernel(const float* __restrict__ C, long long ldc, int k, int d,
                                    float* __restrict__ Cop, __nv_bfloat16* __restrict__ Cb,
                                    long long ldcb, float* __restrict__ cn, float* cmax,
                                    const int* stop, float* __restrict__ cinit, int kpad,
                                    __nv_bfloat16* __restrict__ Cl,
                                    __nv_bfloat16* __restrict__ cbias) {
  if (stopped(stop)) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= k) {
    if (cinit && warp < kpad && lane == 0) cinit[warp] = -3.0e38f;
    if (cbias && warp < kpad) write_bias_row(cbias + (size_t)warp * kBiasCols, -3.0e38f, lane);
    return;
  }
  const float* c = C + (size_t)warp * ldc;
  double s = 0.0;
  bool bad = false;
  for (int t = lane; t < d; t += 32) {
    const float v = c[t];
    bad |= !isfinite(v);
    s = fma((double)v, (double)v, s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  bad = __any_sync(0xffffffffu, bad);
  float* op = Cop + (size_t)warp * ldc;
  for (int t = lane; t < (int)ldc; t += 32) op[t] = (bad || t >= d) ? 0.0f : c[t];
  if (Cb) {
    __nv_bfloat16* ob = Cb + (size_t)warp * ldcb;
    __nv_bfloat16* ol = Cl ? Cl + (size_t)warp * ldcb : nullptr;
    for (int t = lane; t < (int)ldcb; t += 32) {
      const float v = (bad || t >= d) ? 0.0f : c[t];
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      ob[t] = hi;
      if (ol) ol[t] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
  }
  if (cbias)
    write_bias_row(cbias + (size_t)warp * kBiasCols,
                   bad ? -3.0e38f : -0.5f * __double2float_rn(s), lane);
  if (lane == 0) {
    if (bad) {
      cn[warp] = INFINITY;
      if (cinit) cinit[warp] = -3.0e38f;
    } else {
      cn[warp] = __double2float_rn(s);
      if (cinit) cinit[warp] = -0.5f * __double2float_rn(s);
      // upper bound of ||c||: round the FP64 sqrt up and add a relative margin
      const float nrm = __double2float_ru(sqrt(s) * (1.0 + 1e-12));
      atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(nrm));
    }
  }
}

__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// One warp per point: qn = ||x||^2 (FP64), xn = FP32 upper bound of ||x||. GB300's FP64 pipe is
// narrow, so the sum runs on the FP32 pipe as an error-free float-float value: exact squares
// (p + e by FMA), TwoSum accumulation per lane, a float-float tree over the warp, and a single
// FP64 addition per point. The float-float sum is within (d/32 + 8) 2^-46 of ||x||^2 relative;
// xn adds 2^-20 before its upward-rounded square root. Rows whose squares leave the FP32 range
// are summed in FP64 instead.
__global__ void point_norms_kernel(const float* __restrict__ X, long long ldx, long long n, int d,
                                   double* __restrict__ qn, float* __restrict__ xn) {
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const float* x = X + (size_t)warp * ldx;
  float hi = 0.0f, lo = 0.0f;
  for (int t = lane; t < d; t += 32) {
    const float v = __ldg(x + t);
    const float p = __fmul_rn(v, v);
    const float e = __fmaf_rn(v, v, -p);  // v*v - p exactly
    float s1, err;
    ff_two_sum(hi, p, s1, err);
    hi = s1;
    lo = __fadd_rn(lo, __fadd_rn(err, e));
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    float s1, err;
    ff_two_sum(hi, oh, s1, err);
    hi = s1;
    lo = __fadd_rn(lo, __fadd_rn(ol, err));
  }
  if (!(fabsf(hi) < 1.0e37f)) {  // overflow (or NaN input): FP64 sum, same for every lane
    double sd = 0.0;
    for (int t = lane; t < d; t += 32) {
      const double v = (double)__ldg(x + t);
      sd = fma(v, v, sd);
    }
    for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
    if (lane == 0) {
      if (qn) qn[warp] = sd;
      if (xn) xn[warp] = __double2float_ru(sqrt(sd) * (1.0 + 1e-12));
    }
    return;
  }
  if (lane == 0) {
    if (qn) qn[warp] = (double)hi + (double)lo;
    if (xn) xn[warp] = __fsqrt_ru(__fmul_ru(__fadd_ru(hi, fabsf(lo)), 1.0f + 0x1p-20f));
  }
}

// One warp per row (grid-stride over rows): BF16 value plane and, when requested, the BF16
// residual plane bf16(x - bf16(x)).
// inexact (nullable): set to 1 when some value of X is not a BF16 number (v != bf16(v); NaN
// included), i.e. when the residual plane carries information.
__global__ void to_bf16_kernel(const float* __restrict__ X, long long ldx, long long n, int d,
                               __nv_bfloat16* __restrict__ Xb, long long ldb, const int* stop,
                               __nv_bfloat16* __restrict__ Xl, int* inexact) {
  if (stopped(stop)) return;
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  bool off = false;
  for (long long r = w0; r < n; r += nw) {
    const float* x = X + (size_t)r * ldx;
    __nv_bfloat16* ob = Xb + (size_t)r * ldb;
    __nv_bfloat16* ol = Xl ? Xl + (size_t)r * ldb : nullptr;
    for (int c = lane; c < (int)ldb; c += 32) {
      const float v = c < d ? __ldg(x + c) : 0.0f;
      const __nv_bfloat16 hi = __float2bfloat16_rn(v);
      ob[c] = hi;
      off |= !(v == __bfloat162float(hi));
      if (ol) ol[c] = __float2bfloat16_rn(v - __bfloat162float(hi));
    }
  }
  if (inexact && __any_sync(0xffffffffu, off) && lane == 0) atomicExch(inexact, 1);
}

__global__ void gather_rows_kernel(const float* __restrict__ Xs, long long ldx,
                                   const int* __restrict__ perm, long long m, long long start,
                                   long long m_mb, int d, float* __restrict__ Xd, long long ldd,
                                   const int* stop) {
  if (stopped(stop)) return;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= m_mb) return;
  long long pos = start + warp;
  if (pos >= m) pos -= m;
  const float* src = Xs + (size_t)perm[pos] * ldx;
  float* dst = Xd + (size_t)warp * ldd;
  for (int t = lane; t < (int)ldd; t += 32) dst[t] = t < d ? src[t] : 0.0f;
}

__global__ void gather_vec_kernel(const double* __restrict__ qs, const float* __restrict__ xs,
                                  const int* __restrict__ perm, long long m, long long start,
                                  long long m_mb, double* __restrict__ qd, float* __restrict__ xd,
                                  const int* stop) {
  if (stopped(stop)) return;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < m_mb;
       r += (long long)gridDim.x * blockDim.x) {
    long long pos = start + r;
    if (pos >= m) pos -= m;
    const int src = perm[pos];
    qd[r] = qs[src];
    xd[r] = xs[src];
  }
}

// FP8 E4M3 operands with power-of-two scales: x = s * x8 + error, s = 2^(e - 8) where the scaled
// quantity (a row's largest |x_i|, or for the centers the largest ||c||) is below 2^e, so every
// scaled value is below 2^8 = 256 < 448 (the largest E4M3 number: no saturation) and the division
// by s is exact; the conversion rounds to nearest even, each element within 2^-4 relative of its
// value when normal and within s 2^-10 when it falls among the subnormals.
__device__ __forceinline__ float pow2_scale_for(float mx) {
  if (!(mx > 0.0f) || !(mx < INFINITY)) return 1.0f;
  int e;
  frexpf(mx, &e);  // mx = f 2^e, f in [0.5, 1)
  return ldexpf(1.0f, e - 8);
}

// One warp per row: the row's scale (sx[row]) and its E4M3 copy, zero padded to ld8 bytes.
__global__ void to_fp8_kernel(const float* __restrict__ X, long long ldx, long long n, int d,
                              uint8_t* __restrict__ X8, long long ld8, float* __restrict__ sx,
                              const int* stop) {
  if (stopped(stop)) return;
  const int lane = threadIdx.x & 31;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((long long)gridDim.x * blockDim.x) >> 5) {
    const float* x = X + (size_t)r * ldx;
    float mx = 0.0f;
    for (int t = lane; t < d; t += 32) mx = fmaxf(mx, fabsf(x[t]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const float sc = pow2_scale_for(mx);
    const float inv = 1.0f / sc;  // a power of two: exact
    for (long long t = lane; t < ld8; t += 32)
      X8[(size_t)r * ld8 + t] =
          t < d ? (uint8_t)__nv_cvt_float_to_fp8(x[t] * inv, __NV_SATFINITE, __NV_E4M3) : 0;
    if (lane == 0) sx[r] = sc;
  }
}

// The centers' E4M3 copy with one scale for all of them, from the operand copy (unusable centers
// are zero rows) and the bound of the largest center norm: cscale = 2^(e - 8), cmax < 2^e.
__global__ void centers_fp8_kernel(const float* __restrict__ Cop, long long ldc, int k, int d,
                                   const float* __restrict__ cmax, uint8_t* __restrict__ C8,
                                   long long ld8, float* __restrict__ cscale, const int* stop) {
  if (stopped(stop)) return;
  const float sc = pow2_scale_for(*cmax);
  const float inv = 1.0f / sc;
  if (blockIdx.x == 0 && threadIdx.x == 0) *cscale = sc;
  const long long total = (long long)k * ld8;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long c = i / ld8, t = i % ld8;
    C8[i] = t < d ? (uint8_t)__nv_cvt_float_to_fp8(Cop[(size_t)c * ldc + t] * inv,
                                                     __NV_SATFINITE, __NV_E4M3)
                  : 0;
  }
}

}  // namespace

cudaError_t launch_to_fp8(const float* X, long long ldx, long long n, int d, void* X8,
                          long long ld8, float* sx, cudaStream_t s, const int* stop) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (n <= 0) return cudaSuccess;
  if (ld8 % 16 || ld8 < d) return cudaErrorInvalidValue;
  to_fp8_kernel<<<kmgb::num_sms() * 16, 256, 0, s>>>(X, ldx, n, d, static_cast<uint8_t*>(X8), ld8,
                                                     sx, stop);
  kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_centers_fp8(const float* Cop, long long ldc, int k, int d, const float* cmax,
                               void* C8, long long ld8, float* cscale, cudaStream_t s,
                               const int* stop) {
  if (k <= 0) return cudaSuccess;
  if (ld8 % 16 || ld8 < d) return cudaErrorInvalidValue;
  centers_fp8_kernel<<<kmgb::num_sms() * 4, 256, 0, s>>>(Cop, ldc, k, d, cmax,
                                                         static_cast<uint8_t*>(C8), ld8, cscale,
                                                         stop);
  kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_prep_centers(const float* C, long long ldc, int k, int d, float* Cop, void* Cb,
                                long long ldcb, float* cn, float* cmax, cudaStream_t s,
                                const int* stop, float* cinit, void* Cl, void* cbias) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (k <= 0) return cudaSuccess;
  const int threads = 256;
  const int kpad = (k + kCenterPad - 1) / kCenterPad * kCenterPad;
  const int blocks = (int)(((long long)(cinit || cbias ? kpad : k) * 32 + threads - 1) / threads);
  prep_centers_kernel<<<blocks, threads, 0, s>>>(C, ldc, k, d, Cop,
                                                 reinterpret_cast<__nv_bfloat16*>(Cb), ldcb, cn,
                                                 cmax, stop, cinit, kpad,
                                                 reinterpret_cast<__nv_bfloat16*>(Cl),
                                                 reinterpret_cast<__nv_bfloat16*>(cbias));
  kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_point_norms(const float* X, long long ldx, long long n, int d, double* qn,
                               float* xn, cudaStream_t s) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (n <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (n * 32 + threads - 1) / threads;
  point_norms_kernel<<<(unsigned)blocks, threads, 0, s>>>(X, ldx, n, d, qn, xn); kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_to_bf16(const float* X, long long ldx, long long n, int d, void* Xb,
                           long long ldb, cudaStream_t s, const int* stop, void* Xl,
                           int* inexact) {
  if (inject_fault(kFaultLaunch)) return cudaErrorLaunchOutOfResources;
  if (n <= 0) return cudaSuccess;
  to_bf16_kernel<<<kmgb::num_sms() * 16, 256, 0, s>>>(X, ldx, n, d, reinterpret_cast<__nv_bfloat16*>(Xb),
                                          ldb, stop, reinterpret_cast<__nv_bfloat16*>(Xl),
                                          inexact); kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_gather_rows(const float* Xsrc, long long ldx, const int* perm, long long m,
                               long long start, long long m_mb, int d, float* Xdst, long long ldd,
                               cudaStream_t s, const int* stop) {
  if (m_mb <= 0) return cudaSuccess;
  const int threads = 256;
  const long long blocks = (m_mb * 32 + threads - 1) / threads;
  gather_rows_kernel<<<(unsigned)blocks, threads, 0, s>>>(Xsrc, ldx, perm, m, start, m_mb, d,
                                                          Xdst, ldd, stop); kmgb::count_launches(1);
  return cudaGetLastError();
}

cudaError_t launch_gather_vec(const double* qsrc, const float* xsrc, const int* perm, long long m,
                              long long start, long long m_mb, double* qdst, float* xdst,
                              cudaStream_t s, const int* stop) {
  if (m_mb <= 0) return cudaSuccess;
  gather_vec_kernel<<<kmgb::num_sms() * 4, 256, 0, s>>>(qsrc, xsrc, perm, m, start, m_mb, qdst, xdst, stop); kmgb::count_launches(1);
  return cudaGetLastError();
}

}  // namespace kmgb
