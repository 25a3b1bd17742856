// Shared device/host helpers for the GB300 (sm_103a) Lloyd kernels.
//
// Every wait on an mbarrier is bounded: a wait gives up after KMGB_WAIT_CYCLES SM clock cycles
// (about 2 s at 2 GHz), records an error code in the launch's error word and returns false; an
// abort flag in shared memory then makes every later wait of the CTA return at once so the CTA
// drains and exits (no unbounded spin, no __trap). The limit is counted with clock64, a cheap
// register read: a %globaltimer read takes hundreds of cycles on GB300 and, inside the wait
// loop, delayed every wake-up of the pipelines by about that much.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#ifndef KMGB_WAIT_CYCLES
#define KMGB_WAIT_CYCLES 4000000000ull  // about 2 s per wait at a 2 GHz SM clock
#endif

// Error codes written to the device error word (first writer wins).
enum kmgb_dev_error {
  KMGB_DEV_OK = 0,
  KMGB_DEV_TIMEOUT_FULL = 1,     // consumer waited too long for a TMA stage
  KMGB_DEV_TIMEOUT_EMPTY = 2,    // producer waited too long for a free stage
  KMGB_DEV_TIMEOUT_ACC = 3,      // MMA / epilogue accumulator hand-off timed out
  KMGB_DEV_BAD_LABEL = 4,        // a label outside [0, K) reached the update
  KMGB_DEV_BAD_SHAPE = 5,
};

namespace kmgb {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void set_error(int* err, int code) {
  if (err) atomicCAS(err, 0, code);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait. `abort_flag` is a CTA-shared word: once set, waits return false at once.
// `limit`: SM cycles before giving up (KMGB_WAIT_CYCLES unless a test shortens it).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          int* err, int code,
                                          unsigned long long limit = KMGB_WAIT_CYCLES) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if ((unsigned long long)(clock64() - t0) > limit) {
      *abort_flag = 1;
      set_error(err, code);
      return false;
    }
  }
}

// 2-D TMA tile load into shared memory, completion signalled on `bar` (complete_tx bytes).
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar,
                                            int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Byte offset of the 16-byte chunk `chunk` of row `row` inside a tile written by TMA with
// CU_TENSOR_MAP_SWIZZLE_128B (rows of 128 bytes, tile base 1024-byte aligned): the chunk index
// is XOR-ed with the row index modulo 8.
__device__ __forceinline__ uint32_t swz128(uint32_t row, uint32_t chunk) {
  return row * 128u + ((chunk ^ (row & 7u)) << 4);
}

// Device-side stop rule of the Lloyd loop: once the flag is set every later kernel of the run
// returns at once, so the host never has to synchronise to evaluate the criterion.
__device__ __forceinline__ bool stopped(const int* stop) {
  return stop != nullptr && *reinterpret_cast<volatile const int*>(stop) != 0;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Bits of a label below k (0 for k <= 1).
__device__ __forceinline__ int label_bits(int k) { return k <= 1 ? 0 : 32 - __clz(k - 1); }

// The lanes of the warp holding the same label as this lane (labels in [0, 2^nbits), or -1 for
// "none": the -1 lanes form one group of their own). One ballot per label bit: with mostly
// distinct labels in a warp (K ~ 1000 centers) this is much cheaper than __match_any_sync.
// Every lane of the warp calls it with the same nbits.
__device__ __forceinline__ unsigned warp_peers(int l, int nbits) {
  const unsigned valid = __ballot_sync(0xffffffffu, l >= 0);
  unsigned m = l >= 0 ? valid : ~valid;
  for (int b = 0; b < nbits; ++b) {
    const bool bit = (l >> b) & 1;
    const unsigned set = __ballot_sync(0xffffffffu, bit);
    m &= bit ? set : ~set;
  }
  return m;
}

}  // namespace kmgb

// Host-side: 2-D row-major tensor map (inner dim = columns) with 128-byte swizzle.
// dtype: CU_TENSOR_MAP_DATA_TYPE_FLOAT32 or _BFLOAT16. Returns cudaSuccess or an error.
cudaError_t kmgb_make_tmap_2d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype,
                              int elem_bytes, uint64_t cols, uint64_t rows, uint64_t row_stride_bytes,
                              uint32_t box_cols, uint32_t box_rows);
// The same with a given swizzle (the box's inner extent at most the swizzle width).
cudaError_t kmgb_make_tmap_2d_swz(CUtensorMap* map, const void* base, CUtensorMapDataType dtype,
                                  int elem_bytes, uint64_t cols, uint64_t rows,
                                  uint64_t row_stride_bytes, uint32_t box_cols, uint32_t box_rows,
                                  CUtensorMapSwizzle swizzle);

// Number of kernels this library has launched (process-wide), for launch accounting.
namespace kmgb {
void count_launches(long long n);
long long launch_count();
}  // namespace kmgb

#define KMGB_CUDA_TRY(expr)                        \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return _e;              \
  } while (0)
