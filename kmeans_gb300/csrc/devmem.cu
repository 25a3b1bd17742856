// Device memory of handles: one stream-ordered memory pool per device, owned by the library.
//
// A handle's fixed buffers are one arena (engine.cu). With cudaMalloc/cudaFree a one-shot call
// on the 4M x 128, K=1024 workload spent ~1 ms allocating and ~3.3 ms freeing its ~7 GB (the
// free synchronizes the device and unmaps). Here the arena comes from a pool whose release
// threshold is unbounded: cudaFreeAsync hands the memory back to the pool, and the next handle
// of the same or a smaller size takes it again without mapping anything. The pool keeps what it
// holds until kmgb_release_cached_memory() (or a failed allocation, which trims it and retries
// once); KMGB_POOL=0 trims after every free, which gives back cudaMalloc/cudaFree behaviour.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "../../include/kmeans_gb300.h"
#include "kernels.h"

namespace kmgb {
namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
cudaMemPool_t g_pools[kMaxDevices] = {};

bool keep_freed_memory() {
  static const bool keep = [] {
    const char* v = std::getenv("KMGB_POOL");
    return !(v && std::strcmp(v, "0") == 0);
  }();
  return keep;
}

cudaError_t pool_of_current_device(cudaMemPool_t* out) {
  int dev = 0;
  cudaError_t r = cudaGetDevice(&dev);
  if (r != cudaSuccess) return r;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_pools[dev]) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    r = cudaMemPoolCreate(&p, &props);
    if (r != cudaSuccess) return r;
    uint64_t threshold = UINT64_MAX;
    r = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &threshold);
    if (r != cudaSuccess) {
      cudaMemPoolDestroy(p);
      return r;
    }
    g_pools[dev] = p;
  }
  *out = g_pools[dev];
  return cudaSuccess;
}

}  // namespace

// Test hooks: a countdown per event kind; the event that brings it to zero fails once.
std::atomic<long long> g_fail_countdown[4];
std::atomic<long long> g_test_withhold{0};
std::atomic<unsigned long long> g_test_wait{0};

bool inject_fault(int kind) {
  if (kind < 1 || kind > 3) return false;
  long long v = g_fail_countdown[kind].load(std::memory_order_relaxed);
  while (v > 0) {
    if (g_fail_countdown[kind].compare_exchange_weak(v, v - 1, std::memory_order_relaxed))
      return v == 1;
  }
  return false;
}

void test_wait_hook(long long* withhold, unsigned long long* wait_cycles) {
  *withhold = g_test_withhold.load(std::memory_order_relaxed);
  *wait_cycles = g_test_wait.load(std::memory_order_relaxed);
}

int num_sms() {
  static std::atomic<int> cached[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 148;
  int v = cached[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 148;  // any positive count only sizes grids; every kernel strides over its work
    cached[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s) {
  *p = nullptr;
  if (inject_fault(kFaultAlloc)) return cudaErrorMemoryAllocation;
  if (bytes == 0) bytes = 1;
  cudaMemPool_t pool = nullptr;
  cudaError_t r = pool_of_current_device(&pool);
  if (r != cudaSuccess) return r;
  r = cudaMallocFromPoolAsync(p, bytes, pool, s);
  if (r == cudaErrorMemoryAllocation) {
    // memory the pool holds but nobody uses goes back to the device, then one more try
    cudaGetLastError();
    cudaDeviceSynchronize();
    cudaMemPoolTrimTo(pool, 0);
    r = cudaMallocFromPoolAsync(p, bytes, pool, s);
  }
  if (r != cudaSuccess) {
    *p = nullptr;
    return r;
  }
  // usable from every stream (copies on the legacy stream, a handle's copy stream) at once
  return cudaStreamSynchronize(s);
}

void dev_free(void* p, cudaStream_t s) {
  if (!p) return;
  cudaFreeAsync(p, s);
  if (!keep_freed_memory()) {
    cudaStreamSynchronize(s);
    cudaMemPool_t pool = nullptr;
    if (pool_of_current_device(&pool) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
  }
}

cudaError_t dev_release_cached() {
  cudaError_t r = cudaDeviceSynchronize();
  std::lock_guard<std::mutex> g(g_mu);
  for (int d = 0; d < kMaxDevices; ++d)
    if (g_pools[d]) {
      const cudaError_t t = cudaMemPoolTrimTo(g_pools[d], 0);
      if (r == cudaSuccess) r = t;
    }
  return r;
}

}  // namespace kmgb

extern "C" {

void kmgb_debug_fail_nth(int kind, long long nth) {
  if (kind < 1 || kind > 3) return;
  kmgb::g_fail_countdown[kind].store(nth > 0 ? nth : 0, std::memory_order_relaxed);
}

void kmgb_debug_withhold_stage(long long stage, unsigned long long wait_cycles) {
  kmgb::g_test_withhold.store(stage > 0 ? stage : 0, std::memory_order_relaxed);
  kmgb::g_test_wait.store(stage > 0 ? wait_cycles : 0, std::memory_order_relaxed);
}

long long kmgb_debug_pool_used_bytes(void) {
  cudaMemPool_t pool = nullptr;
  if (kmgb::pool_of_current_device(&pool) != cudaSuccess) return -1;
  uint64_t used = 0;
  if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess) return -1;
  return (long long)used;
}

int kmgb_release_cached_memory(void) {
  const cudaError_t r = kmgb::dev_release_cached();
  if (r != cudaSuccess) {
    kmgb::set_last_error(cudaGetErrorString(r));
    return 1;
  }
  return 0;
}

}  // extern "C"
