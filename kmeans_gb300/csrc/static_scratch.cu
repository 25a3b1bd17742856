// ClusterCentersF for callers that cannot allocate device memory.
//
// ClusterCentersF needs working memory for its deterministic update (the label histogram, the
// label-sorted point ids and the FP64 per-piece partial sums) and takes it from the
// stream-ordered allocator on every call. Some callers cannot let a library allocate: programs
// that reserve all device memory up front and forbid allocation afterwards (real-time and
// embedded loops, services whose memory pool owns the whole GPU), or code that must not touch the
// allocator at all on its hot path. This variant takes its working memory from a fixed array in
// device global memory instead.
//
// The array is a file-scope __device__ object of KMGB_NOALLOC_SCRATCH_BYTES (8 MiB): every GPU
// that loads the library holds it until the process exits. In host code the array's name is a
// host-side stand-in, not a device address, so its device address is looked up once per device
// with cudaGetSymbolAddress (with that device current) and cached. The first call on a device
// performs that lookup; make that first call before any stream capture. The cached address
// belongs to the device's primary context: after cudaDeviceReset (or anything else that destroys
// that context) the module is loaded again and the array may sit elsewhere, so a reset drops the
// cache (the lookup is keyed on the context that is current when the call is made).
//
// All calls share the one array and it keeps the last call's contents; everything that must start
// at zero (the histogram) is cleared by the call itself. Calls that overlap on the GPU (different
// streams or threads, or ClusterCentersF_noalloc calls queued from several host threads) race on
// the array and must be serialised by the caller. Sizes whose working memory exceeds the array
// are rejected with ERROR_CLUSTERCENTERS and a message from kmgb_last_error().
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/kmeans_gb300.h"
#include "common.cuh"
#include "kernels.h"

#define KMGB_NOALLOC_SCRATCH_BYTES (8u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[KMGB_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};  // context the cached address belongs to

// The current driver context (through the runtime's driver entry point: no -lcuda link).
CUcontext current_context() {
  static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
  });
  CUcontext ctx = nullptr;
  if (!fn || fn(&ctx) != CUDA_SUCCESS) return nullptr;
  return ctx;
}

// Device address of the scratch array on the current device, looked up once per device and
// context: a new primary context (after a device reset) gets a fresh lookup.
cudaError_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  // null until the runtime has made the device's primary context current
  const CUcontext ctx = current_context();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!ctx || !g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // also initialises the context
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
    g_scratch_ctx[dev] = current_context();
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

size_t align256(size_t v) { return (v + 255) & ~static_cast<size_t>(255); }

}  // namespace

extern "C" kmeansCudaErrorStatus ClusterCentersF_noalloc(const int m0, const int m, const int n,
                                                         const int k, const bool lastTile,
                                                         const float* data, const int* indices,
                                                         float* centers_large, int* counts_large,
                                                         float* centers, int* counts) {
  using namespace kmgb;
  if (m < 0 || n <= 0 || k <= 0 || !centers_large || !counts_large || (m > 0 && (!data || !indices)))
    return ERROR_CLUSTERCENTERS;
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
  // carve the working memory out of the fixed array
  const size_t o_hist = 0;
  const size_t o_scan = o_hist + align256(sizeof(int) * (size_t)hist_elems);
  const size_t o_off = o_scan + align256(sizeof(int) * update_scan_tmp_elems(
                                                           hist_elems > k + 1 ? hist_elems : k + 1));
  const size_t o_pcnt = o_off + align256(sizeof(int) * (size_t)(k + 1));
  const size_t o_sorted = o_pcnt + align256(sizeof(int) * (size_t)(k + 1));
  const size_t o_part = o_sorted + align256(sizeof(int) * (size_t)(m > 0 ? m : 1));
  const size_t total = o_part + align256(sizeof(double) * (size_t)w.max_pieces * n);
  const cudaStream_t stream = 0;  // the reference's per-kernel entries run on the default stream
  cudaError_t e = cudaSuccess;
  // only a call with rows uses the working memory: a finalize-only call (m == 0, lastTile) is
  // accepted at any size, as ClusterCentersF accepts it
  if (m > 0) {
    if (total > KMGB_NOALLOC_SCRATCH_BYTES) {
      set_last_error("ClusterCentersF_noalloc: this m, n, k needs more working memory than the "
                     "8 MiB static scratch array holds");
      return ERROR_CLUSTERCENTERS;
    }
    void* base = nullptr;
    if (scratch_address(&base) != cudaSuccess) {
      set_last_error("ClusterCentersF_noalloc: cudaGetSymbolAddress of the scratch array failed");
      return ERROR_CLUSTERCENTERS;
    }
    unsigned char* s = static_cast<unsigned char*>(base);
    w.hist = reinterpret_cast<int*>(s + o_hist);
    w.scan_tmp = reinterpret_cast<int*>(s + o_scan);
    w.label_off = reinterpret_cast<int*>(s + o_off);
    w.piece_cnt = reinterpret_cast<int*>(s + o_pcnt);
    w.sorted = reinterpret_cast<int*>(s + o_sorted);
    w.part = reinterpret_cast<double*>(s + o_part);
    // clears the histogram itself before counting
    e = launch_tile_accumulate<float>(data, n, indices + m0, w, acc, counts_large, stream);
  }
  if (e == cudaSuccess && lastTile)
    e = launch_finalize_acc<float>(acc, counts_large, k, n, centers, counts, stream);
  return e == cudaSuccess ? NO_ERROR : ERROR_CLUSTERCENTERS;
}
