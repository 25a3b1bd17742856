// Test infrastructure: runs the REFERENCE's own assignment, center and compactness kernels on
// the GPU.
//
// The reference's ClosestCenters.cu (main/cuda/ClosestCenters.cu) is compiled from its sources
// into a cubin for sm_103a (oracle/__init__.py build_ref(), with oracle/ref_shfl_shim.h
// force-included). The reference's sources exist only in the development container, whose host
// binaries are x86 and cannot run on the Arm GPU host (and its host driver, main/cpp/kmeans.cpp,
// also needs a CMake-generated config.h and cuBLAS), so device code travels as a cubin and this
// loader, built on the GPU host from this repository, takes the host side's place: it loads the cubin with the CUDA driver API, finds the kernel instantiations the
// reference's float entry uses (`_dev_ClosestCentersBegin<float, float4, DELTA, 4>`, DELTA =
// 1..16, and `_dev_ClosestCentersEndNew<float>`), sets the reference's __constant__ shape
// variables and launches them with the reference's grid (ClosestCenters.cu:181-231, 312-315:
// 16x16 threads per 64x64 tile, DELTA = D - 16*(ceil(D/16)-1), then SMs*8 blocks of 128 threads
// for the final arg-min over the column-block partials). Only tests/ and the reference arm of
// bench.py use it, to pin the oracle's assignment rule against the reference's kernels and to
// time them.
//
// Buffer contract (the reference's kernels read past the logical matrices; see the harness in
// tests/test_gpu_reference_kernels.py): A holds round_up(n, 64) + 1 rows of d floats plus 16 more
// floats, B is d x k with 16 spare rows after it, k % 4 == 0, C and Cindices hold
// ceil(k/64) x n entries.
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <cxxabi.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

namespace {

PFN_cuModuleLoad_v2000 p_load = nullptr;
PFN_cuModuleGetFunctionCount_v12040 p_count = nullptr;
PFN_cuModuleEnumerateFunctions_v12040 p_enum = nullptr;
PFN_cuFuncGetName_v12030 p_name = nullptr;
PFN_cuModuleGetGlobal_v3020 p_global = nullptr;
PFN_cuLaunchKernel_v4000 p_launch = nullptr;
PFN_cuMemcpyHtoD_v3020 p_htod = nullptr;

CUmodule g_mod = nullptr;
CUfunction g_begin[17] = {};
CUfunction g_end = nullptr;
// ClusterCenters.cu / Compactness.cu: _dev_ClusterCentersBegin/End<float>,
// _dev_Compactness/_dev_CompactnessEnd<float, 128>
CUmodule g_mod_cc = nullptr, g_mod_cp = nullptr;
CUfunction g_cc_begin = nullptr, g_cc_end = nullptr, g_cp = nullptr, g_cp_end = nullptr;
char g_err[512] = "";

template <typename F>
bool entry(const char* name, int version, F* out) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p) {
    std::snprintf(g_err, sizeof(g_err), "driver entry point %s unavailable", name);
    return false;
  }
  *out = reinterpret_cast<F>(p);
  return true;
}

int set_const(const char* name, int value) {
  CUdeviceptr d = 0;
  size_t bytes = 0;
  if (p_global(&d, &bytes, g_mod, name) != CUDA_SUCCESS || bytes != sizeof(int)) {
    std::snprintf(g_err, sizeof(g_err), "constant %s not found in the cubin", name);
    return -1;
  }
  if (p_htod(d, &value, sizeof(int)) != CUDA_SUCCESS) {
    std::snprintf(g_err, sizeof(g_err), "setting constant %s failed", name);
    return -1;
  }
  return 0;
}

std::string demangled(CUfunction f) {
  const char* mangled = nullptr;
  if (p_name(&mangled, f) != CUDA_SUCCESS || !mangled) return std::string();
  int st = 0;
  char* dem = abi::__cxa_demangle(mangled, nullptr, nullptr, &st);
  const std::string s = (st == 0 && dem) ? std::string(dem) : std::string(mangled);
  std::free(dem);
  return s;
}

// Loads a cubin and returns the functions whose demangled names start with the given prefixes.
int load_named(const char* path, CUmodule* mod, const char* const* prefixes, CUfunction* out,
               int count) {
  if (p_load(mod, path) != CUDA_SUCCESS) {
    std::snprintf(g_err, sizeof(g_err), "cuModuleLoad(%s) failed", path);
    return -1;
  }
  unsigned int n = 0;
  if (p_count(&n, *mod) != CUDA_SUCCESS || n == 0 || n > 4096) return -1;
  CUfunction* fs = static_cast<CUfunction*>(std::calloc(n, sizeof(CUfunction)));
  if (!fs || p_enum(fs, n, *mod) != CUDA_SUCCESS) {
    std::free(fs);
    return -1;
  }
  int found = 0;
  for (unsigned int i = 0; i < n; ++i) {
    const std::string name = demangled(fs[i]);
    for (int j = 0; j < count; ++j)
      if (!out[j] && name.compare(0, std::strlen(prefixes[j]), prefixes[j]) == 0) {
        out[j] = fs[i];
        ++found;
      }
  }
  std::free(fs);
  return found;
}

int num_sms() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace

extern "C" {

const char* refk_last_error() { return g_err; }

// Loads the cubin into the current device's primary context. Returns the number of kernel
// instantiations found (17 expected: DELTA 1..16 and the final reduction), or -1.
int refk_load(const char* cubin_path) {
  if (cudaFree(nullptr) != cudaSuccess) {
    std::snprintf(g_err, sizeof(g_err), "CUDA runtime initialisation failed");
    return -1;
  }
  if (!entry("cuModuleLoad", 2000, &p_load) || !entry("cuModuleGetFunctionCount", 12040, &p_count) ||
      !entry("cuModuleEnumerateFunctions", 12040, &p_enum) ||
      !entry("cuFuncGetName", 12030, &p_name) || !entry("cuModuleGetGlobal", 3020, &p_global) ||
      !entry("cuLaunchKernel", 4000, &p_launch) || !entry("cuMemcpyHtoD", 3020, &p_htod))
    return -1;
  if (p_load(&g_mod, cubin_path) != CUDA_SUCCESS) {
    std::snprintf(g_err, sizeof(g_err), "cuModuleLoad(%s) failed", cubin_path);
    return -1;
  }
  unsigned int n = 0;
  if (p_count(&n, g_mod) != CUDA_SUCCESS || n == 0 || n > 4096) {
    std::snprintf(g_err, sizeof(g_err), "no kernels in the cubin");
    return -1;
  }
  CUfunction* fs = static_cast<CUfunction*>(std::calloc(n, sizeof(CUfunction)));
  if (!fs || p_enum(fs, n, g_mod) != CUDA_SUCCESS) {
    std::free(fs);
    std::snprintf(g_err, sizeof(g_err), "cuModuleEnumerateFunctions failed");
    return -1;
  }
  int found = 0;
  const std::string begin_prefix = "void _dev_ClosestCentersBegin<float, float4, ";
  const std::string end_prefix = "void _dev_ClosestCentersEndNew<float>(";
  for (unsigned int i = 0; i < n; ++i) {
    const std::string s = demangled(fs[i]);
    if (s.compare(0, begin_prefix.size(), begin_prefix) == 0) {
      int delta = 0, unroll = 0;
      if (std::sscanf(s.c_str() + begin_prefix.size(), "%d, %d>", &delta, &unroll) == 2 &&
          unroll == 4 && delta >= 1 && delta <= 16 && !g_begin[delta]) {
        g_begin[delta] = fs[i];
        ++found;
      }
    } else if (s.compare(0, end_prefix.size(), end_prefix) == 0 && !g_end) {
      g_end = fs[i];
      ++found;
    }
  }
  std::free(fs);
  return found;
}

// The reference's ClosestCentersF with Bpadded = NULL (ClosestCenters.cu:181-231, 312-315,
// 391-401): labels[m0 + i] = arg-min_j (||c_j||^2 - 2 a_i.c_j) in the reference's FP32
// arithmetic. A: n x d (row-major), B: d x k, normB: k. Launches on the legacy default stream.
int refk_closest_centers_f(int m0, int n, int d, const float* A, int k, const float* B,
                           const float* normB, int ncolsc, float* C, int* Cidx, int* labels) {
  if (!g_mod || !g_end) {
    std::snprintf(g_err, sizeof(g_err), "cubin not loaded");
    return -1;
  }
  if (n <= 0 || d <= 0 || k <= 0 || (k % 4) != 0) {
    std::snprintf(g_err, sizeof(g_err), "unsupported shape (k must be a multiple of 4)");
    return -1;
  }
  const int unroll = 4, tile = 16;
  const int nby = (n + unroll * tile - 1) / (unroll * tile);
  const int nbx = (k + unroll * tile - 1) / (unroll * tile);
  if (ncolsc < nbx) {
    std::snprintf(g_err, sizeof(g_err), "ncolsc must be >= ceil(k/64)");
    return -1;
  }
  int nt = (d + tile - 1) / tile;
  const int delta = d - (nt - 1) * tile;
  nt -= 1;
  if (!g_begin[delta]) {
    std::snprintf(g_err, sizeof(g_err), "no kernel for DELTA=%d", delta);
    return -1;
  }
  const int rows_padded = nby * unroll * tile;
  if (set_const("dev_N", nt) || set_const("dev_nRowsA", n) ||
      set_const("dev_nRowsAPadded", rows_padded) || set_const("dev_nColsA", d) ||
      set_const("dev_nRowsB", d) || set_const("dev_nColsB", k) || set_const("dev_nColsC", ncolsc) ||
      set_const("ASTRIDE", d) || set_const("dev_nColsBPadded", k) || set_const("BSTRIDE", k * tile))
    return -1;
  void* a_begin[] = {&A, &B, &normB, &C, &Cidx};
  if (p_launch(g_begin[delta], (unsigned)nbx, (unsigned)nby, 1, tile, tile, 1, 0, nullptr, a_begin,
               nullptr) != CUDA_SUCCESS) {
    std::snprintf(g_err, sizeof(g_err), "launch of the reference's ClosestCentersBegin failed");
    return -1;
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  void* a_end[] = {&m0, &n, &C, &Cidx, &labels};
  if (p_launch(g_end, (unsigned)(sms * 8), 1, 1, 128, 1, 1, 0, nullptr, a_end, nullptr) !=
      CUDA_SUCCESS) {
    std::snprintf(g_err, sizeof(g_err), "launch of the reference's ClosestCentersEndNew failed");
    return -1;
  }
  return 0;
}

// Loads the reference's ClusterCenters.cu and Compactness.cu cubins (after refk_load). Returns
// the number of kernels found (4 expected) or -1.
int refk_load_update(const char* cluster_cubin, const char* compact_cubin) {
  if (!p_load) {
    std::snprintf(g_err, sizeof(g_err), "refk_load first");
    return -1;
  }
  const char* cc_names[2] = {"void _dev_ClusterCentersBegin<float>(",
                             "void _dev_ClusterCentersEnd<float>("};
  CUfunction cc[2] = {nullptr, nullptr};
  const char* cp_names[2] = {"void _dev_Compactness<float, 128>(",
                             "void _dev_CompactnessEnd<float, 128>("};
  CUfunction cp[2] = {nullptr, nullptr};
  const int a = load_named(cluster_cubin, &g_mod_cc, cc_names, cc, 2);
  const int b = load_named(compact_cubin, &g_mod_cp, cp_names, cp, 2);
  if (a < 0 || b < 0) return -1;
  g_cc_begin = cc[0];
  g_cc_end = cc[1];
  g_cp = cp[0];
  g_cp_end = cp[1];
  return a + b;
}

// The reference's ClusterCentersF over one tile holding all m rows (lastTile; ClusterCenters.cu:
// 101-133): 128-thread blocks, SMs*8 of them accumulate FP32 partial sums and counts per block
// into centers_large (p x k x n) and counts_large (p x k), which the caller zeroes; then one
// block per center adds the p partials and divides (0/0 = NaN for an empty cluster).
int refk_cluster_centers_f(int m, int n, int k, const float* data, const int* labels,
                           float* centers_large, int* counts_large, float* centers, int* counts) {
  if (!g_cc_begin || !g_cc_end) {
    std::snprintf(g_err, sizeof(g_err), "update cubins not loaded");
    return -1;
  }
  int m0 = 0;
  int p = num_sms() * 8;
  void* a1[] = {&m0, &m, &n, &k, &data, &labels, &centers_large, &counts_large};
  if (p_launch(g_cc_begin, (unsigned)p, 1, 1, 128, 1, 1, 0, nullptr, a1, nullptr) != CUDA_SUCCESS)
    return -1;
  void* a2[] = {&p, &n, &k, &centers_large, &counts_large, &centers, &counts};
  const unsigned shm = (unsigned)(n * sizeof(float) + sizeof(int));
  if (p_launch(g_cc_end, (unsigned)k, 1, 1, 128, 1, 1, shm, nullptr, a2, nullptr) != CUDA_SUCCESS)
    return -1;
  return 0;
}

// The reference's CompactnessF over one tile (Compactness.cu:70-96): SMs*8 blocks of 128
// threads add sum_d (x_d - c_label,d)^2 of their rows into compactness[block] (FP32; the caller
// zeroes p entries), then one block sums the p partials into compactness[0].
int refk_compactness_f(int m, int n, int k, const float* data, const int* labels,
                       const float* centers, float* compactness) {
  if (!g_cp || !g_cp_end) {
    std::snprintf(g_err, sizeof(g_err), "update cubins not loaded");
    return -1;
  }
  int m0 = 0;
  int p = num_sms() * 8;
  void* a1[] = {&m0, &m, &n, &k, &data, &labels, &centers, &compactness};
  if (p_launch(g_cp, (unsigned)p, 1, 1, 128, 1, 1, 0, nullptr, a1, nullptr) != CUDA_SUCCESS)
    return -1;
  void* a2[] = {&p, &compactness};
  if (p_launch(g_cp_end, 1, 1, 1, 128, 1, 1, 0, nullptr, a2, nullptr) != CUDA_SUCCESS) return -1;
  return 0;
}

}  // extern "C"
