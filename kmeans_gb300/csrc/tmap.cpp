// Host-side TMA tensor-map encoding through the driver entry point (no -lcuda link needed).
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}
}  // namespace

cudaError_t kmgb_make_tmap_2d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype,
                              int elem_bytes, uint64_t cols, uint64_t rows,
                              uint64_t row_stride_bytes, uint32_t box_cols, uint32_t box_rows) {
  return kmgb_make_tmap_2d_swz(map, base, dtype, elem_bytes, cols, rows, row_stride_bytes,
                               box_cols, box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

cudaError_t kmgb_make_tmap_2d_swz(CUtensorMap* map, const void* base, CUtensorMapDataType dtype,
                                  int elem_bytes, uint64_t cols, uint64_t rows,
                                  uint64_t row_stride_bytes, uint32_t box_cols, uint32_t box_rows,
                                  CUtensorMapSwizzle swizzle) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  const uint32_t width = swizzle == CU_TENSOR_MAP_SWIZZLE_32B ? 32
                       : swizzle == CU_TENSOR_MAP_SWIZZLE_64B ? 64 : 128;
  if (box_cols * (uint32_t)elem_bytes > width || box_rows > 256 || (row_stride_bytes % 16) ||
      (reinterpret_cast<uintptr_t>(base) & 15))
    return cudaErrorInvalidValue;
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {row_stride_bytes};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}
