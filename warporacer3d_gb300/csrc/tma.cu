// TMA tensor-map encoding through the driver entry point, resolved at run
// time (cudaGetDriverEntryPointByVersion), so the library links without
// libcuda and still loads on a machine without a GPU.
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "tma.h"

namespace racer {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int make_tmap_bf16(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    racer_host::set_error("cuTensorMapEncodeTiled is unavailable");
    return 2;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((ld * 2) & 15) || box_rows == 0 || box_rows > 256) {
    racer_host::set_error("tensor map: base must be 16-byte aligned, rows 16-byte multiples, box <= 256 rows");
    return 1;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {ld * 2};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t elem[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    racer_host::set_error("cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    return 2;
  }
  return 0;
}

int make_tmap_f32(CUtensorMap* map, const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_cols,
                  uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    racer_host::set_error("cuTensorMapEncodeTiled is unavailable");
    return 2;
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) || ((ld * 4) & 15) || box_cols == 0 || box_cols > 256 ||
      ((box_cols * 4) & 15) || box_rows == 0 || box_rows > 256) {
    racer_host::set_error("tensor map: base and rows must be 16-byte aligned, boxes of 16-byte rows up to 256");
    return 1;
  }
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {ld * 4};
  cuuint32_t box[2] = {box_cols, box_rows};
  cuuint32_t elem[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    racer_host::set_error("cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    return 2;
  }
  return 0;
}

}  // namespace racer
