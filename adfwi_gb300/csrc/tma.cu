// Host side of the TMA helpers: tensor-map encoding through the driver entry point.
#include <mutex>

#include "tma.cuh"

namespace adfwi {

EncodeTiledFn encode_tiled_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e == cudaSuccess && q == cudaDriverEntryPointSuccess) fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  if (fn == nullptr) set_error("cuTensorMapEncodeTiled is not available from the CUDA driver");
  return fn;
}

int make_plane_map(CUtensorMap* map, const void* base, int elem_bytes, const Layout& L, int64_t nplanes, int box_x,
                   int box_y) {
  EncodeTiledFn enc = encode_tiled_fn();
  if (enc == nullptr) return kUnsupported;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0) {
    set_error("tensor map base %p is not 16-byte aligned", base);
    return kBadArgument;
  }
  cuuint64_t dims[3] = {(cuuint64_t)L.pitch, (cuuint64_t)L.rows, (cuuint64_t)nplanes};
  cuuint64_t strides[2] = {(cuuint64_t)L.pitch * elem_bytes, (cuuint64_t)L.plane * elem_bytes};
  cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_y, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUtensorMapDataType dt = elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  CUresult r = enc(map, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d) for a %dx%d box over %lldx%dx%d", (int)r, box_x, box_y,
              (long long)nplanes, L.rows, L.pitch);
    return kCudaError;
  }
  return kOk;
}

}  // namespace adfwi
