// Host side of the TMA helpers (tensor-map encoding through the driver entry point) and the
// self-test of the bounded mbarrier waits.
#include <mutex>

#include "../../include/adfwi_gb300.h"
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

// ---------------------------------------------------------------------------------------
// Self-test of the bounded waits: one block waits on phase 0 of a fresh mbarrier that nothing
// arrives at, through the same wait loop as the pipelined kernels, so the wait runs out after
// `limit_ns` and the kernel raises the error flag and returns (no trap, no unbounded spin).
namespace adfwi {
namespace {
__global__ void wait_selftest(unsigned long long limit_ns, int* flag) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !mbar_wait_for(&bar, 0, limit_ns)) raise_flag(flag, kErrWaitTimeout);
}
}  // namespace
}  // namespace adfwi

extern "C" int adfwi_wait_selftest(int64_t limit_ns, int32_t* flag, void* stream) {
  using namespace adfwi;
  ADFWI_CHECK_ARG(flag != nullptr, "null flag");
  ADFWI_CHECK_ARG(limit_ns > 0 && limit_ns <= 2000000000ll, "limit_ns must be in (0, 2 s]");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  ADFWI_LAUNCH(kAux, st, (wait_selftest<<<1, 32, 0, st>>>((unsigned long long)limit_ns, reinterpret_cast<int*>(flag))));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}
