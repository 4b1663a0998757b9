// Shared definitions for the adfwi_gb300 CUDA library (sm_103a).
//
// Storage layout of one wavefield / coefficient plane (nzp x nxp cells):
// rows are padded to a 128-byte multiple pitch and surrounded by ghost cells
// that are zero forever, so that every stencil read of a tile and its halo stays
// inside the allocation without a bounds check:
//
//     element (i, j) of a plane lives at  (i + GZ) * pitch + (j + GX)
//
// with GZ = 4 ghost rows on top, GX = 4 ghost columns on the left, and at least
// TILE + 4 ghost rows / columns at the bottom / right. A shot's fields are
// consecutive planes; all shots of one field form one block of ns planes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "profile.cuh"

namespace adfwi {

constexpr int GZ = 4;
constexpr int GX = 4;

struct Layout {
  int nzp, nxp;    // grid cells (rows, columns)
  int rows;        // allocated rows per plane
  int pitch;       // allocated elements per row
  int64_t plane;   // rows * pitch

  __host__ __device__ __forceinline__ int64_t off(int i, int j) const {
    return (int64_t)(i + GZ) * pitch + (j + GX);
  }
};

// Host: layout for a grid processed by tiles of tz x tx cells.
inline Layout make_layout(int nzp, int nxp, int tz, int tx, int elem_bytes) {
  Layout L;
  L.nzp = nzp;
  L.nxp = nxp;
  L.rows = GZ + nzp + tz + 4;
  int align = 128 / elem_bytes;
  int need = GX + nxp + tx + 4;
  L.pitch = (need + align - 1) / align * align;
  L.plane = (int64_t)L.rows * L.pitch;
  return L;
}

// Status codes returned by every C-ABI entry point (0 = success).
enum Status : int {
  kOk = 0,
  kBadArgument = -1,
  kBadGeometry = -2,
  kWorkspaceTooSmall = -3,
  kCudaError = -4,
  kUnsupported = -5,
  kNonFinite = -6,
};

// Thread-local last-error text, read through adfwi_last_error().
void set_error(const char* fmt, ...);

// Host copy of a plan's tables, page-locked when the CUDA runtime can give page-locked
// memory. Uploading from page-locked memory is a stream-ordered asynchronous copy (a
// pageable source makes the copy wait for the stream), so a solve enqueues without host
// stalls and can be captured into a CUDA graph. Without a device (plans built on a host
// without a GPU, for sizing) the copy is ordinary heap memory.
struct PinnedBytes {
  void* ptr = nullptr;
  size_t bytes = 0;
  bool pinned = false;
  PinnedBytes() = default;
  PinnedBytes(const PinnedBytes&) = delete;
  PinnedBytes& operator=(const PinnedBytes&) = delete;
  ~PinnedBytes() { release(); }
  void release();
  // Copies n bytes from src; returns false (with the error text set) when no host memory
  // can be had at all.
  bool assign(const void* src, size_t n);
};

// Programmatic dependent launch. A step kernel is launched with programmatic stream
// serialisation, so its blocks may become resident while the previous step kernel's last
// blocks still run: every block signals at once that the next launch may start
// (launch_dependents), and waits for the previous grid's completion and memory (wait)
// before its first read of the fields and its first write of anything. In a kernel launched
// without the attribute both are no-ops.
__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Host: launch `kernel` with programmatic stream serialisation (the kernel must call
// griddep_wait() before it touches data of the previous launch on the stream).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl_kernel(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

}  // namespace adfwi

#define ADFWI_CUDA_TRY(expr)                                                      \
  do {                                                                            \
    cudaError_t e__ = (expr);                                                     \
    if (e__ != cudaSuccess) {                                                     \
      ::adfwi::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e__), \
                         __FILE__, __LINE__);                                     \
      return ::adfwi::kCudaError;                                                 \
    }                                                                             \
  } while (0)

// Launch a kernel under the library's launch accounting (see profile.cuh).
#define ADFWI_LAUNCH(cls, st, launch)                          \
  do {                                                         \
    int tok__ = ::adfwi::prof_before((cls), (st));             \
    launch;                                                    \
    ::adfwi::prof_after((cls), (st), tok__);                   \
  } while (0)

#define ADFWI_CHECK_ARG(cond, ...)         \
  do {                                     \
    if (!(cond)) {                         \
      ::adfwi::set_error(__VA_ARGS__);     \
      return ::adfwi::kBadArgument;        \
    }                                      \
  } while (0)
