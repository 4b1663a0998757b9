// TMA (cp.async.bulk.tensor) and mbarrier helpers for sm_103a, written as inline PTX.
//
// Host: tensor maps are encoded with cuTensorMapEncodeTiled, reached through
// cudaGetDriverEntryPoint so the library needs no link-time dependency on libcuda.
// Device: every wait on an mbarrier is bounded; a wait that runs out records an error code
// in a device flag and reports failure to its caller, which leaves the kernel without
// touching the data it was waiting for.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace adfwi {

// ---------------------------------------------------------------------------- host side
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled_fn();  // nullptr (with the error set) if the driver lacks it

// 3-D map over `nplanes` pitched planes: x = column (pitch elements), y = row, z = plane.
// The box is box_x columns by box_y rows of one plane.
int make_plane_map(CUtensorMap* map, const void* base, int elem_bytes, const Layout& L, int64_t nplanes,
                   int box_x, int box_y);

// ---------------------------------------------------------------------------- device side
// Bounded spin: a wait gives up after kWaitNs nanoseconds of the global timer (far beyond any
// legitimate wait; one try_wait may itself suspend the thread for a while, so the bound is
// on elapsed time, not on the number of polls).
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// `count` arrivals at once (release semantics at CTA scope, like every arrive here).
__device__ __forceinline__ void mbar_arrive_cnt(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Wait for the phase with the given parity to complete. Returns false once `limit_ns` of the
// global timer have passed.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
  const uint32_t a = smem_u32(bar);
  unsigned long long t0 = 0;
  for (unsigned n = 0;; ++n) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((n & 63) == 63) {
      const unsigned long long t = global_ns();
      if (t0 == 0)
        t0 = t;
      else if (t - t0 > limit_ns)
        return false;
    }
  }
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) { return mbar_wait_for(bar, parity, kWaitNs); }

// One 3-D tile load into shared memory, completing on `bar` (complete_tx in bytes).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Named barrier among `count` threads (count a multiple of 32), id 1..15.
__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Device error flag codes (written by kernels, read by the host after a solve).
constexpr int kErrWaitTimeout = 1;

__device__ __forceinline__ void raise_flag(int* flag, int code) {
  if (flag) atomicExch(flag, code);
}

}  // namespace adfwi
