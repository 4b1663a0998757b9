// Zeroing of the ghost frames of pitched planes.
//
// Every stencil reads a cell's neighbours without bounds checks, so the cells outside the
// nzp x nxp interior of any plane a kernel reads must hold zero. The kernels only ever write
// interior cells, so a plane's frame stays zero once cleared. Planes whose memory comes
// straight from the caller's workspace and is written by a solve before it is read (the
// wavefield histories) are cleared by this kernel at the start of the solve that first uses
// them; it writes the frame only, about (pitch x rows - nzp x nxp) / (pitch x rows) of the
// plane.
#pragma once
#include <algorithm>
#include <cuda_runtime.h>

#include "common.cuh"

namespace adfwi {

// Per plane the frame is nzp + 1 contiguous runs: [0, GZ*pitch + GX) (the top ghost rows and
// the left ghosts of interior row 0); for k = 1 .. nzp-1 the run from the end of interior row
// k-1 to the start of row k; and the run from the end of the last interior row to the end of
// the plane. One warp clears one run at a time.
template <typename T>
__global__ void __launch_bounds__(256) zero_frames_kernel(T* __restrict__ base, int64_t nplanes, Layout L) {
  const int64_t per = (int64_t)L.nzp + 1;
  const int64_t runs = per * nplanes;
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w0; r < runs; r += nw) {
    const int64_t pl = r / per;
    const int k = (int)(r - pl * per);
    int64_t beg, end;
    if (k == 0) {
      beg = 0;
      end = (int64_t)GZ * L.pitch + GX;
    } else if (k == L.nzp) {
      beg = (int64_t)(GZ + L.nzp - 1) * L.pitch + GX + L.nxp;
      end = L.plane;
    } else {
      beg = (int64_t)(GZ + k - 1) * L.pitch + GX + L.nxp;
      end = (int64_t)(GZ + k) * L.pitch + GX;
    }
    T* p = base + pl * L.plane;
    for (int64_t e = beg + lane; e < end; e += 32) p[e] = T(0);
  }
}

template <typename T>
int zero_frames(T* base, int64_t nplanes, const Layout& L, cudaStream_t st) {
  if (nplanes <= 0) return kOk;
  const int64_t runs = ((int64_t)L.nzp + 1) * nplanes;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((runs + 7) / 8, 152 * 16));
  ADFWI_LAUNCH(kAux, st, (zero_frames_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(base, nplanes, L)));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace adfwi
