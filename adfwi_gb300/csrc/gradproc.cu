// Gaussian smoothing of model-sized planes for the gradient processor (sm_103a, FP64).
//
// Reference (paths inside liufeng2317/ADFWI): ADFWI/propagator/gradient_process.py:14-49
// (gauss2, smooth2d) as used by GradProcessor.forward (74-134) for the illumination
// preconditioner and the gradient smoothing. smooth2d(Z, span) convolves Z ('same' size, zero
// outside) with a normalised 2-D Gaussian of standard deviation `span` sampled at the points
// -2 span, -2 span + 2, ..., 2 span of both axes, and divides by the same convolution of a
// plane of ones. The Gaussian is the outer product of its 1-D sampling, so the convolution is
// applied as two 1-D passes (rows, then columns) with weights w_k = f_k / sum(f),
// f_k = exp(-(x_k / span)^2 / 2), and the normaliser is the product of the 1-D weight sums
// over the taps that fall inside the plane. Everything is FP64, as the reference's numpy.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"

namespace adfwi {
namespace gp {

constexpr int kThreads = 256;

// w[k] = f_k / sum(f) for k = 0 .. 2 span (one block; fixed-order sum).
__global__ void __launch_bounds__(kThreads) gauss_weights(int span, double* __restrict__ w) {
  __shared__ double part[kThreads];
  const int n = 2 * span + 1;
  double acc = 0.0;
  for (int k = threadIdx.x; k < n; k += kThreads) {
    const double x = (-2.0 * span + 2.0 * k) / span;
    const double f = exp(-0.5 * x * x);
    w[k] = f;
    acc += f;
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) part[threadIdx.x] += part[threadIdx.x + s];
    __syncthreads();
  }
  const double total = part[0];
  for (int k = threadIdx.x; k < n; k += kThreads) w[k] = w[k] / total;
}

// Row pass: t(i, j) = sum_b w[span + b] z(i, j + b), zero outside the plane.
__global__ void __launch_bounds__(kThreads) pass_rows(int nz, int nx, int span, const double* __restrict__ w,
                                                      const double* __restrict__ z, double* __restrict__ t) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= nx) return;
  const double* row = z + (int64_t)i * nx;
  const int b0 = max(-span, -j), b1 = min(span, nx - 1 - j);
  double acc = 0.0;
  for (int b = b0; b <= b1; ++b) acc += __ldg(w + span + b) * row[j + b];
  t[(int64_t)i * nx + j] = acc;
}

// Column pass and normalisation: out(i, j) = sum_a w[span + a] t(i + a, j) / (wz(i) wx(j)).
__global__ void __launch_bounds__(kThreads) pass_cols(int nz, int nx, int span, const double* __restrict__ w,
                                                      const double* __restrict__ t, double* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (j >= nx) return;
  const int a0 = max(-span, -i), a1 = min(span, nz - 1 - i);
  const int b0 = max(-span, -j), b1 = min(span, nx - 1 - j);
  double acc = 0.0, wz = 0.0, wx = 0.0;
  for (int a = a0; a <= a1; ++a) {
    const double wa = __ldg(w + span + a);
    acc += wa * t[(int64_t)(i + a) * nx + j];
    wz += wa;
  }
  for (int b = b0; b <= b1; ++b) wx += __ldg(w + span + b);
  out[(int64_t)i * nx + j] = acc / (wz * wx);
}

int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

}  // namespace gp
}  // namespace adfwi

using namespace adfwi;

extern "C" {

int adfwi_smooth2d_workspace_bytes(int32_t nz, int32_t nx, int32_t span, int64_t* bytes) {
  ADFWI_CHECK_ARG(bytes != nullptr, "null output pointer");
  ADFWI_CHECK_ARG(nz > 0 && nx > 0 && span > 0, "nz, nx and span must be positive");
  *bytes = gp::align256((int64_t)nz * nx * 8) + gp::align256((int64_t)(2 * span + 1) * 8);
  return kOk;
}

int adfwi_smooth2d(int32_t nz, int32_t nx, int32_t span, const double* in, double* out, void* workspace,
                   int64_t workspace_bytes, void* stream) {
  ADFWI_CHECK_ARG(nz > 0 && nx > 0 && span > 0, "nz, nx and span must be positive");
  ADFWI_CHECK_ARG(in && out && workspace, "null array");
  int64_t need = 0;
  adfwi_smooth2d_workspace_bytes(nz, nx, span, &need);
  if (workspace_bytes < need) {
    set_error("smooth2d workspace too small: %lld bytes given, %lld needed", (long long)workspace_bytes,
              (long long)need);
    return kWorkspaceTooSmall;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* t = static_cast<double*>(workspace);
  double* w = reinterpret_cast<double*>(static_cast<unsigned char*>(workspace) + gp::align256((int64_t)nz * nx * 8));
  const dim3 grid((unsigned)((nx + gp::kThreads - 1) / gp::kThreads), (unsigned)nz);
  ADFWI_LAUNCH(kAux, st, (gp::gauss_weights<<<1, gp::kThreads, 0, st>>>(span, w)));
  ADFWI_LAUNCH(kAux, st, (gp::pass_rows<<<grid, gp::kThreads, 0, st>>>(nz, nx, span, w, in, t)));
  ADFWI_LAUNCH(kAux, st, (gp::pass_cols<<<grid, gp::kThreads, 0, st>>>(nz, nx, span, w, t, out)));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // extern "C"
