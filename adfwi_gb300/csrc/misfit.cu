// Normalised L2 trace misfit and its adjoint source (sm_103a).
//
// Reference (paths inside liufeng2317/ADFWI):
//   ADFWI/fwi/misfit/L2.py:26-29        L = sum_{s,r} sqrt(sum_t (obs - syn)^2 dt)
//   ADFWI/fwi/acoustic_fwi.py:149-150   both traces divided by their max |value| first
// The reference evaluates it with PyTorch operations (a dozen (ns, nt, nr) round trips, FP32
// sums) and differentiates it with autograd. Here three kernels read the records a few times
// each and write the adjoint source once; every sum over time and over traces is FP64 in a
// fixed order, so the loss and the adjoint source are deterministic.
//
// The per-trace statistics, factors and adjoint-source sample are in l2.cuh (shared with the
// acoustic adjoint step, which forms the pressure records' adjoint source on the fly); here
// three kernels read the records a few times each and write the adjoint source once, and one
// block sums the per-trace norms in a fixed order.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"
#include "l2.cuh"

namespace adfwi {
namespace mf {

using namespace l2;

template <typename T>
__global__ void __launch_bounds__(kThreads) adjoint(int ns, int nt, int nr, double dt, double silent_rel,
                                                    int normalise_obs, const T* __restrict__ syn,
                                                    const T* __restrict__ obs, const TraceStats<T>* __restrict__ st,
                                                    const PeakWord<T>* __restrict__ gsyn,
                                                    const PeakWord<T>* __restrict__ gobs, T* __restrict__ adj,
                                                    double* __restrict__ norms) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
  if (r >= nr) return;
  const int64_t tr = (int64_t)s * nr + r;
  const T* ps = syn + (int64_t)s * nt * nr + r;
  const T* po = obs + (int64_t)s * nt * nr + r;
  double n;
  const TraceFactors<T> f = trace_factors(st[tr], (double)peak_value(gsyn + s), (double)peak_value(gobs + s), ps, po,
                                          nt, nr, dt, silent_rel, normalise_obs, &n);
  norms[tr] = n;
  T* pa = adj + (int64_t)s * nt * nr + r;
  for (int t = 0; t < nt; ++t) pa[(int64_t)t * nr] = source(f, ps[(int64_t)t * nr], po[(int64_t)t * nr], t, normalise_obs);
}

int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

struct MCarve {
  int64_t stats, gsyn, gobs, norms, total;
};

MCarve mcarve(int dtype, int64_t ns, int64_t nr) {
  MCarve c;
  const int64_t es = dtype == ADFWI_F64 ? (int64_t)sizeof(TraceStats<double>) : (int64_t)sizeof(TraceStats<float>);
  const int64_t pw = dtype == ADFWI_F64 ? 8 : 4;
  int64_t o = 0;
  c.stats = o;
  o += align256(ns * nr * es);
  c.gsyn = o;
  o += align256(ns * pw);
  c.gobs = o;
  o += align256(ns * pw);
  c.norms = o;
  o += align256(ns * nr * 8);
  c.total = o;
  return c;
}

template <typename T>
int run(int32_t ns, int32_t nt, int32_t nr, double dt, double silent_rel, int32_t flags, const void* syn,
        const void* obs, void* adj, double* loss, unsigned char* ws, cudaStream_t st) {
  const MCarve c = mcarve(sizeof(T) == 8 ? ADFWI_F64 : ADFWI_F32, ns, nr);
  auto* stats = reinterpret_cast<TraceStats<T>*>(ws + c.stats);
  auto* gsyn = reinterpret_cast<PeakWord<T>*>(ws + c.gsyn);
  auto* gobs = reinterpret_cast<PeakWord<T>*>(ws + c.gobs);
  auto* norms = reinterpret_cast<double*>(ws + c.norms);
  ADFWI_CUDA_TRY(cudaMemsetAsync(ws + c.gsyn, 0, c.norms - c.gsyn, st));  // peaks start at +0
  const dim3 grid((unsigned)((nr + kThreads - 1) / kThreads), (unsigned)ns);
  ADFWI_LAUNCH(kAux, st, (peaks<T><<<grid, kThreads, 0, st>>>(ns, nt, nr, static_cast<const T*>(syn),
                                                                static_cast<const T*>(obs), stats, gsyn, gobs)));
  ADFWI_LAUNCH(kAux, st, (adjoint<T><<<grid, kThreads, 0, st>>>(ns, nt, nr, dt, silent_rel, flags & 1,
                                                                  static_cast<const T*>(syn),
                                                                  static_cast<const T*>(obs), stats, gsyn, gobs,
                                                                  static_cast<T*>(adj), norms)));
  ADFWI_LAUNCH(kAux, st, (sum_norms<<<1, kThreads, 0, st>>>((int64_t)ns * nr, norms, loss)));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mf
}  // namespace adfwi

using namespace adfwi;

extern "C" {

int adfwi_l2_misfit_workspace_bytes(int32_t dtype, int32_t ns, int32_t nr, int64_t* bytes) {
  ADFWI_CHECK_ARG(bytes != nullptr, "null output pointer");
  ADFWI_CHECK_ARG(dtype == ADFWI_F32 || dtype == ADFWI_F64, "dtype must be ADFWI_F32 or ADFWI_F64");
  ADFWI_CHECK_ARG(ns > 0 && nr > 0, "ns and nr must be positive");
  *bytes = mf::mcarve(dtype, ns, nr).total;
  return kOk;
}

int adfwi_l2_misfit(int32_t dtype, int32_t ns, int32_t nt, int32_t nr, double dt, double silent_rel, int32_t flags,
                    const void* syn, const void* obs, void* adj, double* loss, void* workspace, int64_t ws_bytes,
                    void* stream) {
  ADFWI_CHECK_ARG(dtype == ADFWI_F32 || dtype == ADFWI_F64, "dtype must be ADFWI_F32 or ADFWI_F64");
  ADFWI_CHECK_ARG(ns > 0 && nt > 0 && nr > 0, "ns, nt and nr must be positive");
  ADFWI_CHECK_ARG(syn && obs && adj && loss && workspace, "null array");
  ADFWI_CHECK_ARG(dt > 0.0 && silent_rel >= 0.0, "dt must be positive and silent_rel non-negative");
  const int64_t need = mf::mcarve(dtype, ns, nr).total;
  if (ws_bytes < need) {
    set_error("misfit workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)need);
    return kWorkspaceTooSmall;
  }
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == ADFWI_F64)
    return mf::run<double>(ns, nt, nr, dt, silent_rel, flags, syn, obs, adj, loss, ws, st);
  return mf::run<float>(ns, nt, nr, dt, silent_rel, flags, syn, obs, adj, loss, ws, st);
}

}  // extern "C"
