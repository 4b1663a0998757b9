// Normalised L2 trace misfit and its adjoint source (sm_103a).
//
// Reference (paths inside liufeng2317/ADFWI):
//   ADFWI/fwi/misfit/L2.py:26-29        L = sum_{s,r} sqrt(sum_t (obs - syn)^2 dt)
//   ADFWI/fwi/acoustic_fwi.py:149-150   both traces divided by their max |value| first
// The reference evaluates it with PyTorch operations (a dozen (ns, nt, nr) round trips, FP32
// sums) and differentiates it with autograd. Here three bandwidth-bound passes (l2.cuh: peaks,
// factors, sources) read the records three times and write the adjoint source once, and one
// block sums the per-trace norms; every sum over time and over traces is FP64 in a fixed order,
// so the loss and the adjoint source are deterministic. The kernels are the ones the acoustic
// plan's loss uses, so both give the same bits.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"
#include "l2.cuh"

namespace adfwi {
namespace mf {

using namespace l2;

int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

struct MCarve {
  int64_t stats, gsyn, gobs, norms, fac, total;
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
  c.fac = o;
  o += align256(ns * nr *
                (dtype == ADFWI_F64 ? (int64_t)sizeof(TraceFactors<double>) : (int64_t)sizeof(TraceFactors<float>)));
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
  auto* fac = reinterpret_cast<TraceFactors<T>*>(ws + c.fac);
  ADFWI_CUDA_TRY(cudaMemsetAsync(ws + c.gsyn, 0, c.norms - c.gsyn, st));  // peaks start at +0
  const T* sy = static_cast<const T*>(syn);
  const T* ob = static_cast<const T*>(obs);
  const int nob = flags & 1;
  ADFWI_LAUNCH(kAux, st, (peaks<T><<<grid(ns, nr), block(), 0, st>>>(ns, nt, nr, sy, ob, stats, gsyn, gobs)));
  ADFWI_LAUNCH(kAux, st, (factors<T><<<grid(ns, nr), block(), 0, st>>>(ns, nt, nr, dt, silent_rel, nob, sy, ob, stats,
                                                                         gsyn, gobs, fac, norms)));
  ADFWI_LAUNCH(kAux, st, (sources<T><<<grid(ns, nr), block(), 0, st>>>(ns, nt, nr, nob, sy, ob, fac, nullptr,
                                                                         static_cast<T*>(adj))));
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
