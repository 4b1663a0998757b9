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
// Records are (ns, nt, nr) row-major: one thread owns one trace (s, r) and walks its nt
// samples with stride nr, so a warp reads 32 consecutive receivers per sample (coalesced).
//
//   peaks:    per trace max |syn| (its first arg-max and sign) and max |obs|; per shot the
//             peak of both gathers (atomicMax on the bit patterns of non-negative floats:
//             exact and order-independent);
//   adjoint:  per trace, silent traces (peak <= silent_rel x the gather's peak; the reference
//             uses silent_rel = 0) are zero; S2 = sum_t rsd^2, S3 = sum_t rsd * syn with
//             rsd = obs/m_obs - syn/m_syn in the data type (as the reference rounds it) and the
//             sums in FP64; n = sqrt(S2 dt); dL/dsyn_t = -rsd_t dt / (n m_syn), plus the max's
//             share dt S3 / (n m_syn^2) sign at the arg-max sample; n goes to a per-trace array;
//   loss:     one block sums the per-trace norms in a fixed order.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"

namespace adfwi {
namespace mf {

constexpr int kThreads = 256;

template <typename T>
struct TraceStats {
  T m_syn;     // max |syn|
  int arg;     // first sample where |syn| = m_syn
  int neg;     // syn[arg] < 0
  T m_obs;     // max |obs|
};

__device__ __forceinline__ void atomic_max_nonneg(unsigned* addr, float v) { atomicMax(addr, __float_as_uint(v)); }
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ float peak_value(const unsigned* p) { return __uint_as_float(*p); }
__device__ __forceinline__ double peak_value(const unsigned long long* p) { return __longlong_as_double((long long)*p); }

template <typename T>
using PeakWord = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned>::type;

template <typename T>
__global__ void __launch_bounds__(kThreads) peaks(int ns, int nt, int nr, const T* __restrict__ syn,
                                                  const T* __restrict__ obs, TraceStats<T>* __restrict__ st,
                                                  PeakWord<T>* __restrict__ gsyn, PeakWord<T>* __restrict__ gobs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
  if (r >= nr) return;
  const T* ps = syn + (int64_t)s * nt * nr + r;
  const T* po = obs + (int64_t)s * nt * nr + r;
  T ms = T(0), mo = T(0);
  int arg = 0, neg = 0;
  for (int t = 0; t < nt; ++t) {
    const T v = ps[(int64_t)t * nr];
    const T a = v < T(0) ? -v : v;
    if (a > ms) {
      ms = a;
      arg = t;
      neg = v < T(0);
    }
    const T o = po[(int64_t)t * nr];
    const T ao = o < T(0) ? -o : o;
    mo = ao > mo ? ao : mo;
  }
  st[(int64_t)s * nr + r] = TraceStats<T>{ms, arg, neg, mo};
  atomic_max_nonneg(gsyn + s, ms);
  atomic_max_nonneg(gobs + s, mo);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) adjoint(int ns, int nt, int nr, double dt, double silent_rel,
                                                    int normalise_obs, const T* __restrict__ syn,
                                                    const T* __restrict__ obs, const TraceStats<T>* __restrict__ st,
                                                    const PeakWord<T>* __restrict__ gsyn,
                                                    const PeakWord<T>* __restrict__ gobs, T* __restrict__ adj,
                                                    double* __restrict__ norms) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
  if (r >= nr) return;
  const TraceStats<T> q = st[(int64_t)s * nr + r];
  const bool live = q.m_syn > T(0) && (double)q.m_syn > silent_rel * (double)peak_value(gsyn + s);
  const bool olive = !normalise_obs || (q.m_obs > T(0) && (double)q.m_obs > silent_rel * (double)peak_value(gobs + s));
  const T* ps = syn + (int64_t)s * nt * nr + r;
  const T* po = obs + (int64_t)s * nt * nr + r;
  T* pa = adj + (int64_t)s * nt * nr + r;
  double s2 = 0.0, s3 = 0.0;
  for (int t = 0; t < nt; ++t) {
    const T v = ps[(int64_t)t * nr];
    const T o = po[(int64_t)t * nr];
    const T on = !normalise_obs ? o : (olive ? o / q.m_obs : T(0));
    const T sn = live ? v / q.m_syn : T(0);
    const double d = (double)(on - sn);
    s2 += d * d;
    s3 += d * (double)v;
  }
  const double n = sqrt(s2 * dt);
  norms[(int64_t)s * nr + r] = n;
  const bool grad = live && n > 0.0;
  const double scale = grad ? -dt / (n * (double)q.m_syn) : 0.0;
  const double corr = grad ? dt * s3 / (n * (double)q.m_syn * (double)q.m_syn) * (q.neg ? -1.0 : 1.0) : 0.0;
  for (int t = 0; t < nt; ++t) {
    double g = 0.0;
    if (grad) {
      const T v = ps[(int64_t)t * nr];
      const T o = po[(int64_t)t * nr];
      const T on = !normalise_obs ? o : (olive ? o / q.m_obs : T(0));
      const T sn = v / q.m_syn;
      g = (double)(on - sn) * scale;
      if (t == q.arg) g += corr;
    }
    pa[(int64_t)t * nr] = (T)g;
  }
}

__global__ void __launch_bounds__(kThreads) sum_norms(int64_t n, const double* __restrict__ norms,
                                                      double* __restrict__ loss) {
  __shared__ double part[kThreads];
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += kThreads) acc += norms[e];
  part[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = part[0];
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
