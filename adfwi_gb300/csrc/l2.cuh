// Normalised L2 trace misfit: per-trace statistics, factors and the adjoint source sample,
// shared by the stand-alone misfit (misfit.cu) and by the acoustic adjoint step, which forms the
// pressure records' adjoint source from the records and the observed data as it injects it
// (acoustic.cu), so both produce the same bits.
//
// Reference (paths inside liufeng2317/ADFWI):
//   ADFWI/fwi/misfit/L2.py:26-29        L = sum_{s,r} sqrt(sum_t (obs - syn)^2 dt)
//   ADFWI/fwi/acoustic_fwi.py:149-150   both traces divided by their max |value| first
//
// Records are (ns, nt, nr) row-major; one thread owns one trace (s, r) and walks its samples
// with stride nr (a warp reads 32 consecutive receivers per sample).
//   peaks:   per trace max |syn| (its first arg-max and sign) and max |obs|; per shot the peak
//            of both gathers (atomicMax on the bit patterns of non-negative floats: exact and
//            order-independent);
//   factors: silent traces (peak <= silent_rel x the gather's peak; the reference uses
//            silent_rel = 0) are zero; S2 = sum_t rsd^2, S3 = sum_t rsd * syn with
//            rsd = obs/m_obs - syn/m_syn in the data type (as the reference rounds it) and the
//            sums in FP64; n = sqrt(S2 dt); the adjoint source is
//            dL/dsyn_t = -rsd_t dt / (n m_syn), plus the max's share dt S3 / (n m_syn^2) sign at
//            the arg-max sample.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace adfwi {
namespace l2 {

constexpr int kThreads = 256;

template <typename T>
struct TraceStats {
  T m_syn;  // max |syn|
  int arg;  // first sample where |syn| = m_syn
  int neg;  // syn[arg] < 0
  T m_obs;  // max |obs|
};

// What the adjoint source of one trace needs besides its samples.
template <typename T>
struct TraceFactors {
  double scale;  // -dt / (n m_syn), 0 for a trace without gradient
  double corr;   // the max's share at the arg-max sample
  T m_syn, m_obs;
  int arg;
  int flags;     // bit 0: gradient, bit 1: observed trace live
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

// The normalised observed sample (obs as given when normalise_obs is 0).
template <typename T>
__device__ __forceinline__ T obs_n(const TraceFactors<T>& f, T o, int normalise_obs) {
  return !normalise_obs ? o : ((f.flags & 2) ? o / f.m_obs : T(0));
}

// Factors of trace (s, r) and its norm n (its share of the loss).
template <typename T>
__device__ __forceinline__ TraceFactors<T> trace_factors(const TraceStats<T>& q, double gsyn_peak, double gobs_peak,
                                                         const T* ps, const T* po, int nt, int nr, double dt,
                                                         double silent_rel, int normalise_obs, double* n_out) {
  TraceFactors<T> f;
  const bool live = q.m_syn > T(0) && (double)q.m_syn > silent_rel * gsyn_peak;
  const bool olive = !normalise_obs || (q.m_obs > T(0) && (double)q.m_obs > silent_rel * gobs_peak);
  f.m_syn = q.m_syn;
  f.m_obs = q.m_obs;
  f.arg = q.arg;
  f.flags = olive ? 2 : 0;
  double s2 = 0.0, s3 = 0.0;
  for (int t = 0; t < nt; ++t) {
    const T v = ps[(int64_t)t * nr];
    const T on = obs_n(f, po[(int64_t)t * nr], normalise_obs);
    const T sn = live ? v / q.m_syn : T(0);
    const double d = (double)(on - sn);
    s2 += d * d;
    s3 += d * (double)v;
  }
  const double n = sqrt(s2 * dt);
  *n_out = n;
  const bool grad = live && n > 0.0;
  f.scale = grad ? -dt / (n * (double)q.m_syn) : 0.0;
  f.corr = grad ? dt * s3 / (n * (double)q.m_syn * (double)q.m_syn) * (q.neg ? -1.0 : 1.0) : 0.0;
  if (grad) f.flags |= 1;
  return f;
}

// Adjoint source dL/dsyn at sample t of a trace with factors f, times gmul (the gradient of the
// caller's objective with respect to the loss; exactly the unscaled value when gmul is 1).
template <typename T>
__device__ __forceinline__ T source(const TraceFactors<T>& f, T v, T o, int t, int normalise_obs, double gmul = 1.0) {
  if (!(f.flags & 1)) return T(0);
  const T sn = v / f.m_syn;
  double g = (double)(obs_n(f, o, normalise_obs) - sn) * f.scale;
  if (t == f.arg) g += f.corr;
  if (gmul != 1.0) g *= gmul;
  return (T)g;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) factors(int ns, int nt, int nr, double dt, double silent_rel,
                                                    int normalise_obs, const T* __restrict__ syn,
                                                    const T* __restrict__ obs, const TraceStats<T>* __restrict__ st,
                                                    const PeakWord<T>* __restrict__ gsyn,
                                                    const PeakWord<T>* __restrict__ gobs,
                                                    TraceFactors<T>* __restrict__ fac, double* __restrict__ norms) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
  if (r >= nr) return;
  const int64_t tr = (int64_t)s * nr + r;
  double n;
  fac[tr] = trace_factors(st[tr], (double)peak_value(gsyn + s), (double)peak_value(gobs + s),
                          syn + (int64_t)s * nt * nr + r, obs + (int64_t)s * nt * nr + r, nt, nr, dt, silent_rel,
                          normalise_obs, &n);
  norms[tr] = n;
}

// loss = sum of the n norms in a fixed order (one block).
static __global__ void __launch_bounds__(kThreads) sum_norms(int64_t n, const double* __restrict__ norms,
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

}  // namespace l2
}  // namespace adfwi
