// Normalised L2 trace misfit: per-trace statistics, factors and the adjoint source sample,
// shared by the stand-alone misfit (misfit.cu) and by the acoustic adjoint step, which forms the
// pressure records' adjoint source from the records and the observed data as it injects it
// (acoustic.cu), so both produce the same bits.
//
// Reference (paths inside liufeng2317/ADFWI):
//   ADFWI/fwi/misfit/L2.py:26-29        L = sum_{s,r} sqrt(sum_t (obs - syn)^2 dt)
//   ADFWI/fwi/acoustic_fwi.py:149-150   both traces divided by their max |value| first
//
// Records are (ns, nt, nr) row-major. A block takes 32 adjacent receivers of one shot and
// kPhases time phases: thread (x, y) walks samples t = y, y + kPhases, ... of receiver x (a warp
// reads one 128-byte row per sample, the block kPhases consecutive rows), and the phases'
// partial results are combined in phase order, so every pass is bandwidth-bound and
// deterministic.
//   peaks:   per trace max |syn| (its first arg-max and sign) and max |obs| (exact: the phase
//            combination keeps the first arg-max); per shot the peak of both gathers (atomicMax
//            on the bit patterns of non-negative floats: exact and order-independent);
//   factors: silent traces (peak <= silent_rel x the gather's peak; the reference uses
//            silent_rel = 0) are zero; S2 = sum_t rsd^2, S3 = sum_t rsd * syn with
//            rsd = obs/m_obs - syn/m_syn in the data type (as the reference rounds it) and the
//            sums in FP64 (per phase in time order, then over the phases in order);
//            n = sqrt(S2 dt); the adjoint source is
//            dL/dsyn_t = -rsd_t dt / (n m_syn), plus the max's share dt S3 / (n m_syn^2) sign at
//            the arg-max sample, with the two per-trace factors rounded to the data type and the
//            sample formed in it (the acoustic adjoint step can form these samples at its
//            receivers, where FP64 arithmetic would stall the steps).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace adfwi {
namespace l2 {

constexpr int kLanes = 32;                  // receivers of a block
constexpr int kPhases = 16;                 // time phases of a block
constexpr int kThreads = kLanes * kPhases;  // 512
inline dim3 grid(int ns, int nr) { return dim3((unsigned)((nr + kLanes - 1) / kLanes), (unsigned)ns); }
inline dim3 block() { return dim3(kLanes, kPhases); }

template <typename T>
struct TraceStats {
  T m_syn;  // max |syn|
  int arg;  // first sample where |syn| = m_syn
  int neg;  // syn[arg] < 0
  T m_obs;  // max |obs|
};

// What the adjoint source of one trace needs besides its samples (16-byte aligned: a reader
// fetches it with vector loads).
template <typename T>
struct alignas(16) TraceFactors {
  T scale;  // -dt / (n m_syn), 0 for a trace without gradient
  T corr;   // the max's share at the arg-max sample
  T m_syn, m_obs;
  int arg;
  int flags;  // bit 0: gradient, bit 1: observed trace live
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
  __shared__ TraceStats<T> part[kPhases][kLanes];
  const int x = threadIdx.x, y = threadIdx.y;
  const int r = blockIdx.x * kLanes + x, s = blockIdx.y;
  T ms = T(0), mo = T(0);
  int arg = 0, neg = 0;
  if (r < nr) {
    const T* ps = syn + (int64_t)s * nt * nr + r;
    const T* po = obs + (int64_t)s * nt * nr + r;
#pragma unroll 4
    for (int t = y; t < nt; t += kPhases) {
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
  }
  part[y][x] = TraceStats<T>{ms, arg, neg, mo};
  __syncthreads();
  if (y != 0 || r >= nr) return;
  // the first arg-max over all samples: the largest phase maximum, the earliest among equals
  // (a trace without a positive sample keeps arg 0, as a scan in time order does)
  TraceStats<T> q = part[0][x];
  for (int p = 1; p < kPhases; ++p) {
    const TraceStats<T> c = part[p][x];
    if (c.m_syn > q.m_syn || (c.m_syn == q.m_syn && c.m_syn > T(0) && c.arg < q.arg)) {
      q.m_syn = c.m_syn;
      q.arg = c.arg;
      q.neg = c.neg;
    }
    q.m_obs = c.m_obs > q.m_obs ? c.m_obs : q.m_obs;
  }
  st[(int64_t)s * nr + r] = q;
  atomic_max_nonneg(gsyn + s, q.m_syn);
  atomic_max_nonneg(gobs + s, q.m_obs);
}

// The normalised observed sample (obs as given when normalise_obs is 0).
template <typename T>
__device__ __forceinline__ T obs_n(const TraceFactors<T>& f, T o, int normalise_obs) {
  return !normalise_obs ? o : ((f.flags & 2) ? o / f.m_obs : T(0));
}

// Factors of trace (s, r) known before its sums: maxima, arg-max, which traces are live.
template <typename T>
__device__ __forceinline__ TraceFactors<T> trace_head(const TraceStats<T>& q, double gsyn_peak, double gobs_peak,
                                                      double silent_rel, int normalise_obs, bool* live) {
  TraceFactors<T> f;
  *live = q.m_syn > T(0) && (double)q.m_syn > silent_rel * gsyn_peak;
  const bool olive = !normalise_obs || (q.m_obs > T(0) && (double)q.m_obs > silent_rel * gobs_peak);
  f.m_syn = q.m_syn;
  f.m_obs = q.m_obs;
  f.arg = q.arg;
  f.flags = olive ? 2 : 0;
  f.scale = T(0);
  f.corr = T(0);
  return f;
}

// One sample's terms of S2 and S3.
template <typename T>
__device__ __forceinline__ void trace_sums(const TraceFactors<T>& f, bool live, T v, T o, int normalise_obs,
                                           double& s2, double& s3) {
  const T on = obs_n(f, o, normalise_obs);
  const T sn = live ? v / f.m_syn : T(0);
  const double d = (double)(on - sn);
  s2 += d * d;
  s3 += d * (double)v;
}

// The factors from the sums, and the trace's norm n (its share of the loss).
template <typename T>
__device__ __forceinline__ void trace_finish(TraceFactors<T>& f, bool live, int neg, double s2, double s3, double dt,
                                             double* n_out) {
  const double n = sqrt(s2 * dt);
  *n_out = n;
  const bool grad = live && n > 0.0;
  f.scale = (T)(grad ? -dt / (n * (double)f.m_syn) : 0.0);
  f.corr = (T)(grad ? dt * s3 / (n * (double)f.m_syn * (double)f.m_syn) * (neg ? -1.0 : 1.0) : 0.0);
  if (grad) f.flags |= 1;
}

// Adjoint source dL/dsyn at sample t of a trace with factors f, times gmul (the gradient of the
// caller's objective with respect to the loss; exactly the unscaled value when gmul is 1).
template <typename T>
__device__ __forceinline__ T source(const TraceFactors<T>& f, T v, T o, int t, int normalise_obs, T gmul = T(1)) {
  if (!(f.flags & 1)) return T(0);
  const T sn = v / f.m_syn;
  T g = (obs_n(f, o, normalise_obs) - sn) * f.scale;
  if (t == f.arg) g += f.corr;
  if (gmul != T(1)) g *= gmul;
  return g;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) factors(int ns, int nt, int nr, double dt, double silent_rel,
                                                    int normalise_obs, const T* __restrict__ syn,
                                                    const T* __restrict__ obs, const TraceStats<T>* __restrict__ st,
                                                    const PeakWord<T>* __restrict__ gsyn,
                                                    const PeakWord<T>* __restrict__ gobs,
                                                    TraceFactors<T>* __restrict__ fac, double* __restrict__ norms) {
  __shared__ double p2[kPhases][kLanes], p3[kPhases][kLanes];
  const int x = threadIdx.x, y = threadIdx.y;
  const int r = blockIdx.x * kLanes + x, s = blockIdx.y;
  const int64_t tr = (int64_t)s * nr + r;
  double s2 = 0.0, s3 = 0.0;
  TraceFactors<T> f;
  bool live = false;
  if (r < nr) {
    f = trace_head(st[tr], (double)peak_value(gsyn + s), (double)peak_value(gobs + s), silent_rel, normalise_obs,
                   &live);
    const T* ps = syn + (int64_t)s * nt * nr + r;
    const T* po = obs + (int64_t)s * nt * nr + r;
#pragma unroll 4
    for (int t = y; t < nt; t += kPhases) trace_sums(f, live, ps[(int64_t)t * nr], po[(int64_t)t * nr], normalise_obs, s2, s3);
  }
  p2[y][x] = s2;
  p3[y][x] = s3;
  __syncthreads();
  if (y != 0 || r >= nr) return;
  double a2 = 0.0, a3 = 0.0;
  for (int p = 0; p < kPhases; ++p) {
    a2 += p2[p][x];
    a3 += p3[p][x];
  }
  double n;
  trace_finish(f, live, st[tr].neg, a2, a3, dt, &n);
  fac[tr] = f;
  norms[tr] = n;
}

// The adjoint source of every sample, times *gmul when gmul is given.
template <typename T>
__global__ void __launch_bounds__(kThreads) sources(int ns, int nt, int nr, int normalise_obs,
                                                    const T* __restrict__ syn, const T* __restrict__ obs,
                                                    const TraceFactors<T>* __restrict__ fac,
                                                    const double* __restrict__ gmul, T* __restrict__ adj) {
  const int x = threadIdx.x, y = threadIdx.y;
  const int r = blockIdx.x * kLanes + x, s = blockIdx.y;
  if (r >= nr) return;
  const TraceFactors<T> f = fac[(int64_t)s * nr + r];
  const T gm = gmul != nullptr ? (T)*gmul : T(1);
  const int64_t base = (int64_t)s * nt * nr + r;
#pragma unroll 4
  for (int t = y; t < nt; t += kPhases) {
    const int64_t o = base + (int64_t)t * nr;
    adj[o] = source(f, syn[o], obs[o], t, normalise_obs, gm);
  }
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
