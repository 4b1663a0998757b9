// Boundary-saving reconstruction of the acoustic forward states for the gradient (no snapshots,
// no recomputation): the forward keeps, after every step, p, u and w of the "frame" -- every
// cell whose update cannot be undone (the absorbing frame, where the damping is not zero, the
// free-surface rows and the rows / columns outside an update region) -- and the reverse pass
// rebuilds the interior one step back from the state after the step:
//   u = u' + alpha2 Dx p',  w = w' + alpha2 Dz p'     (p' = p after the step),
//   p = (p' - dt wav) + alpha1 div(u, w),
// the forward update (acoustic_kernels.py:113-174, with the damping factors exactly 1 in the
// interior) solved for the state before the step, then restores the frame from what the
// forward kept. The reconstruction is exact in exact arithmetic; in floating point each step
// adds a rounding of the inverted update.
//
// Reference: ADFWI/propagator/acoustic_kernels_bs.py:40-54 (save_boundaries / restore_boundaries)
// and 202-313 (the checkpointed time step that uses them), an unfinished prototype whose reverse
// pass re-applies the forward update instead of inverting it. Here the frame is the whole
// absorbing frame (not a strip of stencil width), so the PML cells' states, which the
// gradient of the padded coefficients needs, are the forward's own.
//
// Saved slot layout: [field p, u, w][shot][frame cell], frame cells listed by plane offset. The
// reverse kernels run over 32 x 8 cell tiles of one shot (grid x: columns, y: rows, z: shots);
// the interior is the box [ilo, ihi] x [jlo, jhi], and only frame cells read their index.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace adfwi {
namespace ac {

struct BsBox {
  int ilo, ihi, jlo, jhi;
  __device__ __forceinline__ bool interior(int i, int j) const { return i >= ilo && i <= ihi && j >= jlo && j <= jhi; }
};

template <typename T>
__global__ void bs_save(Layout L, int ns, int nframe, const int* __restrict__ frame_off, const T* __restrict__ st,
                        T* __restrict__ slot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, s = blockIdx.y;
  if (k >= nframe) return;
  const int64_t PL = L.plane, NSP = (int64_t)ns * PL;
  const int64_t o = (int64_t)s * PL + frame_off[k];
#pragma unroll
  for (int f = 0; f < 3; ++f) slot[((int64_t)f * ns + s) * nframe + k] = st[f * NSP + o];
}

// u, w before step it, from p', u', w' after it (u, w in place); frame cells from the slot kept
// after step it-1 (zero before the first step: slot == nullptr).
template <typename T>
__global__ void bs_reverse_uw(Geo<T> g, BsBox box, const int* __restrict__ fidx, const T* __restrict__ cf,
                              const T* __restrict__ pn, T* __restrict__ u, T* __restrict__ w,
                              const T* __restrict__ slot, int nframe) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  const int s = blockIdx.z;
  if (i >= g.L.nzp || j >= g.L.nxp) return;
  const int64_t PL = g.L.plane, P = g.L.pitch;
  const int64_t oc = g.L.off(i, j), o = (int64_t)s * PL + oc;
  if (!box.interior(i, j)) {
    const int k = fidx[(int64_t)i * g.L.nxp + j];
    u[o] = slot ? slot[((int64_t)1 * g.ns + s) * nframe + k] : T(0);
    w[o] = slot ? slot[((int64_t)2 * g.ns + s) * nframe + k] : T(0);
    return;
  }
  const T dpx = radd(rmul(g.c1, rsub(pn[o + 1], pn[o])), rmul(g.c2, rsub(pn[o + 2], pn[o - 1])));
  const T dpz = radd(rmul(g.c1, rsub(pn[o + P], pn[o])), rmul(g.c2, rsub(pn[o + 2 * P], pn[o - P])));
  u[o] = radd(u[o], rmul(cf[kA2U * PL + oc], dpx));
  w[o] = radd(w[o], rmul(cf[kA2W * PL + oc], dpz));
}

// p before step it into pp, and the divergence of (u, w) that step it used into dh (the
// forward's operation order, zero outside the p update region, as the forward keeps it).
template <typename T>
__global__ void bs_reverse_p(Geo<T> g, BsBox box, int it, const int* __restrict__ fidx, const T* __restrict__ cf,
                             const T* __restrict__ pn, const T* __restrict__ u, const T* __restrict__ w,
                             T* __restrict__ pp, T* __restrict__ dh, const T* __restrict__ slot, int nframe,
                             const T* __restrict__ wav) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  const int s = blockIdx.z;
  if (i >= g.L.nzp || j >= g.L.nxp) return;
  const int64_t PL = g.L.plane, P = g.L.pitch;
  const int64_t oc = g.L.off(i, j), o = (int64_t)s * PL + oc;
  T dv = T(0);
  if (in_p(g, i, j)) {
    const T t1 = rsub(radd(rsub(u[o], u[o - 1]), w[o]), w[o - P]);
    const T t2 = rsub(radd(rsub(u[o + 1], u[o - 2]), w[o + P]), w[o - 2 * P]);
    dv = radd(rmul(g.c1, t1), rmul(g.c2, t2));
  }
  dh[o] = dv;
  if (!box.interior(i, j)) {
    const int k = fidx[(int64_t)i * g.L.nxp + j];
    pp[o] = slot ? slot[(int64_t)s * nframe + k] : T(0);
    return;
  }
  T x = pn[o];
  if (i == g.src_z[s] && j == g.src_x[s]) x = rsub(x, rmul(g.dt, wav[(int64_t)s * g.nt + it]));
  pp[o] = radd(x, rmul(cf[kA1M * PL + oc], dv));
}

}  // namespace ac
}  // namespace adfwi
