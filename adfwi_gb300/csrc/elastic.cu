// 2-D velocity-stress elastic propagator (vx, vz, txx, tzz, txz), 4th / 6th order staggered
// grid, split-field PML or multiplicative absorbing layer, free surface, moment-tensor
// sources, 5-component receivers; exact discrete adjoint for the coefficient gradients;
// checkpoint / recompute driver and the C ABI.
//
// Reference algorithm (paths inside liufeng2317/ADFWI):
//   ADFWI/propagator/elastic_kernels.py:20-108    DiffCoef and the half-cell operators Dxfm/Dxbm/Dzfm/Dzbm
//   ADFWI/propagator/elastic_kernels.py:339-418   PML step (split stresses, source -MT/2 on both parts,
//                                                 totals, free-surface rows h-3..h-1, split velocities,
//                                                 totals, free-surface velocity rows, receivers, energy)
//   ADFWI/propagator/elastic_kernels.py:709-774   absorbing-layer step (unsplit, -MT/3 source, v *= damp)
//   ADFWI/propagator/elastic_kernels.py:917-1037  padding, index shifts, chunked loop, record dict
//
// One time step is a short sequence of launches, each a pointwise or gather stencil over
// (cell, shot): the split fields are updated in place (every update reads only its own
// cell of the field it writes), totals and free-surface rows are rebuilt from the split
// fields. Gradient kernels handle one cell for every shot in a loop, so the coefficient
// gradients are summed over shots in a fixed order (deterministic, no atomics). The
// forward arithmetic uses explicitly rounded operations in the reference's order.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"
#include "frames.cuh"
#include "snapshot.cuh"

namespace adfwi {
namespace el {

__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// Field indices inside the state blocks (each field = ns consecutive planes).
enum { TXX_X = 0, TXX_Z, TZZ_X, TZZ_Z, TXZ_X, TXZ_Z };  // split stresses (PML)
enum { VX_X = 0, VX_Z, VZ_X, VZ_Z };                    // split velocities (PML)
enum { TXX = 0, TZZ, TXZ };                             // stress totals / ABL stresses
enum { VX = 0, VZ };                                    // velocity totals / ABL velocities
enum { C11 = 0, C13, C15, C33, C35, C55, BX, BZ, BCX, BCZ, DAMP = 8 };  // coefficient planes

template <typename T>
struct Geo {
  Layout L;
  int ns, nt, nr;
  int fsurf, h;                // free surface; h = NN + 1
  int ilo, ihi, jlo, jhi;      // update region I = [NN, nzp-NN-1] x [NN, nxp-NN-1]
  int top, nabc, nz, nx;       // energy window
  T dt, dx, dz, dt_dx, dt_dz, hdt;
  T f0, f1, f2;                // staggered coefficients
  const int* src_z;
  const int* src_x;
  const T* src_m;              // ns x 3 source weights (xx, zz, xz) already scaled for the mode
  const int* rcv_z;
  const int* rcv_x;
  const int* ucell_zx;         // unique receiver cells (i << 16 | j)
  const int* ucell_beg;        // ncells+1 offsets into ucell_rcv
  const int* ucell_rcv;
  int ncells;
};

template <typename T>
__device__ __forceinline__ bool in_I(const Geo<T>& g, int i, int j) {
  return i >= g.ilo && i <= g.ihi && j >= g.jlo && j <= g.jhi;
}

// ---- half-cell differences (elastic_kernels.py:66-108): f_k (a[+1+k] - a[-k]) etc.
template <int NN, typename T>
__device__ __forceinline__ T dxf(const Geo<T>& g, const T* a, int64_t o) {
  T r = rmul(g.f0, rsub(a[o + 1], a[o]));
  r = radd(r, rmul(g.f1, rsub(a[o + 2], a[o - 1])));
  if (NN == 3) r = radd(r, rmul(g.f2, rsub(a[o + 3], a[o - 2])));
  return r;
}
template <int NN, typename T>
__device__ __forceinline__ T dxb(const Geo<T>& g, const T* a, int64_t o) {
  T r = rmul(g.f0, rsub(a[o], a[o - 1]));
  r = radd(r, rmul(g.f1, rsub(a[o + 1], a[o - 2])));
  if (NN == 3) r = radd(r, rmul(g.f2, rsub(a[o + 2], a[o - 3])));
  return r;
}
template <int NN, typename T>
__device__ __forceinline__ T dzf(const Geo<T>& g, const T* a, int64_t o, int64_t P) {
  T r = rmul(g.f0, rsub(a[o + P], a[o]));
  r = radd(r, rmul(g.f1, rsub(a[o + 2 * P], a[o - P])));
  if (NN == 3) r = radd(r, rmul(g.f2, rsub(a[o + 3 * P], a[o - 2 * P])));
  return r;
}
template <int NN, typename T>
__device__ __forceinline__ T dzb(const Geo<T>& g, const T* a, int64_t o, int64_t P) {
  T r = rmul(g.f0, rsub(a[o], a[o - P]));
  r = radd(r, rmul(g.f1, rsub(a[o + P], a[o - 2 * P])));
  if (NN == 3) r = radd(r, rmul(g.f2, rsub(a[o + 2 * P], a[o - 3 * P])));
  return r;
}
// planes in global memory (row pitch of the layout)
template <int NN, typename T>
__device__ __forceinline__ T dzf(const Geo<T>& g, const T* a, int64_t o) {
  return dzf<NN>(g, a, o, (int64_t)g.L.pitch);
}
template <int NN, typename T>
__device__ __forceinline__ T dzb(const Geo<T>& g, const T* a, int64_t o) {
  return dzb<NN>(g, a, o, (int64_t)g.L.pitch);
}

// ---- transposes in gather form: contribution to cell (i, j) of q placed at the cells that
// read (i, j). q(i', j') must be zero outside the update region.
//   Dxf^T q (j) = sum_k f_k (q[j-1-k] - q[j+k]);   Dxb^T q (j) = sum_k f_k (q[j-k] - q[j+1+k])
template <int NN, typename T, typename Q>
__device__ __forceinline__ T dxf_t(const Geo<T>& g, const Q& q, int i, int j) {
  T r = g.f0 * (q(i, j - 1) - q(i, j)) + g.f1 * (q(i, j - 2) - q(i, j + 1));
  if (NN == 3) r += g.f2 * (q(i, j - 3) - q(i, j + 2));
  return r;
}
template <int NN, typename T, typename Q>
__device__ __forceinline__ T dxb_t(const Geo<T>& g, const Q& q, int i, int j) {
  T r = g.f0 * (q(i, j) - q(i, j + 1)) + g.f1 * (q(i, j - 1) - q(i, j + 2));
  if (NN == 3) r += g.f2 * (q(i, j - 2) - q(i, j + 3));
  return r;
}
template <int NN, typename T, typename Q>
__device__ __forceinline__ T dzf_t(const Geo<T>& g, const Q& q, int i, int j) {
  T r = g.f0 * (q(i - 1, j) - q(i, j)) + g.f1 * (q(i - 2, j) - q(i + 1, j));
  if (NN == 3) r += g.f2 * (q(i - 3, j) - q(i + 2, j));
  return r;
}
template <int NN, typename T, typename Q>
__device__ __forceinline__ T dzb_t(const Geo<T>& g, const Q& q, int i, int j) {
  T r = g.f0 * (q(i, j) - q(i + 1, j)) + g.f1 * (q(i - 1, j) - q(i + 2, j));
  if (NN == 3) r += g.f2 * (q(i - 2, j) - q(i + 3, j));
  return r;
}

// The cell of this thread in the per-cell kernels: a block of 256 threads covers a tile of
// 32 x 8 cells (full 128-byte rows of a plane; most rows that the vertical stencils read belong
// to the same block, so they come from L1), tiles row-major over the padded grid.
constexpr int kTileX = 32, kTileZ = 8, kTileThreads = kTileX * kTileZ;
#define EL_TILE_IJ                                                                   \
  const int tiles_x_ = (g.L.nxp + kTileX - 1) / kTileX;                              \
  const int ti_ = (int)blockIdx.x / tiles_x_, tj_ = (int)blockIdx.x - ti_ * tiles_x_; \
  const int i = ti_ * kTileZ + (int)threadIdx.x / kTileX;                            \
  const int j = tj_ * kTileX + (int)threadIdx.x % kTileX;                            \
  if (i >= g.L.nzp || j >= g.L.nxp) return;

#define EL_CELL_SHOT                                                                 \
  EL_TILE_IJ                                                                         \
  const int s = blockIdx.y;                                                          \
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL;                            \
  const int64_t o = (int64_t)s * PL + g.L.off(i, j);                                 \
  (void)NSP;

// Per-cell kernels that take several shots of one cell per thread (blockIdx.y picks a block of
// kCellShots consecutive shots): the cell's coefficients and PML factors are loaded and formed
// once, and the shots' field loads are independent, so more of them are in flight.
#ifndef ADFWI_EL_CELL_SHOTS
#define ADFWI_EL_CELL_SHOTS 2
#endif
constexpr int kCellShots = ADFWI_EL_CELL_SHOTS;
#define EL_CELL_SHOTS                                                                \
  EL_TILE_IJ                                                                         \
  const int s_lo = blockIdx.y * kCellShots;                                          \
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL;                            \
  const int64_t occ = g.L.off(i, j);

// x / d where d is a PML denominator 1 + dt/2 d(x): exactly x wherever d is 1 (outside the
// absorbing frame), so the division runs only inside the frame.
template <typename T>
__device__ __forceinline__ T rdiv_pml(T x, T d) {
  return d == T(1) ? x : rdiv(x, d);
}

#define EL_CELL                                                                      \
  EL_TILE_IJ                                                                         \
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL;                            \
  const int64_t oc = g.L.off(i, j);

// Gradient kernels: blockIdx.y picks a group of `eg` consecutive shots; the group's gradient
// partials (8 planes) start at gpart + blockIdx.y * 8 * PL and are summed over the groups in a
// fixed order at the end of the backward pass (deterministic).
#define EL_SHOT_GROUP                                                                \
  const int s_beg = blockIdx.y * eg, s_end = min(g.ns, s_beg + eg);                  \
  T* gbase = gpart + (int64_t)blockIdx.y * 8 * PL;

// Staging of the shot-group gradient kernels. Per shot, a block copies the 32 x 8 tile of every
// plane it reads into shared memory with 16-byte asynchronous copies, with the halo its
// stencils need (4 columns each side for x differences, 3 rows each side for z differences,
// none for pointwise reads), then evaluates its cells there: each staged element is fetched
// once per block instead of once per reading thread.
constexpr int kSW = kTileX + 8;     // staged row: columns j0-4 .. j0+kTileX+3
constexpr int kSZ = kTileZ + 6;     // staged rows: i0-3 .. i0+kTileZ+2
constexpr int kSPlane = kSW * kSZ;  // elements of one staged plane
constexpr int kSC = 3 * kSW + 4;    // staged index of the tile's cell (i0, j0)

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Queue the copies of rows i0-zh .. i0+kTileZ+zh-1 and columns j0-xh .. j0+kTileX+xh-1 (xh 0 or
// 4, zh 0 or 3) of `plane` into the staged plane `dst`. Every copy starts on a 16-byte boundary
// (j0 is a multiple of 32, rows are 128-byte multiples, the ghost frame is 4 columns wide), and
// every row and column read lies in the plane's allocation: the layout keeps 4 ghost rows and
// columns before the grid and a 16-row / 64-column margin after it.
template <typename T>
__device__ __forceinline__ void stage(T* dst, const T* plane, const Layout& L, int i0, int j0, int zh, int xh) {
  constexpr int E = 16 / (int)sizeof(T);
  const int cols = (kTileX + 2 * xh) / E, rows = kTileZ + 2 * zh;
  for (int t = threadIdx.x; t < rows * cols; t += kTileThreads) {
    const int r = t / cols, c = t - r * cols;
    cp_async16(dst + (r - zh + 3) * kSW + (c * E - xh + 4), plane + L.off(i0 - zh + r, j0 - xh + c * E));
  }
}

// A staged plane read at grid cells (ii, jj) of the block's tile.
template <typename T>
struct StagedQ {
  const T* s;
  int i0, j0;
  __device__ __forceinline__ T operator()(int ii, int jj) const { return s[(ii - i0 + 3) * kSW + (jj - j0 + 4)]; }
};

// Compact staged planes: an x plane holds only the tile rows with the x halo (kTileZ x kSW), a z
// plane only the tile columns with the z halo (kSZ x kTileX).
constexpr int kXPlane = kTileZ * kSW, kZPlane = kSZ * kTileX;
template <typename T>
__device__ __forceinline__ void stage_x(T* dst, const T* plane, const Layout& L, int i0, int j0) {
  constexpr int E = 16 / (int)sizeof(T), cols = kSW / E;
  for (int t = threadIdx.x; t < kTileZ * cols; t += kTileThreads) {
    const int r = t / cols, c = t - r * cols;
    cp_async16(dst + r * kSW + c * E, plane + L.off(i0 + r, j0 - 4 + c * E));
  }
}
template <typename T>
__device__ __forceinline__ void stage_z(T* dst, const T* plane, const Layout& L, int i0, int j0) {
  constexpr int E = 16 / (int)sizeof(T), cols = kTileX / E;
  for (int t = threadIdx.x; t < kSZ * cols; t += kTileThreads) {
    const int r = t / cols, c = t - r * cols;
    cp_async16(dst + r * kTileX + c * E, plane + L.off(i0 - 3 + r, j0 + c * E));
  }
}
template <typename T>
struct StagedX {
  const T* s;
  int i0, j0;
  __device__ __forceinline__ T operator()(int ii, int jj) const { return s[(ii - i0) * kSW + (jj - j0 + 4)]; }
};
template <typename T>
struct StagedZ {
  const T* s;
  int i0, j0;
  __device__ __forceinline__ T operator()(int ii, int jj) const { return s[(ii - i0 + 3) * kTileX + (jj - j0)]; }
};

// ======================================================================= forward, PML
// Split-field update of a cell and its totals in one pass (elastic_kernels.py:351-402); the rows
// whose totals read other rows (free surface) are left to the *_fs_rows kernels that follow.
template <typename T>
__device__ __forceinline__ bool stress_fs_row(const Geo<T>& g, int i) {
  return g.fsurf && i >= g.h - 3 && i <= g.h - 1;
}
template <typename T>
__device__ __forceinline__ bool vel_fs_row(const Geo<T>& g, int i, int j) {
  return g.fsurf && j >= g.jlo && j <= g.jhi && (i == g.h - 2 || i == g.h - 3);
}

// Cells that keep split fields: inside the update region, where a PML factor differs from 1,
// and in the rows the free-surface kernels rebuild from split parts (h-3 .. h) plus one. Every
// other cell of the update region advances its totals directly: there the split update is
// x' = x + a, z' = z + b, total = x' + z' (the factors are exactly 1), so the unsplit
// t' = (t + a) + b differs only by one rounding of the sum and moves half the bytes.
template <typename T>
__device__ __forceinline__ bool keeps_split(const Geo<T>& g, int i, T bcx, T bcz) {
  return bcx != T(0) || bcz != T(0) || (g.fsurf && i <= g.h + 1);
}

// tprev: stress totals at the start of the step (tt itself when the totals advance in place);
// tt: where the new totals go.
template <typename T, int NN>
__global__ void stress_pml_tot(Geo<T> g, int it, const T* __restrict__ cf, const T* __restrict__ v,
                               T* __restrict__ ts, T* tt, const T* tprev, const T* __restrict__ wav) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  EL_CELL_SHOTS
  const bool inside = in_I(g, i, j);
  bool split = true;
  T pxn = T(0), pzn = T(0), pxi = T(0), pzi = T(0);
  T c11 = T(0), c13 = T(0), c15 = T(0), c33 = T(0), c35 = T(0), c55 = T(0);
  if (inside) {
    const T bcx = cf[BCX * PL + occ], bcz = cf[BCZ * PL + occ];
    split = keeps_split(g, i, bcx, bcz);
    const T pxd = radd(T(1), rmul(g.hdt, bcx)), pzd = radd(T(1), rmul(g.hdt, bcz));
    pxn = rsub(T(1), rmul(g.hdt, bcx));
    pzn = rsub(T(1), rmul(g.hdt, bcz));
    pxi = rdiv_pml(T(1), pxd);
    pzi = rdiv_pml(T(1), pzd);
    c11 = cf[C11 * PL + occ];
    c13 = cf[C13 * PL + occ];
    c15 = cf[C15 * PL + occ];
    c33 = cf[C33 * PL + occ];
    c35 = cf[C35 * PL + occ];
    c55 = cf[C55 * PL + occ];
  }
#pragma unroll
  for (int q = 0; q < kCellShots; ++q) {
    const int s = s_lo + q;
    if (s >= g.ns) break;
    const int64_t o = (int64_t)s * PL + occ;
    if (!split) {
      const T* vx = v;
      const T* vz = v + NSP;
      const T dxbm_vx = dxb<NN>(g, vx, o), dxbm_vz = dxb<NN>(g, vz, o);
      const T dzbm_vx = dzb<NN>(g, vx, o), dzbm_vz = dzb<NN>(g, vz, o);
      const T dxfm_vx = dxf<NN>(g, vx, o), dzfm_vx = dzf<NN>(g, vx, o);
      const T dxfm_vz = dxf<NN>(g, vz, o), dzfm_vz = dzf<NN>(g, vz, o);
      T xx = radd(radd(tprev[TXX * NSP + o], rmul(g.dt_dx, radd(rmul(c11, dxbm_vx), rmul(c15, dxbm_vz)))),
                  rmul(g.dt_dz, radd(rmul(c15, dzbm_vx), rmul(c13, dzbm_vz))));
      T zz = radd(radd(tprev[TZZ * NSP + o], rmul(g.dt_dx, radd(rmul(c13, dxbm_vx), rmul(c35, dxbm_vz)))),
                  rmul(g.dt_dz, radd(rmul(c35, dzbm_vx), rmul(c33, dzbm_vz))));
      T xz = radd(radd(tprev[TXZ * NSP + o], rmul(g.dt_dx, radd(rmul(c15, dxfm_vx), rmul(c55, dxfm_vz)))),
                  rmul(g.dt_dz, radd(rmul(c55, dzfm_vx), rmul(c35, dzfm_vz))));
      if (i == g.src_z[s] && j == g.src_x[s]) {  // -MT/2 w on both split parts: twice on the total
        const T w = wav[(int64_t)s * g.nt + it];
        xx = radd(xx, rmul(T(2), rmul(g.src_m[3 * s + 0], w)));
        zz = radd(zz, rmul(T(2), rmul(g.src_m[3 * s + 1], w)));
        xz = radd(xz, rmul(T(2), rmul(g.src_m[3 * s + 2], w)));
      }
      tt[TXX * NSP + o] = xx;
      tt[TZZ * NSP + o] = zz;
      tt[TXZ * NSP + o] = xz;
      continue;
    }
    T sp[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) sp[k] = ts[k * NSP + o];
    if (inside) {
      const T* vx = v;
      const T* vz = v + NSP;
      const T dxbm_vx = dxb<NN>(g, vx, o), dxbm_vz = dxb<NN>(g, vz, o);
      const T dzbm_vx = dzb<NN>(g, vx, o), dzbm_vz = dzb<NN>(g, vz, o);
      const T dxfm_vx = dxf<NN>(g, vx, o), dzfm_vx = dzf<NN>(g, vx, o);
      const T dxfm_vz = dxf<NN>(g, vz, o), dzfm_vz = dzf<NN>(g, vz, o);
      sp[TXX_X] = rmul(radd(rmul(pxn, sp[TXX_X]), rmul(g.dt_dx, radd(rmul(c11, dxbm_vx), rmul(c15, dxbm_vz)))), pxi);
      sp[TXX_Z] = rmul(radd(rmul(pzn, sp[TXX_Z]), rmul(g.dt_dz, radd(rmul(c15, dzbm_vx), rmul(c13, dzbm_vz)))), pzi);
      sp[TZZ_X] = rmul(radd(rmul(pxn, sp[TZZ_X]), rmul(g.dt_dx, radd(rmul(c13, dxbm_vx), rmul(c35, dxbm_vz)))), pxi);
      sp[TZZ_Z] = rmul(radd(rmul(pzn, sp[TZZ_Z]), rmul(g.dt_dz, radd(rmul(c35, dzbm_vx), rmul(c33, dzbm_vz)))), pzi);
      sp[TXZ_X] = rmul(radd(rmul(pxn, sp[TXZ_X]), rmul(g.dt_dx, radd(rmul(c15, dxfm_vx), rmul(c55, dxfm_vz)))), pxi);
      sp[TXZ_Z] = rmul(radd(rmul(pzn, sp[TXZ_Z]), rmul(g.dt_dz, radd(rmul(c55, dzfm_vx), rmul(c35, dzfm_vz)))), pzi);
    }
    if (i == g.src_z[s] && j == g.src_x[s]) {
      const T w = wav[(int64_t)s * g.nt + it];
      const T axx = rmul(g.src_m[3 * s + 0], w), azz = rmul(g.src_m[3 * s + 1], w), axz = rmul(g.src_m[3 * s + 2], w);
      sp[TXX_X] = radd(sp[TXX_X], axx);
      sp[TXX_Z] = radd(sp[TXX_Z], axx);
      sp[TZZ_X] = radd(sp[TZZ_X], azz);
      sp[TZZ_Z] = radd(sp[TZZ_Z], azz);
      sp[TXZ_X] = radd(sp[TXZ_X], axz);
      sp[TXZ_Z] = radd(sp[TXZ_Z], axz);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) ts[k * NSP + o] = sp[k];
    if (!stress_fs_row(g, i)) {
      tt[TXX * NSP + o] = radd(sp[TXX_X], sp[TXX_Z]);
      tt[TZZ * NSP + o] = radd(sp[TZZ_X], sp[TZZ_Z]);
      tt[TXZ * NSP + o] = radd(sp[TXZ_X], sp[TXZ_Z]);
    }
  }
}

// Stress totals of the free-surface rows h-3 .. h-1 (elastic_kernels.py:375-384).
template <typename T>
__global__ void stress_fs_rows_pml(Geo<T> g, const T* __restrict__ ts, T* __restrict__ tt) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.L.nxp) return;
  const int i = g.h - 3 + (int)blockIdx.z, s = blockIdx.y;
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL, P = g.L.pitch;
  const int64_t o = (int64_t)s * PL + g.L.off(i, j);
  auto sum = [&](int f, int64_t oo) { return radd(ts[(2 * f) * NSP + oo], ts[(2 * f + 1) * NSP + oo]); };
  T xx = sum(TXX, o), zz = sum(TZZ, o), xz = sum(TXZ, o);
  const int h = g.h;
  if (i == h - 1) zz = T(0);
  if (i == h - 2) zz = -sum(TZZ, o + 2 * P);
  if (i == h - 2) xz = -sum(TXZ, o + P);
  if (i == h - 3) xz = -sum(TXZ, o + 3 * P);
  tt[TXX * NSP + o] = xx;
  tt[TZZ * NSP + o] = zz;
  tt[TXZ * NSP + o] = xz;
}

// vprev: velocity totals at the start of the step (v itself when they advance in place).
template <typename T, int NN>
__global__ void vel_pml_tot(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ tt, T* __restrict__ vs,
                            T* v, const T* vprev) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  EL_CELL_SHOTS
  const bool inside = in_I(g, i, j);
  bool split = true;
  T pxd = T(1), pxn = T(0), pzd = T(1), pzn = T(0), dbx = T(0), dbz = T(0);
  if (inside) {
    const T bcx = cf[BCX * PL + occ], bcz = cf[BCZ * PL + occ];
    split = keeps_split(g, i, bcx, bcz);
    pxd = radd(T(1), rmul(g.hdt, bcx));
    pxn = rsub(T(1), rmul(g.hdt, bcx));
    pzd = radd(T(1), rmul(g.hdt, bcz));
    pzn = rsub(T(1), rmul(g.hdt, bcz));
    dbx = rmul(g.dt, cf[BX * PL + occ]);
    dbz = rmul(g.dt, cf[BZ * PL + occ]);
  }
#pragma unroll
  for (int q = 0; q < kCellShots; ++q) {
    const int s = s_lo + q;
    if (s >= g.ns) break;
    const int64_t o = (int64_t)s * PL + occ;
    if (!split) {
      const T dxfm_txx = dxf<NN>(g, tt + TXX * NSP, o);
      const T dzbm_txz = dzb<NN>(g, tt + TXZ * NSP, o);
      const T dxbm_txz = dxb<NN>(g, tt + TXZ * NSP, o);
      const T dzfm_tzz = dzf<NN>(g, tt + TZZ * NSP, o);
      const T vx = radd(radd(vprev[VX * NSP + o], rdiv(rmul(dbx, dxfm_txx), g.dx)), rdiv(rmul(dbx, dzbm_txz), g.dz));
      const T vz = radd(radd(vprev[VZ * NSP + o], rdiv(rmul(dbz, dxbm_txz), g.dx)), rdiv(rmul(dbz, dzfm_tzz), g.dz));
      v[VX * NSP + o] = vx;
      v[VZ * NSP + o] = vz;
      continue;
    }
    T sv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) sv[k] = vs[k * NSP + o];
    if (inside) {
      const T dxfm_txx = dxf<NN>(g, tt + TXX * NSP, o);
      const T dzbm_txz = dzb<NN>(g, tt + TXZ * NSP, o);
      const T dxbm_txz = dxb<NN>(g, tt + TXZ * NSP, o);
      const T dzfm_tzz = dzf<NN>(g, tt + TZZ * NSP, o);
      sv[VX_X] = rdiv_pml(radd(rmul(pxn, sv[VX_X]), rdiv(rmul(dbx, dxfm_txx), g.dx)), pxd);
      sv[VX_Z] = rdiv_pml(radd(rmul(pzn, sv[VX_Z]), rdiv(rmul(dbx, dzbm_txz), g.dz)), pzd);
      sv[VZ_X] = rdiv_pml(radd(rmul(pxn, sv[VZ_X]), rdiv(rmul(dbz, dxbm_txz), g.dx)), pxd);
      sv[VZ_Z] = rdiv_pml(radd(rmul(pzn, sv[VZ_Z]), rdiv(rmul(dbz, dzfm_tzz), g.dz)), pzd);
#pragma unroll
      for (int k = 0; k < 4; ++k) vs[k * NSP + o] = sv[k];
    }
    if (!vel_fs_row(g, i, j)) {
      v[VX * NSP + o] = radd(sv[VX_X], sv[VX_Z]);
      v[VZ * NSP + o] = radd(sv[VZ_X], sv[VZ_Z]);
    }
  }
}

// Velocity totals of the free-surface rows h-3, h-2 (elastic_kernels.py:395-402), from the
// split velocities of all rows.
template <typename T>
__global__ void vel_fs_rows_pml(Geo<T> g, const T* __restrict__ vs, T* __restrict__ v) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < g.jlo || j > g.jhi || j >= g.L.nxp) return;
  const int i = g.h - 3 + (int)blockIdx.z, s = blockIdx.y;
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL, P = g.L.pitch;
  const int64_t o = (int64_t)s * PL + g.L.off(i, j);
  auto vxs = [&](int64_t oo) { return radd(vs[VX_X * NSP + oo], vs[VX_Z * NSP + oo]); };
  auto vzs = [&](int64_t oo) { return radd(vs[VZ_X * NSP + oo], vs[VZ_Z * NSP + oo]); };
  T vx = vxs(o), vz = vzs(o);
  const int h = g.h;
  if (i == h - 2) {
    const T vz_up = vzs(o + P);
    const T vzn_r = (j + 1 <= g.jhi) ? vzs(o + P + 1) : vzs(o + 1);
    vz = vz_up;
    vx = radd(rsub(radd(rsub(vzn_r, vz_up), vzs(o + P + 1)), vz_up), vxs(o + 2 * P));
  } else {
    vz = vzs(o + 2 * P);
  }
  v[VX * NSP + o] = vx;
  v[VZ * NSP + o] = vz;
}

// ======================================================================= forward, absorbing layer
template <typename T, int NN>
__global__ void stress_abl(Geo<T> g, int it, const T* __restrict__ cf, const T* __restrict__ v, T* __restrict__ ts,
                           const T* __restrict__ wav) {
  EL_CELL_SHOT
  const int64_t occ = g.L.off(i, j);
  if (in_I(g, i, j)) {
    const T* vx = v;
    const T* vz = v + NSP;
    const T dxbm_vx = dxb<NN>(g, vx, o), dxbm_vz = dxb<NN>(g, vz, o);
    const T dzbm_vx = dzb<NN>(g, vx, o), dzbm_vz = dzb<NN>(g, vz, o);
    const T dxfm_vx = dxf<NN>(g, vx, o), dzfm_vx = dzf<NN>(g, vx, o);
    const T dxfm_vz = dxf<NN>(g, vz, o), dzfm_vz = dzf<NN>(g, vz, o);
    const T c11 = cf[C11 * PL + occ], c13 = cf[C13 * PL + occ], c15 = cf[C15 * PL + occ];
    const T c33 = cf[C33 * PL + occ], c35 = cf[C35 * PL + occ], c55 = cf[C55 * PL + occ];
    T* f;
    f = ts + TXX * NSP + o;
    *f = radd(*f, rmul(g.dt, radd(rdiv(radd(rmul(c11, dxbm_vx), rmul(c15, dxbm_vz)), g.dx),
                                  rdiv(radd(rmul(c15, dzbm_vx), rmul(c13, dzbm_vz)), g.dz))));
    f = ts + TZZ * NSP + o;
    *f = radd(*f, rmul(g.dt, radd(rdiv(radd(rmul(c13, dxbm_vx), rmul(c35, dxbm_vz)), g.dx),
                                  rdiv(radd(rmul(c35, dzbm_vx), rmul(c33, dzbm_vz)), g.dz))));
    f = ts + TXZ * NSP + o;
    *f = radd(*f, rmul(g.dt, radd(rdiv(radd(rmul(c15, dxfm_vx), rmul(c55, dxfm_vz)), g.dx),
                                  rdiv(radd(rmul(c55, dzfm_vx), rmul(c35, dzfm_vz)), g.dz))));
  }
  if (i == g.src_z[s] && j == g.src_x[s]) {
    const T w = wav[(int64_t)s * g.nt + it];
    ts[TXX * NSP + o] = radd(ts[TXX * NSP + o], rmul(g.src_m[3 * s + 0], w));
    ts[TZZ * NSP + o] = radd(ts[TZZ * NSP + o], rmul(g.src_m[3 * s + 1], w));
    ts[TXZ * NSP + o] = radd(ts[TXZ * NSP + o], rmul(g.src_m[3 * s + 2], w));
  }
}

// Free-surface stress rows in place (elastic_kernels.py:738-742); one thread per column.
template <typename T>
__global__ void stress_fs_abl(Geo<T> g, T* __restrict__ ts) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.L.nxp) return;
  const int s = blockIdx.y, h = g.h;
  const int64_t NSP = (int64_t)g.ns * g.L.plane, so = (int64_t)s * g.L.plane;
  T* zz = ts + TZZ * NSP + so;
  T* xz = ts + TXZ * NSP + so;
  zz[g.L.off(h - 1, j)] = T(0);
  zz[g.L.off(h - 2, j)] = -zz[g.L.off(h, j)];
  xz[g.L.off(h - 2, j)] = -xz[g.L.off(h - 1, j)];
  xz[g.L.off(h - 3, j)] = -xz[g.L.off(h, j)];
}

template <typename T, int NN>
__global__ void vel_abl(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ tt, T* __restrict__ v) {
  EL_CELL_SHOT
  if (!in_I(g, i, j)) return;
  const int64_t occ = g.L.off(i, j);
  const T dxfm_txx = dxf<NN>(g, tt + TXX * NSP, o);
  const T dzbm_txz = dzb<NN>(g, tt + TXZ * NSP, o);
  const T dxbm_txz = dxb<NN>(g, tt + TXZ * NSP, o);
  const T dzfm_tzz = dzf<NN>(g, tt + TZZ * NSP, o);
  const T bx = cf[BX * PL + occ], bz = cf[BZ * PL + occ];
  T* f = v + VX * NSP + o;
  *f = radd(*f, rmul(rmul(g.dt, bx), radd(rdiv(dxfm_txx, g.dx), rdiv(dzbm_txz, g.dz))));
  f = v + VZ * NSP + o;
  *f = radd(*f, rmul(rmul(g.dt, bz), radd(rdiv(dxbm_txz, g.dx), rdiv(dzfm_tzz, g.dz))));
}

// Free-surface velocity rows in place (elastic_kernels.py:753-756); one thread per column in J.
// Reads only rows h-1, h and the cell (h-2, jhi+1), none of which any thread writes.
template <typename T>
__global__ void vel_fs_abl(Geo<T> g, T* __restrict__ v) {
  const int j = g.jlo + blockIdx.x * blockDim.x + threadIdx.x;
  if (j > g.jhi) return;
  const int s = blockIdx.y, h = g.h;
  const int64_t NSP = (int64_t)g.ns * g.L.plane, so = (int64_t)s * g.L.plane;
  T* vx = v + VX * NSP + so;
  T* vz = v + VZ * NSP + so;
  const T vz_up = vz[g.L.off(h - 1, j)];
  const T vzn_r = (j + 1 <= g.jhi) ? vz[g.L.off(h - 1, j + 1)] : vz[g.L.off(h - 2, j + 1)];
  const T vxh = vx[g.L.off(h, j)];
  const T vz_up_r = vz[g.L.off(h - 1, j + 1)];
  vz[g.L.off(h - 2, j)] = vz_up;
  vx[g.L.off(h - 2, j)] = radd(rsub(radd(rsub(vzn_r, vz_up), vz_up_r), vz_up), vxh);
  vz[g.L.off(h - 3, j)] = vz_up;
}

template <typename T>
__global__ void damp_v(Geo<T> g, const T* __restrict__ cf, T* __restrict__ v) {
  EL_CELL_SHOT
  const T d = cf[DAMP * PL + g.L.off(i, j)];
  v[VX * NSP + o] = rmul(v[VX * NSP + o], d);
  v[VZ * NSP + o] = rmul(v[VZ * NSP + o], d);
}

// Receivers: txx, tzz, txz, vx, vz totals at each receiver (elastic_kernels.py:407-411).
template <typename T>
__global__ void record(Geo<T> g, int it, const T* __restrict__ tt, const T* __restrict__ v, T* rec) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.nr) return;
  const int s = blockIdx.y;
  const int64_t NSP = (int64_t)g.ns * g.L.plane;
  const int64_t o = (int64_t)s * g.L.plane + g.L.off(g.rcv_z[r], g.rcv_x[r]);
  const int64_t RS = (int64_t)g.ns * g.nt * g.nr;
  const int64_t q = ((int64_t)s * g.nt + it) * g.nr + r;
  rec[0 * RS + q] = tt[TXX * NSP + o];
  rec[1 * RS + q] = tt[TZZ * NSP + o];
  rec[2 * RS + q] = tt[TXZ * NSP + o];
  rec[3 * RS + q] = v[VX * NSP + o];
  rec[4 * RS + q] = v[VZ * NSP + o];
}

// forward_wavefield_* += sum_s X^2 of the last step of a chunk (elastic_kernels.py:414-418, 1016-1021).
template <typename T>
__global__ void energy(Geo<T> g, const T* __restrict__ tt, const T* __restrict__ v, T* fw) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)g.nz * g.nx) return;
  const int i = (int)(e / g.nx) + g.top, j = (int)(e % g.nx) + g.nabc;
  const int64_t NSP = (int64_t)g.ns * g.L.plane, oc = g.L.off(i, j);
  const int64_t n = (int64_t)g.nz * g.nx;
  const T* src[5] = {tt + TXX * NSP, tt + TZZ * NSP, tt + TXZ * NSP, v + VX * NSP, v + VZ * NSP};
  for (int c = 0; c < 5; ++c) {
    T acc = T(0);
    for (int s = 0; s < g.ns; ++s) {
      T x = src[c][(int64_t)s * g.L.plane + oc];
      acc += x * x;
    }
    fw[c * n + e] += acc;
  }
}

// ======================================================================= adjoint
// Receiver residuals of step `it` into the adjoint stress totals lt (overwritten: zero + injection)
// and added to the adjoint velocity totals lv. One thread per (unique receiver cell, shot).
template <typename T>
__global__ void adj_inject(Geo<T> g, int it, const T* __restrict__ grec, T* lt, T* lv, int parts) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.ncells) return;
  const int s = blockIdx.y;
  const int64_t NSP = (int64_t)g.ns * g.L.plane;
  const int cell = g.ucell_zx[q];
  const int64_t o = (int64_t)s * g.L.plane + g.L.off(cell >> 16, cell & 0xffff);
  const int64_t RS = (int64_t)g.ns * g.nt * g.nr;
  const int64_t base = ((int64_t)s * g.nt + it) * g.nr;
  T a[5] = {T(0), T(0), T(0), T(0), T(0)};
  for (int m = g.ucell_beg[q]; m < g.ucell_beg[q + 1]; ++m) {
    const int64_t qq = base + g.ucell_rcv[m];
    for (int c = 0; c < 5; ++c) a[c] += grec[c * RS + qq];
  }
  if (parts & 2) {  // stresses
    lt[TXX * NSP + o] += a[0];
    lt[TZZ * NSP + o] += a[1];
    lt[TXZ * NSP + o] += a[2];
  }
  if (parts & 1) {  // velocities
    lv[VX * NSP + o] += a[3];
    lv[VZ * NSP + o] += a[4];
  }
}

// Adjoint of the free-surface velocity rows: lambda of the velocity totals BEFORE the rows
// h-3 / h-2 were overwritten (reverse of elastic_kernels.py:400-402), at cell (i, j).
template <typename T>
__device__ __forceinline__ void vfs_adjoint(const Geo<T>& g, const T* lvx, const T* lvz, int i, int j, int64_t o,
                                            T& ax, T& az) {
  const int64_t P = g.L.pitch;
  ax = lvx[o];
  az = lvz[o];
  if (!g.fsurf) return;
  const int h = g.h;
  auto inJ = [&](int m) { return m >= g.jlo && m <= g.jhi; };
  auto A = [&](int m, int64_t om) { return inJ(m) ? lvx[om] : T(0); };  // lambda vx[h-2, m] (om: offset of (h-2, m))
  if (i == h - 3) {
    if (inJ(j)) az = T(0);
  } else if (i == h - 2) {
    if (inJ(j)) {
      ax = T(0);
      az = T(0);
    } else if (inJ(j - 1)) {
      az = lvz[o] + lvx[o - 1];
    }
  } else if (i == h - 1) {
    const int64_t o2 = o - P;  // (h-2, j)
    T a_l = inJ(j - 1) ? lvx[o2 - 1] : T(0);
    T a_c = A(j, o2);
    T r = lvz[o] + a_l - a_c;
    if (inJ(j)) {
      const T b = lvz[o2 - P];  // lambda vz[h-3, j]
      const T cval = lvz[o2] + b + a_l - a_c;
      r += cval;
    }
    az = r;
  } else if (i == h) {
    if (inJ(j)) ax = lvx[o] + lvx[o - 2 * P];
  }
}

// Adjoint of the free-surface stress rows (reverse of elastic_kernels.py:381-384).
template <typename T>
__device__ __forceinline__ void tfs_adjoint(const Geo<T>& g, const T* lzz, const T* lxz, int i, int64_t o, T& azz,
                                            T& axz) {
  const int64_t P = g.L.pitch;
  azz = lzz[o];
  axz = lxz[o];
  if (!g.fsurf) return;
  const int h = g.h;
  if (i == h - 3) axz = T(0);
  if (i == h - 2) {
    axz = T(0);
    azz = T(0);
  }
  if (i == h - 1) {
    azz = T(0);
    axz = lxz[o] - lxz[o - P];
  }
  if (i == h) {
    azz = lzz[o] - lzz[o - 2 * P];
    axz = lxz[o] - lxz[o - 3 * P];
  }
}

template <typename T>
struct Pml {
  T xd, xn, zd, zn;
};
template <typename T>
__device__ __forceinline__ Pml<T> pml_at(const Geo<T>& g, const T* cf, int64_t oc, int64_t PL) {
  const T bcx = cf[BCX * PL + oc], bcz = cf[BCZ * PL + oc];
  Pml<T> p;
  p.xd = T(1) + g.hdt * bcx;
  p.xn = T(1) - g.hdt * bcx;
  p.zd = T(1) + g.hdt * bcz;
  p.zn = T(1) - g.hdt * bcz;
  return p;
}

// One plane of a (field, shot) block read at grid cells; the block's ghost frame is zero.
template <typename T>
struct PlaneQ {
  const T* base;
  Layout L;
  __device__ __forceinline__ T operator()(int ii, int jj) const { return base[L.off(ii, jj)]; }
};

// (B3q) the velocity update's adjoint sources, once per cell and shot (zero outside I):
// q = lambda(v split) * dt * b / (d * pml_d) for (vx_x, vx_z, vz_x, vz_z); PMLM = 0 uses the
// absorbing-layer velocities (no pml_d).
template <typename T, bool PMLM>
__global__ void adj_tq(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lvv, T* __restrict__ q4) {
  EL_CELL_SHOT
  T a = T(0), b = T(0), c = T(0), d = T(0);
  if (in_I(g, i, j)) {
    const int64_t c0 = g.L.off(i, j);
    const T bx = cf[BX * PL + c0], bz = cf[BZ * PL + c0];
    if (PMLM) {
      const Pml<T> p = pml_at(g, cf, c0, PL);
      a = lvv[VX_X * NSP + o] * (g.dt * bx) / (g.dx * p.xd);
      b = lvv[VX_Z * NSP + o] * (g.dt * bx) / (g.dz * p.zd);
      c = lvv[VZ_X * NSP + o] * (g.dt * bz) / (g.dx * p.xd);
      d = lvv[VZ_Z * NSP + o] * (g.dt * bz) / (g.dz * p.zd);
    } else {
      a = lvv[VX * NSP + o] * (g.dt * bx) / g.dx;
      b = lvv[VX * NSP + o] * (g.dt * bx) / g.dz;
      c = lvv[VZ * NSP + o] * (g.dt * bz) / g.dx;
      d = lvv[VZ * NSP + o] * (g.dt * bz) / g.dz;
    }
  }
  q4[0 * NSP + o] = a;
  q4[1 * NSP + o] = b;
  q4[2 * NSP + o] = c;
  q4[3 * NSP + o] = d;
}

// (B4 + B3a) per shot group: the split velocities' lambda after the step (the velocity
// free-surface adjoint, then S * lambda + lambda of the totals; read from lvs_in, written to
// lvs_out, so that no block reads a halo cell another block has already advanced), lt = the
// transposes of the velocity update's stress differences (the dL/d stress records of the step
// are added after it, by adj_inject), and the bx, bz gradients. The update's adjoint sources q
// (lambda of the split velocities times dt b / (d pml_d), zero outside I) are formed in shared
// memory where the transposes read them. Per block the tile's factors are formed once with the
// halo (S and dt b / (d pml_d); x factors on compact x planes, z factors on compact z planes).
// Per shot, the lambda of the four split velocities (x parts on compact x planes, z parts on
// compact z planes), the lambda of the velocity totals and txx, txz, tzz of the forward history
// (full planes) are staged into one of two buffers -- the next shot's copies are in flight while
// a shot is evaluated. Each thread then advances the lambda of its own cell (kept in registers
// for the gradients, stored for the next step) and of at most one halo cell, and turns the
// staged lambda into q in place; the transposes and gradients follow. 43.9 KB of shared memory
// in single precision.
constexpr int kAdjTShot = 2 * kXPlane + 2 * kZPlane + 5 * kSPlane;     // one shot's staged planes
constexpr int kAdjTElems = 3 * kXPlane + 3 * kZPlane + 2 * kAdjTShot;  // factors; two shot buffers
constexpr int kXHalo = kTileZ * 8, kZHalo = 6 * kTileX;  // halo cells of the compact x / z planes
static_assert(kXHalo + kZHalo == kTileThreads, "one halo cell per thread");
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
#ifndef ADFWI_EL_ADJT_MINB
#define ADFWI_EL_ADJT_MINB 5
#endif
template <typename T, int NN>
__global__ void __launch_bounds__(kTileThreads, sizeof(T) == 4 ? ADFWI_EL_ADJT_MINB : 2)
    adj_t_pml(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lv, const T* __restrict__ lvs_in,
              T* __restrict__ lvs_out, T* __restrict__ lt, const T* __restrict__ tt_hist, T* __restrict__ gpart,
              int eg) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  extern __shared__ __align__(16) unsigned char el_smem[];
  T* sFx = reinterpret_cast<T*>(el_smem);  // S_x, dt bx / (dx pml_xd), dt bz / (dx pml_xd) (x planes)
  T* sFz = sFx + 3 * kXPlane;              // S_z, dt bx / (dz pml_zd), dt bz / (dz pml_zd) (z planes)
  T* sB = sFz + 3 * kZPlane;               // two shot buffers
  // a shot buffer: lambda vx_x, vz_x (x planes; q_vxx, q_vzx once formed), lambda vx_z, vz_z (z
  // planes; q_vxz, q_vzz), lambda of the totals vx, vz, txx, txz, tzz (full planes)
  constexpr int oLz = 2 * kXPlane, oV = oLz + 2 * kZPlane, oT = oV + 2 * kSPlane;
  const int tiles_x = (g.L.nxp + kTileX - 1) / kTileX;
  const int i0 = ((int)blockIdx.x / tiles_x) * kTileZ, j0 = ((int)blockIdx.x % tiles_x) * kTileX;
  const int ty = (int)threadIdx.x / kTileX, tx = (int)threadIdx.x % kTileX;
  const int i = i0 + ty, j = j0 + tx;
  const bool valid = i < g.L.nzp && j < g.L.nxp, inside = valid && in_I(g, i, j);
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL, oc = g.L.off(i, j);
  const int sc = kSC + ty * kSW + tx, cx = ty * kSW + tx + 4, cz = (ty + 3) * kTileX + tx;
  // this thread's halo cell: x-plane columns j0-4 .. j0-1 and j0+32 .. j0+35, or z-plane rows
  // i0-3 .. i0-1 and i0+8 .. i0+10
  const bool hx = (int)threadIdx.x < kXHalo;
  int hr, hc;  // the halo cell's row and column relative to (i0, j0)
  if (hx) {
    const int c8 = (int)threadIdx.x & 7;
    hr = (int)threadIdx.x >> 3;
    hc = c8 < 4 ? c8 - 4 : c8 + kTileX - 4;
  } else {
    const int t = (int)threadIdx.x - kXHalo, r6 = t / kTileX;
    hr = r6 < 3 ? r6 - 3 : r6 + kTileZ - 3;
    hc = t - r6 * kTileX;
  }
  const int hi = i0 + hr, hj = j0 + hc;
  const bool hvalid = hi >= 0 && hi < g.L.nzp && hj >= 0 && hj < g.L.nxp;
  const int hs = hx ? hr * kSW + hc + 4 : (hr + 3) * kTileX + hc;  // in its compact plane
  const int hf = (hr + 3) * kSW + hc + 4;                            // in a full plane
  EL_SHOT_GROUP
  T* gbx = gbase + 6 * PL;
  T* gbz = gbase + 7 * PL;
  const T* lvx = lv + VX * NSP;
  const T* lvz = lv + VZ * NSP;
  auto issue = [&](int s, T* B) {
    const int64_t so = (int64_t)s * PL;
    stage_x(B, lvs_in + VX_X * NSP + so, g.L, i0, j0);
    stage_x(B + kXPlane, lvs_in + VZ_X * NSP + so, g.L, i0, j0);
    stage_z(B + oLz, lvs_in + VX_Z * NSP + so, g.L, i0, j0);
    stage_z(B + oLz + kZPlane, lvs_in + VZ_Z * NSP + so, g.L, i0, j0);
    stage(B + oV, lvx + so, g.L, i0, j0, 3, 4);
    stage(B + oV + kSPlane, lvz + so, g.L, i0, j0, 3, 4);
    stage(B + oT, tt_hist + TXX * NSP + so, g.L, i0, j0, 0, 4);
    stage(B + oT + kSPlane, tt_hist + TXZ * NSP + so, g.L, i0, j0, 3, 4);
    stage(B + oT + 2 * kSPlane, tt_hist + TZZ * NSP + so, g.L, i0, j0, 3, 0);
    cp_async_commit();
  };
  if (s_beg < s_end) issue(s_beg, sB);
  // the factors, formed as the per-cell adjoint forms them (S = 1 and the source factors zero
  // outside I), while the first shot's copies land
  for (int t = threadIdx.x; t < kXPlane; t += kTileThreads) {
    const int ii = i0 + t / kSW, jj = j0 - 4 + t % kSW;
    T sx = T(1), fx = T(0), fz = T(0);
    if (in_I(g, ii, jj)) {
      const int64_t c0 = g.L.off(ii, jj);
      const Pml<T> p = pml_at(g, cf, c0, PL);
      const T ix = T(1) / p.xd, kx = g.dt_dx * ix;
      sx = p.xn * ix;
      fx = cf[BX * PL + c0] * kx;
      fz = cf[BZ * PL + c0] * kx;
    }
    sFx[t] = sx;
    sFx[kXPlane + t] = fx;
    sFx[2 * kXPlane + t] = fz;
  }
  for (int t = threadIdx.x; t < kZPlane; t += kTileThreads) {
    const int ii = i0 - 3 + t / kTileX, jj = j0 + t % kTileX;
    T sz = T(1), fx = T(0), fz = T(0);
    if (in_I(g, ii, jj)) {
      const int64_t c0 = g.L.off(ii, jj);
      const Pml<T> p = pml_at(g, cf, c0, PL);
      const T iz = T(1) / p.zd, kz = g.dt_dz * iz;
      sz = p.zn * iz;
      fx = cf[BX * PL + c0] * kz;
      fz = cf[BZ * PL + c0] * kz;
    }
    sFz[t] = sz;
    sFz[kZPlane + t] = fx;
    sFz[2 * kZPlane + t] = fz;
  }
  // (the barrier after the first shot's copies orders these writes before their reads)
  // d(v_x')/d(bx) = dt * D(T) / (d * pml_d), likewise for bz: the cell's factors dt / (d pml_d)
  T kx = T(0), kz = T(0), gx = T(0), gz = T(0);
  if (inside) {
    const Pml<T> p = pml_at(g, cf, oc, PL);
    kx = g.dt / (g.dx * p.xd);
    kz = g.dt / (g.dz * p.zd);
  }
  // rows whose totals' lambda the velocity free-surface adjoint combines across cells
  const int fs_lo = g.fsurf ? g.h - 3 : 1 << 30, fs_hi = g.fsurf ? g.h : -1;
  auto q_of = [](T v, T f) { return f != T(0) ? v * f : T(0); };
  for (int s = s_beg; s < s_end; ++s) {
    T* B = sB + ((s - s_beg) & 1) * kAdjTShot;
    if (s + 1 < s_end) {
      issue(s + 1, sB + ((s + 1 - s_beg) & 1) * kAdjTShot);  // into the buffer the previous shot used
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_group<0>();
    }
    __syncthreads();
    const int64_t so = (int64_t)s * PL;
    T* sLx = B;
    T* sLz = B + oLz;
    // own cell: lambda after the step (cells outside the grid keep their zero), stored; q
    T vxx = sLx[cx], vzx = sLx[kXPlane + cx], vxz = sLz[cz], vzz = sLz[kZPlane + cz];
    if (valid) {
      const int64_t o = so + oc;
      T ax = B[oV + sc], az = B[oV + kSPlane + sc];
      if (i >= fs_lo && i <= fs_hi) vfs_adjoint(g, lvx, lvz, i, j, o, ax, az);
      const T sx = sFx[cx], sz = sFz[cz];
      vxx = sx * vxx + ax;
      vzx = sx * vzx + az;
      vxz = sz * vxz + ax;
      vzz = sz * vzz + az;
      lvs_out[VX_X * NSP + o] = vxx;
      lvs_out[VZ_X * NSP + o] = vzx;
      lvs_out[VX_Z * NSP + o] = vxz;
      lvs_out[VZ_Z * NSP + o] = vzz;
    }
    sLx[cx] = q_of(vxx, sFx[kXPlane + cx]);
    sLx[kXPlane + cx] = q_of(vzx, sFx[2 * kXPlane + cx]);
    sLz[cz] = q_of(vxz, sFz[kZPlane + cz]);
    sLz[kZPlane + cz] = q_of(vzz, sFz[2 * kZPlane + cz]);
    // halo cell: lambda after the step (not stored: another block owns the cell); q
    {
      T* hl = hx ? sLx + hs : sLz + hs;
      const int HP = hx ? kXPlane : kZPlane;
      const T* hF = hx ? sFx + hs : sFz + hs;
      T va = hl[0], vb = hl[HP];
      if (hvalid) {
        T ax = B[oV + hf], az = B[oV + kSPlane + hf];
        if (hi >= fs_lo && hi <= fs_hi) vfs_adjoint(g, lvx, lvz, hi, hj, so + g.L.off(hi, hj), ax, az);
        const T sh = hF[0];
        va = sh * va + ax;
        vb = sh * vb + az;
      }
      hl[0] = q_of(va, hF[HP]);
      hl[HP] = q_of(vb, hF[2 * HP]);
    }
    __syncthreads();
    if (valid) {
      const StagedX<T> q_vxx{sLx, i0, j0}, q_vzx{sLx + kXPlane, i0, j0};
      const StagedZ<T> q_vxz{sLz, i0, j0}, q_vzz{sLz + kZPlane, i0, j0};
      const T* sT = B + oT;
      const int64_t o = so + oc;
      lt[TXX * NSP + o] = dxf_t<NN>(g, q_vxx, i, j);
      lt[TXZ * NSP + o] = dzb_t<NN>(g, q_vxz, i, j) + dxb_t<NN>(g, q_vzx, i, j);
      lt[TZZ * NSP + o] = dzf_t<NN>(g, q_vzz, i, j);
      if (inside) {
        gx += vxx * dxf<NN>(g, sT, sc) * kx + vxz * dzb<NN>(g, sT + kSPlane, sc, kSW) * kz;
        gz += vzx * dxb<NN>(g, sT + kSPlane, sc) * kx + vzz * dzf<NN>(g, sT + 2 * kSPlane, sc, kSW) * kz;
      }
    }
    __syncthreads();  // this buffer is refilled by the copies of the shot after next
  }
  if (inside) {
    gbx[oc] += gx;
    gbz[oc] += gz;
  }
}

// Coefficient-weighted adjoint sources of the stress update at cell (ii, jj):
// q[0..5] = lambda of txx_x, txx_z, tzz_x, tzz_z, txz_x, txz_z times their d(update)/d(C D v).
template <typename T>
struct StressQ {
  T a, b, c, d, e, f;  // xx_x, xx_z, zz_x, zz_z, xz_x, xz_z
};

// Coefficient-weighted adjoint sources of the stress update at cell (i, j) of one shot.
// The cell's factors: dt/dx / pml_xd and dt/dz / pml_zd (PML form), dt/dx and dt/dz (ABL form).
template <typename T, bool PMLM>
__device__ __forceinline__ void stress_k(const Geo<T>& g, const T* __restrict__ cf, int64_t c0, int64_t PL, T& kx,
                                         T& kz) {
  if (PMLM) {
    const Pml<T> p = pml_at(g, cf, c0, PL);
    kx = g.dt_dx / p.xd;
    kz = g.dt_dz / p.zd;
  } else {
    kx = g.dt / g.dx;
    kz = g.dt / g.dz;
  }
}
template <typename T, bool PMLM>
__device__ __forceinline__ StressQ<T> stress_q(const T* __restrict__ lts, int64_t oo, int64_t NSP, T kx, T kz) {
  StressQ<T> r;
  if (PMLM) {
    r.a = lts[TXX_X * NSP + oo] * kx;
    r.b = lts[TXX_Z * NSP + oo] * kz;
    r.c = lts[TZZ_X * NSP + oo] * kx;
    r.d = lts[TZZ_Z * NSP + oo] * kz;
    r.e = lts[TXZ_X * NSP + oo] * kx;
    r.f = lts[TXZ_Z * NSP + oo] * kz;
  } else {
    r.a = lts[TXX * NSP + oo] * kx;
    r.b = lts[TXX * NSP + oo] * kz;
    r.c = lts[TZZ * NSP + oo] * kx;
    r.d = lts[TZZ * NSP + oo] * kz;
    r.e = lts[TXZ * NSP + oo] * kx;
    r.f = lts[TXZ * NSP + oo] * kz;
  }
  return r;
}

// (B1q) the stress update's adjoint sources for the velocity transposes, once per cell and
// shot (zero outside I): sx_b, sx_zb, sx_f, sx_zf, sz_b, sz_zb, sz_f, sz_zf.
template <typename T, bool PMLM>
__global__ void adj_vq(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lts, T* __restrict__ q8) {
  EL_CELL_SHOT
  T v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = T(0);
  if (in_I(g, i, j)) {
    const int64_t c0 = g.L.off(i, j);
    T kx, kz;
    stress_k<T, PMLM>(g, cf, c0, PL, kx, kz);
    const StressQ<T> r = stress_q<T, PMLM>(lts, o, NSP, kx, kz);
    const T c11 = cf[C11 * PL + c0], c13 = cf[C13 * PL + c0], c15 = cf[C15 * PL + c0];
    const T c33 = cf[C33 * PL + c0], c35 = cf[C35 * PL + c0], c55 = cf[C55 * PL + c0];
    v[0] = c11 * r.a + c13 * r.c;
    v[1] = c15 * r.b + c35 * r.d;
    v[2] = c15 * r.e;
    v[3] = c55 * r.f;
    v[4] = c15 * r.a + c35 * r.c;
    v[5] = c13 * r.b + c33 * r.d;
    v[6] = c55 * r.e;
    v[7] = c35 * r.f;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) q8[k * NSP + o] = v[k];
}

// (B1a) lambda of the velocity totals at the start of the step (overwrite) and the C gradients.
// pml = 1: split-field update; pml = 0: absorbing-layer update (lts then holds txx, tzz, txz,
// and lv is accumulated instead of overwritten because v' = v + ...).
// Staged planes per shot: 0-7 the stress update's adjoint sources (sx_b x, sx_zb z, sx_f x,
// sx_zf z, sz_b x, sz_zb z, sz_f x, sz_zf z), 8-9 vx, vz of the forward history (x, z),
// 10.. lambda of the (split) stresses (6 with the PML, 3 without).
template <bool PMLM>
constexpr int adj_v_planes() {
  return PMLM ? 16 : 13;
}
template <typename T, int NN, bool PMLM>
__global__ void __launch_bounds__(kTileThreads)
    adj_v(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lts, const T* __restrict__ q8,
          T* __restrict__ lv, const T* __restrict__ v_hist, T* __restrict__ gpart, int eg) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  extern __shared__ __align__(16) unsigned char el_smem[];
  T* sm = reinterpret_cast<T*>(el_smem);
  const int tiles_x = (g.L.nxp + kTileX - 1) / kTileX;
  const int i0 = ((int)blockIdx.x / tiles_x) * kTileZ, j0 = ((int)blockIdx.x % tiles_x) * kTileX;
  const int ty = (int)threadIdx.x / kTileX, tx = (int)threadIdx.x % kTileX;
  const int i = i0 + ty, j = j0 + tx;
  const bool valid = i < g.L.nzp && j < g.L.nxp, inside = valid && in_I(g, i, j);
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL, oc = g.L.off(i, j);
  const int sc = kSC + ty * kSW + tx;
  EL_SHOT_GROUP
  T* gc = gbase;
  T g11 = T(0), g13 = T(0), g15 = T(0), g33 = T(0), g35 = T(0), g55 = T(0);
  T kx = T(0), kz = T(0);
  if (inside) stress_k<T, PMLM>(g, cf, oc, PL, kx, kz);
  constexpr int nst = PMLM ? 6 : 3;
  for (int s = s_beg; s < s_end; ++s) {
    const int64_t so = (int64_t)s * PL;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      stage(sm + k * kSPlane, q8 + k * NSP + so, g.L, i0, j0, (k & 1) ? 3 : 0, (k & 1) ? 0 : 4);
    stage(sm + 8 * kSPlane, v_hist + VX * NSP + so, g.L, i0, j0, 3, 4);
    stage(sm + 9 * kSPlane, v_hist + VZ * NSP + so, g.L, i0, j0, 3, 4);
#pragma unroll
    for (int k = 0; k < nst; ++k) stage(sm + (10 + k) * kSPlane, lts + k * NSP + so, g.L, i0, j0, 0, 0);
    cp_async_wait_all();
    __syncthreads();
    if (valid) {
      const StagedQ<T> q0{sm, i0, j0}, q1{sm + kSPlane, i0, j0}, q2{sm + 2 * kSPlane, i0, j0},
          q3{sm + 3 * kSPlane, i0, j0}, q4{sm + 4 * kSPlane, i0, j0}, q5{sm + 5 * kSPlane, i0, j0},
          q6{sm + 6 * kSPlane, i0, j0}, q7{sm + 7 * kSPlane, i0, j0};
      const T avx = dxb_t<NN>(g, q0, i, j) + dzb_t<NN>(g, q1, i, j) + dxf_t<NN>(g, q2, i, j) + dzf_t<NN>(g, q3, i, j);
      const T avz = dxb_t<NN>(g, q4, i, j) + dzb_t<NN>(g, q5, i, j) + dxf_t<NN>(g, q6, i, j) + dzf_t<NN>(g, q7, i, j);
      const int64_t o = so + oc;
      if (PMLM) {
        lv[VX * NSP + o] = avx;
        lv[VZ * NSP + o] = avz;
      } else {
        lv[VX * NSP + o] += avx;
        lv[VZ * NSP + o] += avz;
      }
      if (inside) {
        const StressQ<T> r = stress_q<T, PMLM>(sm + 10 * kSPlane + sc, 0, kSPlane, kx, kz);
        const T* vx = sm + 8 * kSPlane;
        const T* vz = sm + 9 * kSPlane;
        const T dxb_vx = dxb<NN>(g, vx, sc), dxb_vz = dxb<NN>(g, vz, sc);
        const T dzb_vx = dzb<NN>(g, vx, sc, kSW), dzb_vz = dzb<NN>(g, vz, sc, kSW);
        const T dxf_vx = dxf<NN>(g, vx, sc), dxf_vz = dxf<NN>(g, vz, sc);
        const T dzf_vx = dzf<NN>(g, vx, sc, kSW), dzf_vz = dzf<NN>(g, vz, sc, kSW);
        g11 += r.a * dxb_vx;
        g13 += r.b * dzb_vz + r.c * dxb_vx;
        g15 += r.a * dxb_vz + r.b * dzb_vx + r.e * dxf_vx;
        g33 += r.d * dzb_vz;
        g35 += r.c * dxb_vz + r.d * dzb_vx + r.f * dzf_vz;
        g55 += r.e * dxf_vz + r.f * dzf_vx;
      }
    }
    __syncthreads();  // the next shot's copies overwrite the staged planes
  }
  if (inside) {
    gc[C11 * PL + oc] += g11;
    gc[C13 * PL + oc] += g13;
    gc[C15 * PL + oc] += g15;
    gc[C33 * PL + oc] += g33;
    gc[C35 * PL + oc] += g35;
    gc[C55 * PL + oc] += g55;
  }
}

// (B2 + B1a, PML) per shot group: the split stresses' lambda after the step (the stress
// free-surface adjoint, then S * lambda + lambda of the totals; read from lts_in, written to
// lts_out, so that no block reads a halo cell another block has already advanced), lambda of the
// velocity totals at the start of the step (overwrite) and the C gradients, with the stress
// update's adjoint sources formed in shared memory. Per block the tile's cell coefficients
// C11 .. C55 (full planes, with the halo) are staged once and the factors S_x and dt/dx / pml_xd
// (compact x planes), S_z and dt/dz / pml_zd (compact z planes; S = 1 and the source factors zero
// outside I) formed once. Per shot the lambda of the six split stresses (x parts on compact x
// planes, z parts on compact z planes), the lambda of the stress totals and vx, vz of the
// forward history (full planes) are staged into one of two buffers -- the next shot's copies
// are in flight while a shot is evaluated. Each thread then advances the lambda of its own cell
// (stored for the next step; its weighted lambda kept for the gradients) and of at most one
// halo cell and forms their eight sources q (sx_b, sx_zb, sx_f, sx_zf, sz_b, sz_zb, sz_f, sz_zf:
// coefficient-weighted lambda, zero outside I), three of each four over the lambda they are
// formed from; the transposes and gradients follow. 63.5 KB of shared memory in single
// precision.
constexpr int kAdjVShot = 3 * kXPlane + 3 * kZPlane + 5 * kSPlane;  // one shot's staged planes
constexpr int kAdjVPmlElems = 6 * kSPlane + 3 * kXPlane + 3 * kZPlane + 2 * kAdjVShot;  // C, factors, q; buffers
template <typename T, int NN>
__global__ void __launch_bounds__(kTileThreads, sizeof(T) == 4 ? 3 : 1)
    adj_v_pml(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lt, const T* __restrict__ lts_in,
              T* __restrict__ lts_out, T* __restrict__ lv, const T* __restrict__ v_hist, T* __restrict__ gpart,
              int eg) {
  griddep_wait();  // launched with programmatic serialisation in the PML time loops
  griddep_launch_dependents();
  extern __shared__ __align__(16) unsigned char el_smem[];
  T* sC = reinterpret_cast<T*>(el_smem);  // 6 full planes
  T* sKx = sC + 6 * kSPlane;              // S_x, dt/dx / pml_xd (x planes)
  T* sKz = sKx + 2 * kXPlane;             // S_z, dt/dz / pml_zd (z planes)
  T* sQx = sKz + 2 * kZPlane;             // the fourth x source q6 (x plane)
  T* sQz = sQx + kXPlane;                 // the fourth z source q7 (z plane)
  T* sB = sQz + kZPlane;                  // two shot buffers
  // a shot buffer: lambda txx_x, tzz_x, txz_x (x planes; then q0, q2, q4), lambda txx_z, tzz_z,
  // txz_z (z planes; then q1, q3, q5), lambda of txx, tzz, txz, and vx, vz (full planes)
  constexpr int oLz = 3 * kXPlane, oA = oLz + 3 * kZPlane, oV = oA + 3 * kSPlane;
  const int tiles_x = (g.L.nxp + kTileX - 1) / kTileX;
  const int i0 = ((int)blockIdx.x / tiles_x) * kTileZ, j0 = ((int)blockIdx.x % tiles_x) * kTileX;
  const int ty = (int)threadIdx.x / kTileX, tx = (int)threadIdx.x % kTileX;
  const int i = i0 + ty, j = j0 + tx;
  const bool valid = i < g.L.nzp && j < g.L.nxp, inside = valid && in_I(g, i, j);
  const int64_t PL = g.L.plane, NSP = (int64_t)g.ns * PL, oc = g.L.off(i, j);
  const int sc = kSC + ty * kSW + tx, cx = ty * kSW + tx + 4, cz = (ty + 3) * kTileX + tx;
  // this thread's halo cell: x-plane columns j0-4 .. j0-1 and j0+32 .. j0+35, or z-plane rows
  // i0-3 .. i0-1 and i0+8 .. i0+10
  const bool hx = (int)threadIdx.x < kXHalo;
  int hr, hc;  // the halo cell's row and column relative to (i0, j0)
  if (hx) {
    const int c8 = (int)threadIdx.x & 7;
    hr = (int)threadIdx.x >> 3;
    hc = c8 < 4 ? c8 - 4 : c8 + kTileX - 4;
  } else {
    const int t = (int)threadIdx.x - kXHalo, r6 = t / kTileX;
    hr = r6 < 3 ? r6 - 3 : r6 + kTileZ - 3;
    hc = t - r6 * kTileX;
  }
  const int hi = i0 + hr, hj = j0 + hc;
  const bool hvalid = hi >= 0 && hi < g.L.nzp && hj >= 0 && hj < g.L.nxp;
  const int hs = hx ? hr * kSW + hc + 4 : (hr + 3) * kTileX + hc;  // in its compact plane
  const int hf = (hr + 3) * kSW + hc + 4;                            // in a full plane
  EL_SHOT_GROUP
  T* gc = gbase;
  const T* lxx = lt + TXX * NSP;
  const T* lzz = lt + TZZ * NSP;
  const T* lxz = lt + TXZ * NSP;
#pragma unroll
  for (int k = 0; k < 6; ++k) stage(sC + k * kSPlane, cf + (C11 + k) * PL, g.L, i0, j0, 3, 4);
  cp_async_commit();
  auto issue = [&](int s, T* B) {
    const int64_t so = (int64_t)s * PL;
    // the x parts of the split stresses feed the sources of x differences, the z parts those of
    // z differences
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      stage_x(B + k * kXPlane, lts_in + (2 * k) * NSP + so, g.L, i0, j0);
      stage_z(B + oLz + k * kZPlane, lts_in + (2 * k + 1) * NSP + so, g.L, i0, j0);
    }
    stage(B + oA, lxx + so, g.L, i0, j0, 3, 4);
    stage(B + oA + kSPlane, lzz + so, g.L, i0, j0, 3, 4);
    stage(B + oA + 2 * kSPlane, lxz + so, g.L, i0, j0, 3, 4);
    stage(B + oV, v_hist + VX * NSP + so, g.L, i0, j0, 3, 4);
    stage(B + oV + kSPlane, v_hist + VZ * NSP + so, g.L, i0, j0, 3, 4);
    cp_async_commit();
  };
  if (s_beg < s_end) issue(s_beg, sB);
  // the factors, formed as the per-cell adjoint forms them, while the first copies land
  for (int t = threadIdx.x; t < kXPlane; t += kTileThreads) {
    const int ii = i0 + t / kSW, jj = j0 - 4 + t % kSW;
    T sx = T(1), kx = T(0);
    if (in_I(g, ii, jj)) {
      const int64_t c0 = g.L.off(ii, jj);
      const Pml<T> p = pml_at(g, cf, c0, PL);
      sx = p.xn * (T(1) / p.xd);
      kx = g.dt_dx / (T(1) + g.hdt * cf[BCX * PL + c0]);
    }
    sKx[t] = sx;
    sKx[kXPlane + t] = kx;
  }
  for (int t = threadIdx.x; t < kZPlane; t += kTileThreads) {
    const int ii = i0 - 3 + t / kTileX, jj = j0 + t % kTileX;
    T sz = T(1), kz = T(0);
    if (in_I(g, ii, jj)) {
      const int64_t c0 = g.L.off(ii, jj);
      const Pml<T> p = pml_at(g, cf, c0, PL);
      sz = p.zn * (T(1) / p.zd);
      kz = g.dt_dz / (T(1) + g.hdt * cf[BCZ * PL + c0]);
    }
    sKz[t] = sz;
    sKz[kZPlane + t] = kz;
  }
  // (the barrier after the first shot's copies orders these writes before their reads)
  // rows whose totals' lambda the stress free-surface adjoint combines across cells
  const int fs_lo = g.fsurf ? g.h - 3 : 1 << 30, fs_hi = g.fsurf ? g.h : -1;
  T g11 = T(0), g13 = T(0), g15 = T(0), g33 = T(0), g35 = T(0), g55 = T(0);
  for (int s = s_beg; s < s_end; ++s) {
    T* B = sB + ((s - s_beg) & 1) * kAdjVShot;
    if (s + 1 < s_end) {
      issue(s + 1, sB + ((s + 1 - s_beg) & 1) * kAdjVShot);  // into the buffer the previous shot used
      cp_async_wait_group<1>();
    } else {
      cp_async_wait_group<0>();
    }
    __syncthreads();
    const int64_t so = (int64_t)s * PL;
    T* sLx = B;
    T* sLz = B + oLz;
    const T* sA = B + oA;
    // own cell: lambda after the step (stored), the stress update's sources at the cell
    // (stress_q's PML form), then q
    StressQ<T> r;
    {
      T lxx_x = sLx[cx], lzz_x = sLx[kXPlane + cx], lxz_x = sLx[2 * kXPlane + cx];
      T lxx_z = sLz[cz], lzz_z = sLz[kZPlane + cz], lxz_z = sLz[2 * kZPlane + cz];
      if (valid) {
        const int64_t o = so + oc;
        const T axx = sA[sc];
        T azz = sA[kSPlane + sc], axz = sA[2 * kSPlane + sc];
        if (i >= fs_lo && i <= fs_hi) tfs_adjoint(g, lzz, lxz, i, o, azz, axz);
        const T sx = sKx[cx], sz = sKz[cz];
        lxx_x = sx * lxx_x + axx;
        lxx_z = sz * lxx_z + axx;
        lzz_x = sx * lzz_x + azz;
        lzz_z = sz * lzz_z + azz;
        lxz_x = sx * lxz_x + axz;
        lxz_z = sz * lxz_z + axz;
        lts_out[TXX_X * NSP + o] = lxx_x;
        lts_out[TXX_Z * NSP + o] = lxx_z;
        lts_out[TZZ_X * NSP + o] = lzz_x;
        lts_out[TZZ_Z * NSP + o] = lzz_z;
        lts_out[TXZ_X * NSP + o] = lxz_x;
        lts_out[TXZ_Z * NSP + o] = lxz_z;
      }
      const T kx = sKx[kXPlane + cx], kz = sKz[kZPlane + cz];
      r.a = lxx_x * kx;
      r.c = lzz_x * kx;
      r.e = lxz_x * kx;
      r.b = lxx_z * kz;
      r.d = lzz_z * kz;
      r.f = lxz_z * kz;
      const T c11 = sC[sc], c13 = sC[kSPlane + sc], c15 = sC[2 * kSPlane + sc];
      const T c33 = sC[3 * kSPlane + sc], c35 = sC[4 * kSPlane + sc], c55 = sC[5 * kSPlane + sc];
      T a = T(0), b = T(0), c = T(0), d = T(0);
      if (kx != T(0)) {  // inside I (the factor is positive there)
        a = c11 * r.a + c13 * r.c;
        b = c15 * r.e;
        c = c15 * r.a + c35 * r.c;
        d = c55 * r.e;
      }
      sLx[cx] = a;
      sLx[kXPlane + cx] = b;
      sLx[2 * kXPlane + cx] = c;
      sQx[cx] = d;
      a = b = c = d = T(0);
      if (kz != T(0)) {
        a = c15 * r.b + c35 * r.d;
        b = c55 * r.f;
        c = c13 * r.b + c33 * r.d;
        d = c35 * r.f;
      }
      sLz[cz] = a;
      sLz[kZPlane + cz] = b;
      sLz[2 * kZPlane + cz] = c;
      sQz[cz] = d;
    }
    // halo cell: lambda after the step (not stored: another block owns the cell), its sources
    {
      T* hl = hx ? sLx + hs : sLz + hs;
      const int HP = hx ? kXPlane : kZPlane;
      const T* hK = hx ? sKx + hs : sKz + hs;
      T l0 = hl[0], l1 = hl[HP], l2 = hl[2 * HP];  // lambda of the txx, tzz, txz part
      if (hvalid) {
        const T axx = sA[hf];
        T azz = sA[kSPlane + hf], axz = sA[2 * kSPlane + hf];
        if (hi >= fs_lo && hi <= fs_hi) tfs_adjoint(g, lzz, lxz, hi, so + g.L.off(hi, hj), azz, axz);
        const T sh = hK[0];
        l0 = sh * l0 + axx;
        l1 = sh * l1 + azz;
        l2 = sh * l2 + axz;
      }
      const T k = hK[HP];
      T a = T(0), b = T(0), c = T(0), d = T(0);
      if (k != T(0)) {
        const T r0 = l0 * k, r1 = l1 * k, r2 = l2 * k;
        if (hx) {  // ra, rc, re
          const T c15 = sC[2 * kSPlane + hf];
          a = sC[hf] * r0 + sC[kSPlane + hf] * r1;
          b = c15 * r2;
          c = c15 * r0 + sC[4 * kSPlane + hf] * r1;
          d = sC[5 * kSPlane + hf] * r2;
        } else {  // rb, rd, rf
          const T c35 = sC[4 * kSPlane + hf];
          a = sC[2 * kSPlane + hf] * r0 + c35 * r1;
          b = sC[5 * kSPlane + hf] * r2;
          c = sC[kSPlane + hf] * r0 + sC[3 * kSPlane + hf] * r1;
          d = c35 * r2;
        }
      }
      hl[0] = a;
      hl[HP] = b;
      hl[2 * HP] = c;
      (hx ? sQx : sQz)[hs] = d;
    }
    __syncthreads();
    if (valid) {
      const StagedX<T> q0{sLx, i0, j0}, q2{sLx + kXPlane, i0, j0}, q4{sLx + 2 * kXPlane, i0, j0}, q6{sQx, i0, j0};
      const StagedZ<T> q1{sLz, i0, j0}, q3{sLz + kZPlane, i0, j0}, q5{sLz + 2 * kZPlane, i0, j0}, q7{sQz, i0, j0};
      const T avx = dxb_t<NN>(g, q0, i, j) + dzb_t<NN>(g, q1, i, j) + dxf_t<NN>(g, q2, i, j) + dzf_t<NN>(g, q3, i, j);
      const T avz = dxb_t<NN>(g, q4, i, j) + dzb_t<NN>(g, q5, i, j) + dxf_t<NN>(g, q6, i, j) + dzf_t<NN>(g, q7, i, j);
      const int64_t o = so + oc;
      lv[VX * NSP + o] = avx;
      lv[VZ * NSP + o] = avz;
      if (inside) {
        const T* vx = B + oV;
        const T* vz = B + oV + kSPlane;
        const T dxb_vx = dxb<NN>(g, vx, sc), dxb_vz = dxb<NN>(g, vz, sc);
        const T dzb_vx = dzb<NN>(g, vx, sc, kSW), dzb_vz = dzb<NN>(g, vz, sc, kSW);
        const T dxf_vx = dxf<NN>(g, vx, sc), dxf_vz = dxf<NN>(g, vz, sc);
        const T dzf_vx = dzf<NN>(g, vx, sc, kSW), dzf_vz = dzf<NN>(g, vz, sc, kSW);
        g11 += r.a * dxb_vx;
        g13 += r.b * dzb_vz + r.c * dxb_vx;
        g15 += r.a * dxb_vz + r.b * dzb_vx + r.e * dxf_vx;
        g33 += r.d * dzb_vz;
        g35 += r.c * dxb_vz + r.d * dzb_vx + r.f * dzf_vz;
        g55 += r.e * dxf_vz + r.f * dzf_vx;
      }
    }
    __syncthreads();  // this buffer is refilled by the copies of the shot after next
  }
  if (inside) {
    gc[C11 * PL + oc] += g11;
    gc[C13 * PL + oc] += g13;
    gc[C15 * PL + oc] += g15;
    gc[C33 * PL + oc] += g33;
    gc[C35 * PL + oc] += g35;
    gc[C55 * PL + oc] += g55;
  }
}

// ABL (reverse of v *= damp and the free-surface velocity rows): lv_out = FS^T(damp * lv_in).
template <typename T>
__global__ void adj_vfs_abl(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lv_in, T* lv_out,
                            T* scratch) {
  EL_CELL_SHOT
  (void)scratch;
  // damp-weighted lambda at the cells the free-surface adjoint reads
  auto dl = [&](int comp, int64_t oo, int ii, int jj) { return cf[DAMP * PL + g.L.off(ii, jj)] * lv_in[comp * NSP + oo]; };
  T ax = dl(VX, o, i, j), az = dl(VZ, o, i, j);
  if (g.fsurf) {
    const int h = g.h;
    const int64_t P = g.L.pitch;
    auto inJ = [&](int m) { return m >= g.jlo && m <= g.jhi; };
    if (i == h - 3) {
      if (inJ(j)) az = T(0);
    } else if (i == h - 2) {
      if (inJ(j)) {
        ax = T(0);
        az = T(0);
      } else if (inJ(j - 1)) {
        az += dl(VX, o - 1, i, j - 1);
      }
    } else if (i == h - 1) {
      const int64_t o2 = o - P;
      const T a_l = inJ(j - 1) ? dl(VX, o2 - 1, i - 1, j - 1) : T(0);
      const T a_c = inJ(j) ? dl(VX, o2, i - 1, j) : T(0);
      T r = az + a_l - a_c;
      if (inJ(j)) r += dl(VZ, o2, i - 1, j) + dl(VZ, o2 - P, i - 2, j) + a_l - a_c;
      az = r;
    } else if (i == h) {
      if (inJ(j)) ax += dl(VX, o - 2 * P, i - 2, j);
    }
  }
  lv_out[VX * NSP + o] = ax;
  lv_out[VZ * NSP + o] = az;
}

// ABL: lt += transposes of the velocity update's stress differences; bx, bz gradients.
template <typename T, int NN>
__global__ void adj_t_abl(Geo<T> g, const T* __restrict__ cf, const T* __restrict__ lv,
                          const T* __restrict__ qv, T* lt, const T* __restrict__ tt_hist, T* gpart, int eg) {
  EL_CELL
  EL_SHOT_GROUP
  T* gbx = gbase + 6 * PL;
  T* gbz = gbase + 7 * PL;
  T gx = T(0), gz = T(0);
  for (int s = s_beg; s < s_end; ++s) {
    const int64_t so = (int64_t)s * PL;
    const PlaneQ<T> q1{qv + 0 * NSP + so, g.L}, q2{qv + 1 * NSP + so, g.L};
    const PlaneQ<T> q3{qv + 2 * NSP + so, g.L}, q4{qv + 3 * NSP + so, g.L};
    const int64_t o = so + oc;
    lt[TXX * NSP + o] += dxf_t<NN>(g, q1, i, j);
    lt[TXZ * NSP + o] += dzb_t<NN>(g, q2, i, j) + dxb_t<NN>(g, q3, i, j);
    lt[TZZ * NSP + o] += dzf_t<NN>(g, q4, i, j);
    if (in_I(g, i, j)) {
      const T* th = tt_hist;
      gx += lv[VX * NSP + o] * g.dt * (dxf<NN>(g, th + TXX * NSP, o) / g.dx + dzb<NN>(g, th + TXZ * NSP, o) / g.dz);
      gz += lv[VZ * NSP + o] * g.dt * (dxb<NN>(g, th + TXZ * NSP, o) / g.dx + dzf<NN>(g, th + TZZ * NSP, o) / g.dz);
    }
  }
  if (in_I(g, i, j)) {
    gbx[oc] += gx;
    gbz[oc] += gz;
  }
}

// ABL: stress free-surface adjoint in place, one thread per column.
template <typename T>
__global__ void adj_tfs_abl(Geo<T> g, T* lt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.L.nxp) return;
  const int s = blockIdx.y, h = g.h;
  const int64_t NSP = (int64_t)g.ns * g.L.plane, so = (int64_t)s * g.L.plane;
  T* zz = lt + TZZ * NSP + so;
  T* xz = lt + TXZ * NSP + so;
  const int64_t o3 = g.L.off(h - 3, j), o2 = g.L.off(h - 2, j), o1 = g.L.off(h - 1, j), o0 = g.L.off(h, j);
  xz[o0] -= xz[o3];
  xz[o3] = T(0);
  xz[o1] -= xz[o2];
  xz[o2] = T(0);
  zz[o0] -= zz[o2];
  zz[o2] = T(0);
  zz[o1] = T(0);
}

// Sum the shot groups' gradient partials (8 planes each) into the first group, in group order.
template <typename T>
__global__ void sum_groups(Layout L, int groups, T* part) {
  const int64_t n = (int64_t)L.nzp * L.nxp;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / L.nxp), j = (int)(e - (int64_t)i * L.nxp);
    const int64_t o = L.off(i, j);
    for (int q = 0; q < 8; ++q) {
      T acc = part[q * L.plane + o];
      for (int gr = 1; gr < groups; ++gr) acc += part[((int64_t)gr * 8 + q) * L.plane + o];
      part[q * L.plane + o] = acc;
    }
  }
}

template <typename T>
__global__ void pack(Layout L, int h, int w, const T* __restrict__ src, T* __restrict__ dst) {
  int64_t n = (int64_t)h * w;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / w), j = (int)(e - (int64_t)i * w);
    dst[L.off(i, j)] = src[e];
  }
}

template <typename T>
__global__ void unpack(Layout L, int h, int w, const T* __restrict__ src, T* __restrict__ dst) {
  int64_t n = (int64_t)h * w;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / w), j = (int)(e - (int64_t)i * w);
    dst[e] = src[L.off(i, j)];
  }
}

}  // namespace el
}  // namespace adfwi

// ----------------------------------------------------------------------------------------
// Plan, workspace and drivers.
// ----------------------------------------------------------------------------------------
using namespace adfwi;

struct adfwi_elastic_plan {
  adfwi_elastic_desc d;
  int nzp, nxp, NN, h, top;
  int nstate;           // state fields per shot: PML 6 split stresses + 4 split velocities + 2 v totals + 3 stress
                        // totals, ABL 3 + 2
  int K, nseg;
  int elem;
  Layout L;
  std::vector<int32_t> tab;
  std::vector<unsigned char> srcm;  // ns x 3 source weights (xx, zz, xz) in the solve's dtype
  PinnedBytes tab_pin, srcm_pin;    // page-locked copies of tab and srcm, the sources of each upload
  int64_t o_srcz, o_srcx, o_rcvz, o_rcvx, o_uzx, o_ubeg, o_urcv;
  int ncells;
  std::vector<int> chunk_end;  // last step of each reference checkpoint chunk
};

namespace {

int64_t al256(int64_t x) { return (x + 255) / 256 * 256; }

struct ECarve {
  int64_t coef, st, tt, vtmp, srcm, tab;       // forward
  int64_t snap, snap_scale, hv, ht, lst, lt, lv, lv2, qsrc, gc;  // gradient
  int64_t total;
};

// Coefficient planes: C11 C13 C15 C33 C35 C55 bx bz + (bcx bcz | damp)
int ncoef(const adfwi_elastic_plan* p) { return p->d.pml ? 10 : 9; }

// Shot groups of the gradient kernels: enough (cell, group) threads to fill the GPU (about
// 300 k), at most one group per shot.
int egroups(const adfwi_elastic_plan* p) {
  const int64_t cells = (int64_t)p->nzp * p->nxp;
#ifndef ADFWI_EL_THREADS
#define ADFWI_EL_THREADS 300000
#endif
  const int64_t want = ((int64_t)ADFWI_EL_THREADS + cells - 1) / cells;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(p->d.ns, want));
  const int eg = (p->d.ns + g - 1) / g;
  return (p->d.ns + eg - 1) / eg;
}
int eshots_per_group(const adfwi_elastic_plan* p) {
  const int g = egroups(p);
  return (p->d.ns + g - 1) / g;
}

ECarve ecarve(const adfwi_elastic_plan* p, bool grad, int K) {
  ECarve c{};
  const int64_t pl = p->L.plane * p->elem, ns = p->d.ns;
  int64_t o = 0;
  auto take = [&](int64_t b) { int64_t at = o; o += al256(b); return at; };
  const int nsplit = p->d.pml ? 10 : 3;  // fields updated in place (split stresses+velocities | stresses)
  c.coef = take(ncoef(p) * pl);
  c.st = take((int64_t)(p->d.pml ? 10 : 3) * ns * pl);  // PML: 6 split stresses + 4 split velocities
  c.tt = take(3 * ns * pl);                               // stress totals (PML) | unused (ABL)
  c.vtmp = take(2 * ns * pl);                             // velocity totals / ABL velocities
  c.srcm = take(ns * 3 * p->elem);
  c.tab = take((int64_t)p->tab.size() * 4);
  (void)nsplit;
  if (grad) {
    const bool full = K >= p->d.nt;
    const int nseg = (p->d.nt + K - 1) / K;
    const int64_t se = snapshot_value_bytes(p->d.snapshot_precision, p->elem);
    const int64_t nstate = p->nstate;
    c.snap = take(full ? 0 : (int64_t)nseg * nstate * ns * p->L.plane * se);
    c.snap_scale = take(full ? 0 : (int64_t)nseg * nstate * ns * 4);
    c.hv = take((int64_t)K * 2 * ns * pl);  // velocity totals at the start of each step
    c.ht = take((int64_t)K * 3 * ns * pl);  // stress totals after each step's free surface
    // lambda of the split stresses (6) and of the split velocities (4), twice each (a reverse
    // step reads one copy and writes the other)
    c.lst = take((int64_t)(p->d.pml ? 20 : 3) * ns * pl);
    c.lt = take(3 * ns * pl);
    c.lv = take(2 * ns * pl);
    c.lv2 = take(2 * ns * pl);
    // adjoint sources of the absorbing-layer step transposes (8 planes per shot; the PML kernels
    // form theirs in shared memory)
    c.qsrc = take(p->d.pml ? 0 : 8 * ns * pl);
    c.gc = take(8 * pl * egroups(p));
  }
  c.total = o;
  return c;
}

int echoose_K(const adfwi_elastic_plan* p) {
  const int nt = p->d.nt;
  const int64_t budget = p->d.memory_budget;
  if (p->d.snapshot_every > 0) return std::min(p->d.snapshot_every, nt);
  if (budget <= 0) return std::min(nt, std::max(1, (int)std::ceil(std::sqrt(2.4 * nt))));
  if (ecarve(p, true, nt).total <= budget) return nt;
  int kstar = std::min(nt - 1, std::max(1, (int)std::lround(std::sqrt(2.4 * nt))));
  while (kstar > 1 && ecarve(p, true, kstar - 1).total < ecarve(p, true, kstar).total) --kstar;
  while (kstar < nt - 1 && ecarve(p, true, kstar + 1).total < ecarve(p, true, kstar).total) ++kstar;
  if (ecarve(p, true, kstar).total > budget) return kstar;
  int lo = kstar, hi = nt - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (ecarve(p, true, mid).total <= budget) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
el::Geo<T> egeo(const adfwi_elastic_plan* p, const unsigned char* ws, const ECarve& c) {
  el::Geo<T> g;
  const adfwi_elastic_desc& d = p->d;
  g.L = p->L;
  g.ns = d.ns;
  g.nt = d.nt;
  g.nr = d.nr;
  g.fsurf = d.free_surface;
  g.h = p->h;
  g.ilo = p->NN;
  g.ihi = p->nzp - p->NN - 1;
  g.jlo = p->NN;
  g.jhi = p->nxp - p->NN - 1;
  g.top = p->top;
  g.nabc = d.nabc;
  g.nz = d.nz;
  g.nx = d.nx;
  g.dt = (T)d.dt;
  g.dx = (T)d.dx;
  g.dz = (T)d.dz;
  g.dt_dx = (T)(d.dt / d.dx);
  g.dt_dz = (T)(d.dt / d.dz);
  g.hdt = (T)(0.5 * d.dt);
  g.f0 = (T)d.fdc[0];
  g.f1 = (T)d.fdc[1];
  g.f2 = (T)(p->NN == 3 ? d.fdc[2] : 0.0);
  const int32_t* tb = reinterpret_cast<const int32_t*>(ws + c.tab);
  g.src_z = tb + p->o_srcz;
  g.src_x = tb + p->o_srcx;
  g.src_m = reinterpret_cast<const T*>(ws + c.srcm);
  g.rcv_z = tb + p->o_rcvz;
  g.rcv_x = tb + p->o_rcvx;
  g.ucell_zx = tb + p->o_uzx;
  g.ucell_beg = tb + p->o_ubeg;
  g.ucell_rcv = tb + p->o_urcv;
  g.ncells = p->ncells;
  return g;
}

// Blocks of the per-cell kernels (el::kTileThreads threads each): one per 32 x 8 tile.
inline dim3 cells_grid(const adfwi_elastic_plan* p, int ns) {
  const int64_t tiles = (int64_t)((p->nzp + el::kTileZ - 1) / el::kTileZ) * ((p->nxp + el::kTileX - 1) / el::kTileX);
  return dim3((unsigned)tiles, ns);
}

template <typename T>
int esetup(const adfwi_elastic_plan* p, unsigned char* ws, const ECarve& c, const void* const* coef,
           const int32_t* shapes, cudaStream_t st) {
  const int64_t pl = p->L.plane * p->elem;
  ADFWI_CUDA_TRY(cudaMemsetAsync(ws, 0, c.srcm, st));  // coefficient ghosts, state, totals
  ADFWI_CUDA_TRY(cudaMemcpyAsync(ws + c.tab, p->tab_pin.ptr, p->tab.size() * 4, cudaMemcpyHostToDevice, st));
  ADFWI_CUDA_TRY(cudaMemcpyAsync(ws + c.srcm, p->srcm_pin.ptr, p->srcm.size(), cudaMemcpyHostToDevice, st));
  for (int q = 0; q < ncoef(p); ++q) {
    const int h = shapes[2 * q], w = shapes[2 * q + 1];
    if (h < 1 || w < 1 || h > p->nzp || w > p->nxp) {
      set_error("coefficient %d has shape %dx%d, outside the %dx%d grid", q, h, w, p->nzp, p->nxp);
      return kBadArgument;
    }
    const int64_t n = (int64_t)h * w;
    ADFWI_LAUNCH(kAux, st, (el::pack<T><<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(
                               p->L, h, w, static_cast<const T*>(coef[q]),
                               reinterpret_cast<T*>(ws + c.coef + q * pl))));
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// One forward step. vin: velocity totals at the start of the step; vout: where the new
// totals go; tt: where the stress totals go (PML). ABL keeps v in vin (= vout) in place.
template <typename T, int NN>
void estep(const adfwi_elastic_plan* p, const el::Geo<T>& g, int it, const T* cf, const T* wav, T* st, T* tt,
           const T* tprev, const T* vin, T* vout, cudaStream_t s) {
  const dim3 gc = cells_grid(p, p->d.ns), b(el::kTileThreads);
  const int64_t NSP = (int64_t)p->d.ns * p->L.plane;
  if (p->d.pml) {
    T* ts = st;
    T* vs = st + 6 * NSP;
    const dim3 gcs = cells_grid(p, (p->d.ns + el::kCellShots - 1) / el::kCellShots);
    // programmatically serialised launches: each kernel waits for the previous one's data
    ADFWI_LAUNCH(kElFwdStep, s,
                 (void)launch_pdl_kernel(el::stress_pml_tot<T, NN>, gcs, b, 0, s, g, it, cf, vin, ts, tt, tprev, wav));
    if (p->d.free_surface) {
      const dim3 gfs((unsigned)((p->nxp + 127) / 128), p->d.ns, 3);
      ADFWI_LAUNCH(kElFwdStep, s, (void)launch_pdl_kernel(el::stress_fs_rows_pml<T>, gfs, dim3(128), 0, s, g, ts, tt));
    }
    ADFWI_LAUNCH(kElFwdStep, s, (void)launch_pdl_kernel(el::vel_pml_tot<T, NN>, gcs, b, 0, s, g, cf, tt, vs, vout, vin));
    if (p->d.free_surface) {
      const dim3 gfs((unsigned)((p->nxp + 127) / 128), p->d.ns, 2);
      ADFWI_LAUNCH(kElFwdStep, s, (void)launch_pdl_kernel(el::vel_fs_rows_pml<T>, gfs, dim3(128), 0, s, g, vs, vout));
    }
  } else {
    // ABL: stresses live in `tt`, velocities in place in vin (== vout)
    T* v = vout;
    if (vin != vout) cudaMemcpyAsync(v, vin, 2 * NSP * sizeof(T), cudaMemcpyDeviceToDevice, s);
    const dim3 gcol((unsigned)((p->nxp + 127) / 128), p->d.ns);
    ADFWI_LAUNCH(kElFwdStep, s, (el::stress_abl<T, NN><<<gc, b, 0, s>>>(g, it, cf, v, tt, wav)));
    if (p->d.free_surface) ADFWI_LAUNCH(kElFwdStep, s, (el::stress_fs_abl<T><<<gcol, 128, 0, s>>>(g, tt)));
    ADFWI_LAUNCH(kElFwdStep, s, (el::vel_abl<T, NN><<<gc, b, 0, s>>>(g, cf, tt, v)));
    if (p->d.free_surface) ADFWI_LAUNCH(kElFwdStep, s, (el::vel_fs_abl<T><<<gcol, 128, 0, s>>>(g, v)));
    ADFWI_LAUNCH(kElFwdStep, s, (el::damp_v<T><<<gc, b, 0, s>>>(g, cf, v)));
  }
}

// Snapshot helpers: the state of a step start is (PML) 10 split fields in st + 2 velocity
// totals + 3 stress totals (the cells without split fields keep their state in the totals), or
// (ABL) 3 stresses in tt + 2 velocities (nc = 0).
template <typename T>
int esnap(const adfwi_elastic_plan* p, bool store, unsigned char* ws, const ECarve& c, T* a, int64_t na, T* b,
          int64_t nb, T* cc, int64_t nc, int seg, cudaStream_t s) {
  const int64_t pl = p->L.plane;
  const int64_t first = (int64_t)seg * (na + nb + nc);
  T* parts[3] = {a, b, cc};
  const int64_t n[3] = {na, nb, nc};
  int64_t at = first;
  for (int q = 0; q < 3; ++q) {
    if (n[q] == 0) continue;
    const int rc =
        store ? snapshot_store<T>(p->d.snapshot_precision, parts[q], n[q], pl, ws + c.snap, ws + c.snap_scale, at, s)
              : snapshot_load<T>(p->d.snapshot_precision, parts[q], n[q], pl, ws + c.snap, ws + c.snap_scale, at, s);
    if (rc) return rc;
    at += n[q];
  }
  return kOk;
}

template <typename T, int NN>
int eforward(const adfwi_elastic_plan* p, const void* const* coef, const int32_t* shapes, const void* wavelet,
             void* rec, void* fw, bool grad, unsigned char* ws, int64_t ws_bytes, cudaStream_t s) {
  const int K = grad ? p->K : 1;
  ECarve c = ecarve(p, grad, K);
  if (ws_bytes < c.total) {
    set_error("workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)c.total);
    return kWorkspaceTooSmall;
  }
  int rc = esetup<T>(p, ws, c, coef, shapes, s);
  if (rc) return rc;
  el::Geo<T> g = egeo<T>(p, ws, c);
  const int64_t NSP = (int64_t)p->d.ns * p->L.plane;
  const T* cf = reinterpret_cast<const T*>(ws + c.coef);
  const T* wav = static_cast<const T*>(wavelet);
  T* stt = reinterpret_cast<T*>(ws + c.st);
  T* tt0 = reinterpret_cast<T*>(ws + c.tt);
  T* v0 = reinterpret_cast<T*>(ws + c.vtmp);
  const bool full = grad && K >= p->d.nt;
  T* hv = grad ? reinterpret_cast<T*>(ws + c.hv) : nullptr;
  T* ht = grad ? reinterpret_cast<T*>(ws + c.ht) : nullptr;
  const int nt = p->d.nt;
  if (fw) ADFWI_CUDA_TRY(cudaMemsetAsync(fw, 0, 5 * (int64_t)p->d.nz * p->d.nx * sizeof(T), s));
  if (full) {
    // the histories double as the state and are read with their halos
    int rc0 = zero_frames<T>(hv, (int64_t)K * 2 * p->d.ns, p->L, s);
    if (!rc0 && p->d.pml) rc0 = zero_frames<T>(ht, (int64_t)K * 3 * p->d.ns, p->L, s);
    if (rc0) return rc0;
  }
  size_t chunk = 0;
  for (int it = 0; it < nt; ++it) {
    if (grad && !full && it % K == 0) {
      if (p->d.pml)
        rc = esnap<T>(p, true, ws, c, stt, 10 * p->d.ns, v0, 2 * p->d.ns, tt0, 3 * p->d.ns, it / K, s);
      else
        rc = esnap<T>(p, true, ws, c, tt0, 3 * p->d.ns, v0, 2 * p->d.ns, nullptr, 0, it / K, s);
      if (rc) return rc;
    }
    T* vin = v0;
    T* vout = v0;
    T* tt = tt0;
    const T* tprev = tt0;  // stress totals at the start of the step
    if (full) {
      // the histories double as the state: Hv[it] = v at the start of step it, Ht[it] = T after it
      vin = it == 0 ? v0 : hv + (int64_t)it * 2 * NSP;
      vout = it + 1 < nt ? hv + (int64_t)(it + 1) * 2 * NSP : v0;
      if (it == 0) ADFWI_CUDA_TRY(cudaMemsetAsync(hv, 0, 2 * NSP * sizeof(T), s));
      if (it == 0) vin = hv;
      tt = p->d.pml ? ht + (int64_t)it * 3 * NSP : tt0;
      if (p->d.pml && it > 0) tprev = ht + (int64_t)(it - 1) * 3 * NSP;
    }
    estep<T, NN>(p, g, it, cf, wav, stt, tt, tprev, vin, vout, s);
    if (full && !p->d.pml) {
      // ABL: stresses evolve in tt0; keep a copy of this step's stresses for the adjoint
      ADFWI_CUDA_TRY(cudaMemcpyAsync(ht + (int64_t)it * 3 * NSP, tt0, 3 * NSP * sizeof(T), cudaMemcpyDeviceToDevice, s));
    }
    if (rec && p->d.nr > 0) {
      dim3 gr((unsigned)((p->d.nr + 127) / 128), p->d.ns);
      ADFWI_LAUNCH(kAux, s, (void)launch_pdl_kernel(el::record<T>, gr, dim3(128), 0, s, g, it, (const T*)tt, (const T*)vout,
                                                    static_cast<T*>(rec)));
    }
    if (fw && chunk < p->chunk_end.size() && it == p->chunk_end[chunk]) {
      const int64_t n = (int64_t)p->d.nz * p->d.nx;
      ADFWI_LAUNCH(kAux, s, (el::energy<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, tt, vout, static_cast<T*>(fw))));
      ++chunk;
    }
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

template <typename T, int NN>
int ebackward(const adfwi_elastic_plan* p, const void* wavelet, const void* grec, void* const* gcoef,
              const int32_t* shapes, unsigned char* ws, int64_t ws_bytes, cudaStream_t s) {
  const int K = p->K;
  ECarve c = ecarve(p, true, K);
  if (ws_bytes < c.total) {
    set_error("workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)c.total);
    return kWorkspaceTooSmall;
  }
  el::Geo<T> g = egeo<T>(p, ws, c);
  const int ns = p->d.ns, nt = p->d.nt;
  const int64_t PL = p->L.plane, NSP = (int64_t)ns * PL;
  const bool full = K >= nt;
  const T* cf = reinterpret_cast<const T*>(ws + c.coef);
  const T* wav = static_cast<const T*>(wavelet);
  T* stt = reinterpret_cast<T*>(ws + c.st);
  T* tt0 = reinterpret_cast<T*>(ws + c.tt);
  T* v0 = reinterpret_cast<T*>(ws + c.vtmp);
  T* hv = reinterpret_cast<T*>(ws + c.hv);
  T* ht = reinterpret_cast<T*>(ws + c.ht);
  T* lst = reinterpret_cast<T*>(ws + c.lst);
  T* lt = reinterpret_cast<T*>(ws + c.lt);
  T* lv = reinterpret_cast<T*>(ws + c.lv);
  T* lv2 = reinterpret_cast<T*>(ws + c.lv2);
  T* gcp = reinterpret_cast<T*>(ws + c.gc);
  T* qsrc = reinterpret_cast<T*>(ws + c.qsrc);
  const T* gr = static_cast<const T*>(grec);
  const int nsf = p->d.pml ? 20 : 3;
  ADFWI_CUDA_TRY(cudaMemsetAsync(lst, 0, nsf * NSP * sizeof(T), s));
  ADFWI_CUDA_TRY(cudaMemsetAsync(lt, 0, 3 * NSP * sizeof(T), s));
  ADFWI_CUDA_TRY(cudaMemsetAsync(lv, 0, 2 * NSP * sizeof(T), s));
  const int egr = egroups(p), eg = eshots_per_group(p);
  ADFWI_CUDA_TRY(cudaMemsetAsync(gcp, 0, (int64_t)egr * 8 * PL * sizeof(T), s));
  if (!p->d.pml) {
    // the source planes are read with their halos by the transposed stencils
    int rc0 = zero_frames<T>(qsrc, (int64_t)8 * ns, p->L, s);
    if (rc0) return rc0;
  }
  ADFWI_CUDA_TRY(cudaMemsetAsync(lv2, 0, 2 * NSP * sizeof(T), s));
  if (!full) {
    // recomputed histories are read with their halos
    int rc0 = zero_frames<T>(hv, (int64_t)K * 2 * ns, p->L, s);
    if (!rc0 && p->d.pml) rc0 = zero_frames<T>(ht, (int64_t)K * 3 * ns, p->L, s);
    if (rc0) return rc0;
  }
  const dim3 gcs = cells_grid(p, ns), gcg = cells_grid(p, egroups(p)), b(el::kTileThreads);
  const dim3 gcm = cells_grid(p, (ns + el::kCellShots - 1) / el::kCellShots);
  // shared memory of the staged gradient kernels (above the 48 KB default in double precision)
  const int smem_t = el::kAdjTElems * (int)sizeof(T);
  const int smem_vp = el::kAdjVPmlElems * (int)sizeof(T);
  const int smem_va = el::adj_v_planes<false>() * el::kSPlane * (int)sizeof(T);
  ADFWI_CUDA_TRY(cudaFuncSetAttribute(el::adj_t_pml<T, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_t));
  ADFWI_CUDA_TRY(cudaFuncSetAttribute(el::adj_v_pml<T, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_vp));
  ADFWI_CUDA_TRY(cudaFuncSetAttribute(el::adj_v<T, NN, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_va));
  const dim3 gcol((unsigned)((p->nxp + 127) / 128), ns);
  const dim3 ginj((unsigned)std::max(1, (p->ncells + 127) / 128), ns);
  const int nseg = full ? 1 : (nt + K - 1) / K;
  int flip = 0;  // which copy of the split velocities' lambda the next reverse step reads
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int t0 = full ? 0 : seg * K;
    const int t1 = full ? nt : std::min(nt, t0 + K);
    if (!full) {
      // restore the state at t0 (v totals straight into Hv[0]) and recompute the segment
      int rc = p->d.pml ? esnap<T>(p, false, ws, c, stt, 10 * ns, hv, 2 * ns, tt0, 3 * ns, seg, s)
                        : esnap<T>(p, false, ws, c, tt0, 3 * ns, hv, 2 * ns, nullptr, 0, seg, s);
      if (rc) return rc;
      for (int it = t0; it < t1; ++it) {
        const int k = it - t0;
        T* vin = hv + (int64_t)k * 2 * NSP;
        T* vout = k + 1 < K && it + 1 < t1 ? hv + (int64_t)(k + 1) * 2 * NSP : v0;
        T* tt = p->d.pml ? ht + (int64_t)k * 3 * NSP : tt0;
        const T* tprev = p->d.pml && k > 0 ? ht + (int64_t)(k - 1) * 3 * NSP : tt0;
        if (!p->d.pml && vout != vin) ADFWI_CUDA_TRY(cudaMemcpyAsync(vout, vin, 2 * NSP * sizeof(T), cudaMemcpyDeviceToDevice, s));
        estep<T, NN>(p, g, it, cf, wav, stt, tt, tprev, p->d.pml ? vin : vout, vout, s);
        if (!p->d.pml) ADFWI_CUDA_TRY(cudaMemcpyAsync(ht + (int64_t)k * 3 * NSP, tt0, 3 * NSP * sizeof(T), cudaMemcpyDeviceToDevice, s));
      }
    }
    for (int it = t1 - 1; it >= t0; --it) {
      const int k = it - t0;
      const T* vh = hv + (int64_t)k * 2 * NSP;  // velocity totals at the start of step it
      const T* th = ht + (int64_t)k * 3 * NSP;  // stress totals of step it
      if (p->d.pml) {
        // one stream of programmatically serialised launches per reverse step; lt is
        // overwritten by adj_t_pml before the stress-record gradients are added to it
        if (gr) ADFWI_LAUNCH(kAux, s, (void)launch_pdl_kernel(el::adj_inject<T>, ginj, dim3(128), 0, s, g, it, gr, lt, lv, 1));
        // lambda of the split stresses: planes 0-5 / 6-11 of lst, of the split velocities 12-15 /
        // 16-19; each reverse step reads one copy and writes the other
        const int f = flip;
        flip ^= 1;
        T* lvs_in = lst + (12 + 4 * f) * NSP;
        T* lvs_out = lst + (16 - 4 * f) * NSP;
        T* lts_in = lst + (6 * f) * NSP;
        T* lts_out = lst + (6 - 6 * f) * NSP;
        ADFWI_LAUNCH(kElAdjStep, s, (void)launch_pdl_kernel(el::adj_t_pml<T, NN>, gcg, b, (size_t)smem_t, s, g, cf,
                                                            (const T*)lv, (const T*)lvs_in, lvs_out, lt, th, gcp, eg));
        if (gr) ADFWI_LAUNCH(kAux, s, (void)launch_pdl_kernel(el::adj_inject<T>, ginj, dim3(128), 0, s, g, it, gr, lt, lv, 2));
        ADFWI_LAUNCH(kElAdjStep, s, (void)launch_pdl_kernel(el::adj_v_pml<T, NN>, gcg, b, (size_t)smem_vp, s, g, cf,
                                                            (const T*)lt, (const T*)lts_in, lts_out, lv, vh, gcp, eg));
      } else {
        if (gr) ADFWI_LAUNCH(kAux, s, (el::adj_inject<T><<<ginj, 128, 0, s>>>(g, it, gr, lst, lv, 3)));
        ADFWI_LAUNCH(kElAdjStep, s, (el::adj_vfs_abl<T><<<gcs, b, 0, s>>>(g, cf, lv, lv2, nullptr)));
        std::swap(lv, lv2);
        ADFWI_LAUNCH(kElAdjStep, s, (el::adj_tq<T, false><<<gcs, b, 0, s>>>(g, cf, lv, qsrc)));
        ADFWI_LAUNCH(kElAdjStep, s, (el::adj_t_abl<T, NN><<<gcg, b, 0, s>>>(g, cf, lv, qsrc, lst, th, gcp, eg)));
        if (p->d.free_surface) ADFWI_LAUNCH(kElAdjStep, s, (el::adj_tfs_abl<T><<<gcol, 128, 0, s>>>(g, lst)));
        ADFWI_LAUNCH(kElAdjStep, s, (el::adj_vq<T, false><<<gcs, b, 0, s>>>(g, cf, lst, qsrc)));
        ADFWI_LAUNCH(kElAdjStep, s, (el::adj_v<T, NN, false><<<gcg, b, smem_va, s>>>(g, cf, lst, qsrc, lv, vh, gcp, eg)));
      }
    }
    ADFWI_CUDA_TRY(cudaGetLastError());
  }
  if (egr > 1) {
    const int64_t n = (int64_t)p->nzp * p->nxp;
    ADFWI_LAUNCH(kAux, s, (el::sum_groups<T><<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
                              p->L, egr, gcp)));
  }
  // gradients out: C11 C13 C15 C33 C35 C55 bx bz, each cropped to its input shape
  for (int q = 0; q < 8; ++q) {
    if (gcoef[q] == nullptr) continue;
    const int h = shapes[2 * q], w = shapes[2 * q + 1];
    const int64_t n = (int64_t)h * w;
    ADFWI_LAUNCH(kAux, s, (el::unpack<T><<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
                              p->L, h, w, gcp + q * PL, static_cast<T*>(gcoef[q]))));
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace

extern "C" {

int adfwi_elastic_plan_create(const adfwi_elastic_desc* desc, const int32_t* src_z, const int32_t* src_x,
                              const int32_t* rcv_z, const int32_t* rcv_x, const double* moment_tensor,
                              adfwi_elastic_plan** out) {
  ADFWI_CHECK_ARG(desc && out, "null descriptor or output pointer");
  *out = nullptr;
  const adfwi_elastic_desc& d = *desc;
  ADFWI_CHECK_ARG(d.fd_order == 4 || d.fd_order == 6, "fd_order must be 4 or 6");
  ADFWI_CHECK_ARG(d.nz >= 3 && d.nx >= 3 && d.nabc >= 1, "need nz, nx >= 3 and nabc >= 1");
  ADFWI_CHECK_ARG(d.ns >= 1 && d.nt >= 1 && d.nr >= 0, "need ns >= 1, nt >= 1, nr >= 0");
  ADFWI_CHECK_ARG(d.dtype == ADFWI_F32 || d.dtype == ADFWI_F64, "dtype must be ADFWI_F32 or ADFWI_F64");
  ADFWI_CHECK_ARG(d.checkpoint_segments >= 1, "checkpoint_segments must be >= 1");
  ADFWI_CHECK_ARG(d.snapshot_precision >= 0 && d.snapshot_precision <= 3, "bad snapshot_precision");
  ADFWI_CHECK_ARG(src_z && src_x && moment_tensor && (d.nr == 0 || (rcv_z && rcv_x)), "null geometry array");
  adfwi_elastic_plan* p = new (std::nothrow) adfwi_elastic_plan();
  if (!p) {
    set_error("host allocation failed");
    return kBadArgument;
  }
  p->d = d;
  p->NN = d.fd_order / 2;
  p->h = p->NN + 1;
  const int fs_off = d.fd_order / 2;
  p->nxp = d.nx + 2 * d.nabc;
  p->nzp = d.nz + (d.free_surface ? d.nabc + fs_off : 2 * d.nabc + fs_off);
  p->top = d.free_surface ? fs_off : fs_off + d.nabc;
  p->elem = d.dtype == ADFWI_F64 ? 8 : 4;
  p->nstate = d.pml ? 15 : 5;
  p->L = make_layout(p->nzp, p->nxp, 16, 64, p->elem);
  std::vector<int32_t>& t = p->tab;
  p->o_srcz = t.size();
  for (int s = 0; s < d.ns; ++s) {
    const int z = src_z[s] + p->top, x = src_x[s] + d.nabc;
    if (z < 0 || z >= p->nzp || x < 0 || x >= p->nxp) {
      set_error("source %d at (z=%d, x=%d) lies outside the model", s, src_z[s], src_x[s]);
      delete p;
      return kBadGeometry;
    }
    t.push_back(z);
  }
  p->o_srcx = t.size();
  for (int s = 0; s < d.ns; ++s) t.push_back(src_x[s] + d.nabc);
  // source weights: PML adds -MT/2 * w to both split parts, ABL adds -1/3 * MT * w
  p->srcm.resize((size_t)3 * d.ns * p->elem);
  for (int s = 0; s < d.ns; ++s) {
    const double* m = moment_tensor + 9 * s;
    const int idx[3] = {0, 8, 2};  // MT[0,0], MT[2,2], MT[0,2]
    for (int k = 0; k < 3; ++k) {
      unsigned char* dst = p->srcm.data() + (size_t)(3 * s + k) * p->elem;
      if (d.dtype == ADFWI_F32) {
        const float mv = (float)m[idx[k]];
        const float w = d.pml ? -(mv / 2.0f) : (float)(-1.0 / 3.0) * mv;
        memcpy(dst, &w, sizeof(w));
      } else {
        const double w = d.pml ? -(m[idx[k]] / 2.0) : (-1.0 / 3.0) * m[idx[k]];
        memcpy(dst, &w, sizeof(w));
      }
    }
  }
  p->o_rcvz = t.size();
  for (int r = 0; r < d.nr; ++r) {
    const int z = rcv_z[r] + p->top, x = rcv_x[r] + d.nabc;
    if (z < 0 || z >= p->nzp || x < 0 || x >= p->nxp) {
      set_error("receiver %d at (z=%d, x=%d) lies outside the model", r, rcv_z[r], rcv_x[r]);
      delete p;
      return kBadGeometry;
    }
    t.push_back(z);
  }
  p->o_rcvx = t.size();
  for (int r = 0; r < d.nr; ++r) t.push_back(rcv_x[r] + d.nabc);
  // unique receiver cells
  std::vector<std::pair<int, int>> cells(d.nr);
  for (int r = 0; r < d.nr; ++r) cells[r] = {((rcv_z[r] + p->top) << 16) | (rcv_x[r] + d.nabc), r};
  std::stable_sort(cells.begin(), cells.end());
  std::vector<int32_t> uzx, ubeg, urcv;
  for (int q = 0; q < d.nr; ++q) {
    if (q == 0 || cells[q].first != cells[q - 1].first) {
      uzx.push_back(cells[q].first);
      ubeg.push_back((int32_t)urcv.size());
    }
    urcv.push_back(cells[q].second);
  }
  ubeg.push_back((int32_t)urcv.size());
  p->ncells = (int)uzx.size();
  p->o_uzx = t.size();
  t.insert(t.end(), uzx.begin(), uzx.end());
  p->o_ubeg = t.size();
  t.insert(t.end(), ubeg.begin(), ubeg.end());
  p->o_urcv = t.size();
  t.insert(t.end(), urcv.begin(), urcv.end());
  if (t.empty()) t.push_back(0);
  // torch.chunk(wavelet, checkpoint_segments): the energy maps keep the last step of each chunk
  const int chunk = (d.nt + d.checkpoint_segments - 1) / d.checkpoint_segments;
  for (int e = chunk - 1; e < d.nt; e += chunk) p->chunk_end.push_back(e);
  if (p->chunk_end.empty() || p->chunk_end.back() != d.nt - 1) p->chunk_end.push_back(d.nt - 1);
  if (!p->tab_pin.assign(p->tab.data(), p->tab.size() * 4) || !p->srcm_pin.assign(p->srcm.data(), p->srcm.size())) {
    delete p;
    return kCudaError;
  }
  p->K = echoose_K(p);
  p->nseg = (d.nt + p->K - 1) / p->K;
  *out = p;
  return kOk;
}

void adfwi_elastic_plan_destroy(adfwi_elastic_plan* p) { delete p; }

int adfwi_elastic_workspace_bytes(const adfwi_elastic_plan* p, int32_t with_gradient, int64_t* bytes) {
  ADFWI_CHECK_ARG(p && bytes, "null plan or output pointer");
  *bytes = ecarve(p, with_gradient != 0, with_gradient ? p->K : 1).total;
  return kOk;
}

int adfwi_elastic_snapshot_every(const adfwi_elastic_plan* p, int32_t* steps) {
  ADFWI_CHECK_ARG(p && steps, "null plan or output pointer");
  *steps = p->K;
  return kOk;
}

int adfwi_elastic_forward(const adfwi_elastic_plan* p, const void* const* coef, const int32_t* shapes,
                          const void* wavelet, void* rec, void* fw, int32_t with_gradient, void* workspace,
                          int64_t workspace_bytes, void* stream) {
  ADFWI_CHECK_ARG(p && coef && shapes && wavelet && workspace, "null argument");
  for (int q = 0; q < ncoef(p); ++q) ADFWI_CHECK_ARG(coef[q] != nullptr, "coefficient %d is null", q);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  const bool g = with_gradient != 0;
  if (p->d.dtype == ADFWI_F64)
    return p->NN == 2 ? eforward<double, 2>(p, coef, shapes, wavelet, rec, fw, g, ws, workspace_bytes, s)
                      : eforward<double, 3>(p, coef, shapes, wavelet, rec, fw, g, ws, workspace_bytes, s);
  return p->NN == 2 ? eforward<float, 2>(p, coef, shapes, wavelet, rec, fw, g, ws, workspace_bytes, s)
                    : eforward<float, 3>(p, coef, shapes, wavelet, rec, fw, g, ws, workspace_bytes, s);
}

int adfwi_elastic_backward(const adfwi_elastic_plan* p, const void* wavelet, const void* grad_rec,
                           void* const* grad_coef, const int32_t* shapes, void* workspace, int64_t workspace_bytes,
                           void* stream) {
  ADFWI_CHECK_ARG(p && wavelet && grad_coef && shapes && workspace, "null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (p->d.dtype == ADFWI_F64)
    return p->NN == 2 ? ebackward<double, 2>(p, wavelet, grad_rec, grad_coef, shapes, ws, workspace_bytes, s)
                      : ebackward<double, 3>(p, wavelet, grad_rec, grad_coef, shapes, ws, workspace_bytes, s);
  return p->NN == 2 ? ebackward<float, 2>(p, wavelet, grad_rec, grad_coef, shapes, ws, workspace_bytes, s)
                    : ebackward<float, 3>(p, wavelet, grad_rec, grad_coef, shapes, ws, workspace_bytes, s);
}

}  // extern "C"
