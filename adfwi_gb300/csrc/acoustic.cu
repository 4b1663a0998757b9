// Acoustic (p, u, w) 4th-order staggered-grid propagator for sm_103a: forward step,
// exact discrete adjoint step, checkpoint / recompute driver and the C ABI.
//
// Reference algorithm (paths inside liufeng2317/ADFWI):
//   ADFWI/propagator/acoustic_kernels.py:113-174  one time step (p update, source, free-surface
//                                                 mirror, u and w updates, w mirror, receivers,
//                                                 illumination sums)
//   ADFWI/propagator/acoustic_kernels.py:252-265  alpha / kappa coefficient definitions
//   ADFWI/propagator/acoustic_kernels.py:268-301  chunked time loop and the record dict
//
// One launch advances one time step of all shots (acoustic_tma.cuh, acoustic_vec.cuh):
// persistent, warp-specialised blocks stream (tile, shot) items through a TMA / mbarrier
// pipeline; per item the consumers compute the new pressure on a 16 x 64 tile plus its halo
// (1 row / column before, 2 after) and then the new u and w on the tile, four adjacent
// columns per thread, so p, u and w each cross HBM once per step (ping-pong buffers keep the
// Jacobi semantics of the reference's slice assignments). The forward arithmetic uses explicitly rounded operations (no FMA
// contraction) in the reference's evaluation order, so float32 records reproduce the
// reference's PyTorch CPU results bit for bit. The adjoint step is the exact transpose of
// the forward step, in reverse operation order.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/adfwi_gb300.h"
#include "common.cuh"
#include "frames.cuh"
#include "l2.cuh"
#include "snapshot.cuh"
#include "tma.cuh"

namespace adfwi {
namespace ac {

// Explicitly rounded arithmetic (keeps the reference's operation order; no FMA contraction).
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }

template <typename T>
struct Geo {
  Layout L;
  int ns, nt, nr;
  int fs;     // first stencil row of u/w (nabc with a free surface, else 1)
  int fsurf;  // free surface on / off
  int zbeg;   // first tiled row (fs-1 with a free surface: rows above never change)
  int tiles_x;
  int nabc, nz, nx;
  T dt;
  T c1, c2;
  const int* src_z;          // padded source rows (ns)
  const int* src_x;          // padded source columns (ns)
  const int* tile_rcv_beg;   // ntiles+1 offsets into trcv_*
  const int* trcv_cell;      // (local row << 16) | local column
  const int* trcv_id;        // receiver index
  const int* tile_cell_beg;  // ntiles+1 offsets into tcell_*
  const int* tcell_cell;     // unique receiver cells of a tile, packed like trcv_cell
  const int* tcell_rbeg;     // ncells+1 offsets into cell_rcv
  const int* cell_rcv;       // receiver indices grouped by unique cell
  const int* grp_beg;        // ngroups+1 offsets: shots of each shot group (a group has one model)
  const int* grp_model;      // model of each shot group
  // Fused misfit: when fz_tr is set, the dL/d p-records handed to the adjoint are the
  // normalised L2 misfit's adjoint source, formed from the synthetic records (the p-record
  // gradient pointer then holds them) and fz_obs with the per-trace factors fz_tr.
  const T* fz_obs;
  const l2::TraceFactors<T>* fz_tr;
  const double* fz_gmul;     // device scale of the source (the objective's gradient w.r.t. the loss)
  int fz_norm_obs;
};

// dL/d p-record of shot sh, step t, receiver rid: from the gradient array gp, or formed from the
// records (gp) and the observed data with the misfit's factors when the misfit is fused. In two
// parts, the loads (RecPIn) and the value from them, so that a caller handling several
// receivers issues every load before the arithmetic (the IEEE divisions of the source have an
// out-of-line slow path, across which later loads are not hoisted).
// (gmul: the source's scale, read once by the caller with fused_scale)
template <typename T>
struct RecPIn {
  T v, o;
  l2::TraceFactors<T> f;
};
template <typename T>
__device__ __forceinline__ RecPIn<T> grad_rec_p_load(const Geo<T>& g, const T* gp, int sh, int t, int rid) {
  RecPIn<T> r;
  const int64_t o = ((int64_t)sh * g.nt + t) * g.nr + rid;
  r.v = gp[o];
  if (g.fz_tr != nullptr) {
    r.o = g.fz_obs[o];
    r.f = g.fz_tr[(int64_t)sh * g.nr + rid];
  }
  return r;
}
template <typename T>
__device__ __forceinline__ T grad_rec_p_value(const Geo<T>& g, const RecPIn<T>& r, int t, T gmul) {
  return g.fz_tr == nullptr ? r.v : l2::source(r.f, r.v, r.o, t, g.fz_norm_obs, gmul);
}
template <typename T>
__device__ __forceinline__ T grad_rec_p(const Geo<T>& g, const T* gp, int sh, int t, int rid, T gmul) {
  return grad_rec_p_value(g, grad_rec_p_load(g, gp, sh, t, rid), t, gmul);
}
template <typename T>
__device__ __forceinline__ T fused_scale(const Geo<T>& g) {
  return g.fz_gmul != nullptr ? (T)*g.fz_gmul : T(1);
}

// Update regions of acoustic_kernels.py:115, 139, 151.
template <typename T>
__device__ __forceinline__ bool in_p(const Geo<T>& g, int i, int j) {
  return i >= g.fs + 1 && i <= g.L.nzp - 3 && j >= 2 && j <= g.L.nxp - 3;
}
template <typename T>
__device__ __forceinline__ bool in_u(const Geo<T>& g, int i, int j) {
  return i >= g.fs && i <= g.L.nzp - 2 && j >= 1 && j <= g.L.nxp - 3;
}
template <typename T>
__device__ __forceinline__ bool in_w(const Geo<T>& g, int i, int j) {
  return i >= g.fs && i <= g.L.nzp - 3 && j >= 1 && j <= g.L.nxp - 2;
}
template <typename T>
__device__ __forceinline__ bool in_window(const Geo<T>& g, int i, int j) {
  return i >= g.nabc && i < g.nabc + g.nz && j >= g.nabc && j < g.nabc + g.nx;
}

// Seed of the reverse pass: lambda = injection of the records of the last step.
template <typename T>
__global__ void adj_seed(Geo<T> g, int ntiles, int tz, int tx, const T* __restrict__ gr_p, const T* __restrict__ gr_u,
                         const T* __restrict__ gr_w, T* lp, T* lu, T* lw) {
  const int sh = blockIdx.y;
  const int64_t rowbase = ((int64_t)sh * g.nt + (g.nt - 1)) * g.nr;
  const int ncell = g.tile_cell_beg[ntiles];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ncell; q += gridDim.x * blockDim.x) {
    int tile = 0;
    {  // locate the tile of unique cell q (binary search on tile_cell_beg)
      int lo = 0, hi = ntiles;
      while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (g.tile_cell_beg[mid] <= q) lo = mid; else hi = mid;
      }
      tile = lo;
    }
    int cell = g.tcell_cell[q];
    int i = g.zbeg + (tile / g.tiles_x) * tz + (cell >> 16);
    int j = (tile % g.tiles_x) * tx + (cell & 0xffff);
    T ap = T(0), au = T(0), aw = T(0);
    const T gmul = fused_scale(g);
    for (int m = g.tcell_rbeg[q]; m < g.tcell_rbeg[q + 1]; ++m) {
      int64_t o = rowbase + g.cell_rcv[m];
      if (gr_p) ap += grad_rec_p(g, gr_p, sh, g.nt - 1, g.cell_rcv[m], gmul);
      if (gr_u) au += gr_u[o];
      if (gr_w) aw += gr_w[o];
    }
    int64_t o = (int64_t)sh * g.L.plane + g.L.off(i, j);
    lp[o] += ap;
    lu[o] += au;
    lw[o] += aw;
  }
}

// Copy a dense (h, w) array into a pitched plane at cell (0, 0) (ghosts untouched).
template <typename T>
__global__ void pack_plane(Layout L, int h, int w, const T* __restrict__ src, T* __restrict__ dst) {
  int64_t n = (int64_t)h * w;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / w), j = (int)(e - (int64_t)i * w);
    dst[L.off(i, j)] = src[e];
  }
}

// dst(h, w) = sum over `groups` partial planes of the window starting at (oi, oj).
template <typename T>
__global__ void reduce_planes(Layout L, int groups, int oi, int oj, int h, int w, const T* __restrict__ src,
                              T* __restrict__ dst) {
  int64_t n = (int64_t)h * w;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / w), j = (int)(e - (int64_t)i * w);
    T acc = T(0);
    for (int q = 0; q < groups; ++q) acc += src[(int64_t)q * L.plane + L.off(oi + i, oj + j)];
    dst[e] = acc;
  }
}

// forward_wavefield_{p,u,w} of the reference (acoustic_kernels.py:172-174, 285-288):
// fw_p = P, fw_u = P + U(last chunk), fw_w = fw_p + (U(last chunk) + sum_s w(last step)^2).
template <typename T>
__global__ void illum_finalize(Layout L, int groups, int ns, int nabc, int nz, int nx, const T* __restrict__ ip,
                               const T* __restrict__ iu, const T* __restrict__ wlast, T* fw_p, T* fw_u,
                               T* fw_w) {
  int64_t n = (int64_t)nz * nx;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(e / nx) + nabc, j = (int)(e % nx) + nabc;
    T P = T(0), U = T(0), W = T(0);
    for (int q = 0; q < groups; ++q) {
      P += ip[(int64_t)q * L.plane + L.off(i, j)];
      U += iu[(int64_t)q * L.plane + L.off(i, j)];
    }
    for (int s = 0; s < ns; ++s) {
      T v = wlast[(int64_t)s * L.plane + L.off(i, j)];
      W += v * v;
    }
    if (fw_p) fw_p[e] = P;
    if (fw_u) fw_u[e] = P + U;
    if (fw_w) fw_w[e] = P + (U + W);
  }
}

// Masked coefficient planes for the branch-free pipelined kernels, computed with the
// reference's own operations (acoustic_kernels.py:257-265, and 1 - kappa of 115-160):
//   A1M = alpha1 on the p region, 0 elsewhere;  B1 = 1 - damp*dt on the p region, 1 elsewhere;
//   A2U / A2W = alpha2 on the u / w regions, 0 elsewhere;
//   B2 / B3 = 1 - 0.5*(d + d_right)*dt / 1 - 0.5*(d + d_below)*dt on the u / w regions, 1 elsewhere.
// Ghost cells stay 0. Planes follow the raw a1, a2, damp planes in the coefficient block.
enum { kA1 = 0, kA2 = 1, kDamp = 2, kA1M = 3, kB1 = 4, kA2U = 5, kA2W = 6, kB2 = 7, kB3 = 8, kNumCoef = 9 };

template <typename T>
__global__ void mask_coefficients(Geo<T> g, T* cf) {
  const Layout L = g.L;
  const int64_t n = (int64_t)L.nzp * L.nxp;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / L.nxp), j = (int)(e - (int64_t)i * L.nxp);
    const int64_t o = L.off(i, j);
    const T* d = cf + kDamp * L.plane;
    const T a1 = cf[kA1 * L.plane + o], a2 = cf[kA2 * L.plane + o];
    const bool pin = in_p(g, i, j), uin = in_u(g, i, j), win = in_w(g, i, j);
    cf[kA1M * L.plane + o] = pin ? a1 : T(0);
    cf[kB1 * L.plane + o] = pin ? rsub(T(1), rmul(d[o], g.dt)) : T(1);
    cf[kA2U * L.plane + o] = uin ? a2 : T(0);
    cf[kB2 * L.plane + o] = uin ? rsub(T(1), rmul(rmul(T(0.5), radd(d[o], d[o + 1])), g.dt)) : T(1);
    cf[kA2W * L.plane + o] = win ? a2 : T(0);
    cf[kB3 * L.plane + o] = win ? rsub(T(1), rmul(rmul(T(0.5), radd(d[o], d[o + L.pitch])), g.dt)) : T(1);
  }
}

}  // namespace ac
}  // namespace adfwi

#include "acoustic_tma.cuh"
#include "acoustic_vec.cuh"
#include "bsave.cuh"

// ----------------------------------------------------------------------------------------
// Plan, workspace and drivers.
// ----------------------------------------------------------------------------------------
using namespace adfwi;

// Tiling of the grid for one kernel generation, with its receiver tables (offsets into tab).
struct Tiling {
  int tz, tx;
  int tiles_x, tiles_z, ntiles;
  int G, ngroups;  // shots per unit / units per tile
  int blocks;      // launch width of the adjoint step (persistent kernel)
  int fwd_blocks;  // launch width of the forward step (persistent kernel)
  int64_t o_trb, o_trc, o_tri, o_tcb, o_tcc, o_tcr, o_cr, o_gb, o_gm;
  int ncells;
};

struct adfwi_acoustic_plan {
  adfwi_acoustic_desc d;
  int nzp, nxp, fs, zbeg;
  Tiling t2;             // 16 x 64 tiles of the pipelined forward and adjoint steps
  int K, nseg;           // snapshot interval and number of segments (gradient mode)
  int last_chunk_start;  // first step of the reference's last checkpoint chunk
  int elem;              // bytes per element
  bool deep = false;     // deep-ring variants of the step kernels (FP32 only)
  bool bsave = false;    // gradient by boundary saving (snapshot_every = ADFWI_SNAP_EVERY_BOUNDARY)
  int nframe = 0;        // frame cells of a plane (boundary saving)
  int64_t o_fidx = 0, o_foff = 0;  // tab offsets: frame index of every cell (-1: interior), frame offsets
  ac::BsBox bbox{0, -1, 0, -1};     // the interior the reverse pass rebuilds
  int nm;                // models of a batched plan (1 otherwise)
  std::vector<int> model_shot_beg;  // nm+1 offsets: the shots of each model
  std::vector<int> model_grp_beg;   // nm+1 offsets: the shot groups of each model
  Layout L;
  std::vector<int32_t> tab;  // geometry tables, uploaded into the workspace
  PinnedBytes tab_pin;       // page-locked copy of tab, the source of each upload
  int64_t o_srcz, o_srcx;
};

namespace {

struct Carve {
  int64_t coef, fa, fb, ilp, ilu, tab, flag;  // forward
  int64_t snap, snap_scale, bsv, hp, hd, la, lb, g1, g2;  // gradient extras
  int64_t mst, mpk, mnorm, mfac;                     // fused misfit: trace stats, gather peaks, norms, factors
  int64_t total;
};

int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

// A gradient plan in boundary-saving mode (with a single step there is nothing to rebuild: the
// history of that step is kept).
bool boundary_saving(const adfwi_acoustic_plan* p) { return p->bsave && p->d.nt > 1; }

Carve carve(const adfwi_acoustic_plan* p, bool grad, int K) {
  Carve c{};
  const int64_t pl = p->L.plane * p->elem;
  const int64_t ns = p->d.ns;
  int64_t o = 0;
  auto take = [&](int64_t bytes) { int64_t at = o; o += align256(bytes); return at; };
  c.coef = take((int64_t)p->nm * ac::kNumCoef * pl);
  c.fa = take(3 * ns * pl);
  c.fb = take(3 * ns * pl);
  c.ilp = take((int64_t)p->t2.ngroups * pl);
  c.ilu = take((int64_t)p->t2.ngroups * pl);
  c.tab = take((int64_t)p->tab.size() * 4);
  c.flag = take(256);
  if (grad) {
    const int nseg = (p->d.nt + K - 1) / K;
    const bool bs = boundary_saving(p);
    const bool full = !bs && K >= p->d.nt;
    const int64_t snap_elem = snapshot_value_bytes(p->d.snapshot_precision, p->elem);
    c.snap = take(full || bs ? 0 : (int64_t)nseg * 3 * ns * p->L.plane * snap_elem);
    c.snap_scale = take(full || bs ? 0 : (int64_t)nseg * 3 * ns * 4);
    // boundary saving: the frame's p, u, w after each step (slot it: the state before step it)
    c.bsv = take(bs ? (int64_t)p->d.nt * 3 * ns * p->nframe * p->elem : 0);
    c.hp = take((int64_t)K * ns * pl);
    c.hd = take((int64_t)K * ns * pl);
    c.la = take(3 * ns * pl);
    c.lb = take(3 * ns * pl);
    c.g1 = take((int64_t)p->t2.ngroups * pl);
    c.g2 = take((int64_t)p->t2.ngroups * pl);
    const int64_t traces = (int64_t)ns * std::max(1, p->d.nr);
    const bool f64 = p->elem == 8;
    c.mst = take(traces * (f64 ? (int64_t)sizeof(l2::TraceStats<double>) : (int64_t)sizeof(l2::TraceStats<float>)));
    c.mpk = take(2 * ns * 8);
    c.mnorm = take(traces * 8);
    c.mfac = take(traces * (f64 ? (int64_t)sizeof(l2::TraceFactors<double>) : (int64_t)sizeof(l2::TraceFactors<float>)));
  }
  c.total = o;
  return c;
}

int choose_K(const adfwi_acoustic_plan* p) {
  const int nt = p->d.nt;
  const int64_t budget = p->d.memory_budget;
  if (p->bsave) return 1;  // one slot of divergence history, rebuilt step by step
  if (p->d.snapshot_every > 0) return std::min(p->d.snapshot_every, nt);
  if (budget <= 0) return std::min(nt, std::max(1, (int)std::ceil(std::sqrt(1.5 * nt))));
  // The whole history fits: the forward pass keeps it and no step is recomputed.
  if (carve(p, true, nt).total <= budget) return nt;
  // Otherwise: memory(K) = snapshots (falling with K) + segment history (rising with K) is
  // smallest near K* = sqrt(1.5 nt); take the longest segment beyond K* that still fits
  // (one recomputation pass either way, fewer snapshots).
  int kstar = std::min(nt - 1, std::max(1, (int)std::lround(std::sqrt(1.5 * nt))));
  while (kstar > 1 && carve(p, true, kstar - 1).total < carve(p, true, kstar).total) --kstar;
  while (kstar < nt - 1 && carve(p, true, kstar + 1).total < carve(p, true, kstar).total) ++kstar;
  if (carve(p, true, kstar).total > budget) return kstar;  // does not fit at all: the call reports it
  int lo = kstar, hi = nt - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) / 2;
    if (carve(p, true, mid).total <= budget) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
ac::Geo<T> make_geo(const adfwi_acoustic_plan* p, const unsigned char* ws, const Carve& c, const Tiling& t) {
  ac::Geo<T> g;
  g.L = p->L;
  g.ns = p->d.ns;
  g.nt = p->d.nt;
  g.nr = p->d.nr;
  g.fs = p->fs;
  g.fsurf = p->d.free_surface;
  g.zbeg = p->zbeg;
  g.tiles_x = t.tiles_x;
  g.nabc = p->d.nabc;
  g.nz = p->d.nz;
  g.nx = p->d.nx;
  g.dt = (T)p->d.dt;
  g.c1 = (T)(9.0 / 8.0);
  g.c2 = (T)(-1.0 / 24.0);
  const int32_t* tb = reinterpret_cast<const int32_t*>(ws + c.tab);
  g.src_z = tb + p->o_srcz;
  g.src_x = tb + p->o_srcx;
  g.tile_rcv_beg = tb + t.o_trb;
  g.trcv_cell = tb + t.o_trc;
  g.trcv_id = tb + t.o_tri;
  g.tile_cell_beg = tb + t.o_tcb;
  g.tcell_cell = tb + t.o_tcc;
  g.tcell_rbeg = tb + t.o_tcr;
  g.cell_rcv = tb + t.o_cr;
  g.grp_beg = tb + t.o_gb;
  g.grp_model = tb + t.o_gm;
  g.fz_obs = nullptr;
  g.fz_tr = nullptr;
  g.fz_gmul = nullptr;
  g.fz_norm_obs = 0;
  return g;
}

int grid_blocks(int64_t n) { return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 152 * 16); }

template <typename T>
int setup_common(const adfwi_acoustic_plan* p, unsigned char* ws, const Carve& c, const void* alpha1,
                 const void* alpha2, const void* damp, cudaStream_t st) {
  const int64_t pl = p->L.plane * p->elem;
  // Zero coefficient planes (ghosts), field buffers and illumination partials.
  ADFWI_CUDA_TRY(cudaMemsetAsync(ws + c.coef, 0, c.tab - c.coef, st));
  ADFWI_CUDA_TRY(cudaMemsetAsync(ws + c.flag, 0, 256, st));
  ADFWI_CUDA_TRY(cudaMemcpyAsync(ws + c.tab, p->tab_pin.ptr, p->tab.size() * 4, cudaMemcpyHostToDevice, st));
  const int64_t n = (int64_t)p->nzp * p->nxp;
  const void* src[3] = {alpha1, alpha2, damp};
  ac::Geo<T> g = make_geo<T>(p, ws, c, p->t2);
  for (int m = 0; m < p->nm; ++m) {  // model m's (nzp, nxp) planes into its coefficient block
    T* cf = reinterpret_cast<T*>(ws + c.coef + (int64_t)m * ac::kNumCoef * pl);
    for (int q = 0; q < 3; ++q) {
      ADFWI_LAUNCH(kAux, st, (ac::pack_plane<T><<<grid_blocks(n), 256, 0, st>>>(
                                  p->L, p->nzp, p->nxp, static_cast<const T*>(src[q]) + (int64_t)m * n,
                                  reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(cf) + q * pl))));
    }
    ADFWI_LAUNCH(kAux, st, (ac::mask_coefficients<T><<<grid_blocks(n), 256, 0, st>>>(g, cf)));
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// Stages of the TMA ring of each variant (deep: the FP32 variants compiled for VDEEP blocks per
// SM; FP64 has one variant).
template <typename T>
int vec_adj_stages(bool deep) {
  return sizeof(T) == 8 ? 2 : ((deep ? ac2::VDEEP : ac2::VAMINB) >= 3 ? 2 : 3);
}
template <typename T>
int vec_stages(bool deep) {
  return sizeof(T) == 8 ? 2 : ((deep ? ac2::VDEEP : ac2::VMINB) >= 3 ? 3 : 4);
}
template <typename T>
using StepKernel = void (*)(ac2::Maps, ac::Geo<T>, ac2::StepArgs<T>);
template <typename T>
StepKernel<T> fwd_kernel(bool deep) {
  if constexpr (sizeof(T) == 4) {
    if (deep) return ac2::fwd_step_vec<T, ac2::VDEEP>;
  }
  return ac2::fwd_step_vec<T, ac2::VMINB>;
}
template <typename T>
StepKernel<T> adj_kernel(bool deep) {
  if constexpr (sizeof(T) == 4) {
    if (deep) return ac2::adj_step_vec<T, ac2::VDEEP>;
  }
  return ac2::adj_step_vec<T, ac2::VAMINB>;
}

// Launch of a persistent step kernel with programmatic stream serialisation (the kernel
// calls griddepcontrol.wait before touching data of the previous launch).
template <typename T>
cudaError_t launch_pdl(void (*kernel)(ac2::Maps, ac::Geo<T>, ac2::StepArgs<T>), int blocks, int smem, cudaStream_t st,
                       const ac2::Maps& maps, const ac::Geo<T>& g, const ac2::StepArgs<T>& a) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(ac2::VTHREADS);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, maps, g, a);
}

template <typename T>
ac2::StepArgs<T> step_args(const adfwi_acoustic_plan* p, int it, const T* cf, int* flag) {
  ac2::StepArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.it = it;
  a.G = p->t2.G;
  a.ngroups = p->t2.ngroups;
  a.ntiles = p->t2.ntiles;
  a.cf = cf;
  a.cf_stride = (int64_t)ac::kNumCoef * p->L.plane;
  a.flag = flag;
  return a;
}

template <typename T>
int launch_fwd(const adfwi_acoustic_plan* p, const ac::Geo<T>& g, int it, int accum_u, const T* cf,
               const T* wav, const T* p0, const T* u0, const T* w0, T* p1, T* u1, T* w1, T* d1, T* rp, T* ru,
               T* rw, T* ilp, T* ilu, int* flag, cudaStream_t st) {
  const int64_t ns = p->d.ns;
  ac2::Maps maps;
  int rc = make_plane_map(&maps.a, u0, sizeof(T), p->L, ns, ac2::BOXX, ac2::EZ);
  if (!rc) rc = make_plane_map(&maps.b, w0, sizeof(T), p->L, ns, ac2::BOXX, ac2::WZ);
  if (!rc) rc = make_plane_map(&maps.c, p0, sizeof(T), p->L, ns, ac2::BOXX, ac2::EZ);
  if (rc) return rc;
  ac2::StepArgs<T> a = step_args<T>(p, it, cf, flag);
  a.accum_u = accum_u;
  a.stages = vec_stages<T>(p->deep);
  a.wav = wav;
  a.o0 = p1;
  a.o1 = u1;
  a.o2 = w1;
  a.d1 = d1;
  a.rec_p = rp;
  a.rec_u = ru;
  a.rec_w = rw;
  a.acc0 = ilp;
  a.acc1 = ilu;
  const int smem = ac2::VecFwdLayout<T>::bytes(a.stages);
  ADFWI_LAUNCH(kAcFwdStep, st,
               ADFWI_CUDA_TRY(launch_pdl(fwd_kernel<T>(p->deep), p->t2.fwd_blocks, smem, st, maps, g, a)));
  return kOk;
}

template <typename T>
int launch_adj(const adfwi_acoustic_plan* p, const ac::Geo<T>& g, int it, const T* cf, const T* lp0, const T* lu0,
               const T* lw0, T* lp1, T* lu1, T* lw1, const T* ph, const T* dh, const T* gp, const T* gu, const T* gw,
               T* g1, T* g2, int* flag, cudaStream_t st) {
  const int64_t ns = p->d.ns;
  ac2::Maps maps;
  int rc = make_plane_map(&maps.a, lu0, sizeof(T), p->L, ns, ac2::BOXX, ac2::EZ);
  if (!rc) rc = make_plane_map(&maps.b, lw0, sizeof(T), p->L, ns, ac2::BOXX, ac2::WZ);
  if (!rc) rc = make_plane_map(&maps.c, lp0, sizeof(T), p->L, ns, ac2::BOXX, ac2::EZ);
  if (!rc) rc = make_plane_map(&maps.d, ph, sizeof(T), p->L, ns, ac2::BOXX, ac2::EZ);
  if (!rc) rc = make_plane_map(&maps.e, dh, sizeof(T), p->L, ns, ac2::BOXX, ac2::EZ);
  if (rc) return rc;
  ac2::StepArgs<T> a = step_args<T>(p, it, cf, flag);
  a.stages = vec_adj_stages<T>(p->deep);
  a.o0 = lp1;
  a.o1 = lu1;
  a.o2 = lw1;
  a.rec_p = gp;
  a.rec_u = gu;
  a.rec_w = gw;
  a.acc0 = g1;
  a.acc1 = g2;
  const int smem = ac2::VecAdjLayout<T>::bytes(a.stages);
  ADFWI_LAUNCH(kAcAdjStep, st,
               ADFWI_CUDA_TRY(launch_pdl(adj_kernel<T>(p->deep), p->t2.blocks, smem, st, maps, g, a)));
  return kOk;
}

// The opt-in above 48 KB of dynamic shared memory is a property of the kernel in one device's
// context, so it is set once per device ordinal (and per element type), under a mutex: the
// serving workers call solves from several threads, and a process may drive more than one GPU.
std::mutex g_smem_mu;
std::vector<unsigned char> g_smem_done;  // bit 0: float kernels, bit 1: double kernels, per device

template <typename T>
int set_smem_limits() {
  int dev = 0;
  ADFWI_CUDA_TRY(cudaGetDevice(&dev));
  const unsigned char bit = sizeof(T) == 8 ? 2 : 1;
  std::lock_guard<std::mutex> lk(g_smem_mu);
  if ((int)g_smem_done.size() <= dev) g_smem_done.resize(dev + 1, 0);
  if (!(g_smem_done[dev] & bit)) {
    for (int deep = 0; deep < (sizeof(T) == 4 ? 2 : 1); ++deep) {
      ADFWI_CUDA_TRY(cudaFuncSetAttribute(fwd_kernel<T>(deep), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          ac2::VecFwdLayout<T>::bytes(vec_stages<T>(deep))));
      ADFWI_CUDA_TRY(cudaFuncSetAttribute(adj_kernel<T>(deep), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          ac2::VecAdjLayout<T>::bytes(vec_adj_stages<T>(deep))));
    }
    g_smem_done[dev] |= bit;
  }
  return kOk;
}

template <typename T>
int forward_impl(const adfwi_acoustic_plan* p, const void* alpha1, const void* alpha2, const void* damp,
                 const void* wavelet, void* rec_p, void* rec_u, void* rec_w, void* fw_p, void* fw_u,
                 void* fw_w, bool grad, unsigned char* ws, int64_t ws_bytes, cudaStream_t st) {
  int rc = set_smem_limits<T>();
  if (rc) return rc;
  const int K = grad ? p->K : 1;
  Carve c = carve(p, grad, K);
  if (ws_bytes < c.total) {
    set_error("workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)c.total);
    return kWorkspaceTooSmall;
  }
  rc = setup_common<T>(p, ws, c, alpha1, alpha2, damp, st);
  if (rc) return rc;
  ac::Geo<T> g = make_geo<T>(p, ws, c, p->t2);
  const int64_t pl = p->L.plane;
  const int64_t ns = p->d.ns;
  const T* cf = reinterpret_cast<const T*>(ws + c.coef);
  T* fa = reinterpret_cast<T*>(ws + c.fa);
  T* fb = reinterpret_cast<T*>(ws + c.fb);
  T* ilp = reinterpret_cast<T*>(ws + c.ilp);
  T* ilu = reinterpret_cast<T*>(ws + c.ilu);
  int* flag = reinterpret_cast<int*>(ws + c.flag);
  const T* wav = static_cast<const T*>(wavelet);
  const bool bs = grad && boundary_saving(p);
  const bool full = grad && !bs && K >= p->d.nt;
  T* hp = grad ? reinterpret_cast<T*>(ws + c.hp) : nullptr;
  T* hd = grad ? reinterpret_cast<T*>(ws + c.hd) : nullptr;
  if (full) {
    // the pressure history is read with its halo (as the next step's input and by the adjoint)
    rc = zero_frames<T>(hp, (int64_t)K * ns, p->L, st);
    if (rc) return rc;
  }
  T* cur = fa;
  T* nxt = fb;
  const int64_t bslot = (int64_t)3 * ns * p->nframe;  // elements of one boundary-saving slot
  for (int it = 0; it < p->d.nt; ++it) {
    if (grad && !full && !bs && it % K == 0) {
      rc = snapshot_store<T>(p->d.snapshot_precision, cur, 3 * ns, pl, ws + c.snap, ws + c.snap_scale,
                             (int64_t)(it / K) * 3 * ns, st);
      if (rc) return rc;
    }
    const T* p0 = cur;
    T* p1 = nxt;
    T* d1 = nullptr;
    if (full) {
      // the whole pressure history doubles as the pressure ping-pong buffer
      p0 = it == 0 ? cur : hp + (int64_t)(it - 1) * ns * pl;
      p1 = hp + (int64_t)it * ns * pl;
      d1 = hd + (int64_t)it * ns * pl;
    }
    rc = launch_fwd<T>(p, g, it, it >= p->last_chunk_start ? 1 : 0, cf, wav, p0, cur + ns * pl, cur + 2 * ns * pl,
                       p1, nxt + ns * pl, nxt + 2 * ns * pl, d1, static_cast<T*>(rec_p), static_cast<T*>(rec_u),
                       static_cast<T*>(rec_w), ilp, ilu, flag, st);
    if (rc) return rc;
    if (bs && it + 1 < p->d.nt) {
      const dim3 gs((unsigned)((p->nframe + 255) / 256), (unsigned)ns);
      const int* foff = reinterpret_cast<const int*>(ws + c.tab) + p->o_foff;
      ADFWI_LAUNCH(kAux, st, (ac::bs_save<T><<<gs, 256, 0, st>>>(p->L, (int)ns, p->nframe, foff, nxt,
                                                                  reinterpret_cast<T*>(ws + c.bsv) +
                                                                      (it + 1) * bslot)));
    }
    std::swap(cur, nxt);
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  if (fw_p || fw_u || fw_w) {
    const int64_t n = (int64_t)p->d.nz * p->d.nx;
    auto at = [&](void* f, int m) { return f ? static_cast<T*>(f) + (int64_t)m * n : nullptr; };
    for (int m = 0; m < p->nm; ++m) {  // model m: its groups' partial planes and its shots' last w
      const int g0 = p->model_grp_beg[m], s0 = p->model_shot_beg[m];
      ADFWI_LAUNCH(kAux, st, (ac::illum_finalize<T><<<grid_blocks(n), 256, 0, st>>>(
                                  p->L, p->model_grp_beg[m + 1] - g0, p->model_shot_beg[m + 1] - s0, p->d.nabc,
                                  p->d.nz, p->d.nx, ilp + (int64_t)g0 * pl, ilu + (int64_t)g0 * pl,
                                  cur + 2 * ns * pl + (int64_t)s0 * pl, at(fw_p, m), at(fw_u, m), at(fw_w, m))));
    }
    ADFWI_CUDA_TRY(cudaGetLastError());
  }
  return kOk;
}

// The normalised L2 misfit fused into the adjoint: the dL/d p-records are formed from the
// records (passed as the p-record gradient) and the observed data with the factors that
// l2_loss_impl left in the workspace, scaled by *gmul.
struct FusedL2 {
  const void* obs;
  const double* gmul;
  int norm_obs;
};

template <typename T>
int backward_impl(const adfwi_acoustic_plan* p, const void* wavelet, const void* grp, const void* gru,
                  const void* grw, void* ga1, void* ga2, unsigned char* ws, int64_t ws_bytes, cudaStream_t st,
                  const FusedL2* fz = nullptr) {
  int rc = set_smem_limits<T>();
  if (rc) return rc;
  const int K = p->K;
  Carve c = carve(p, true, K);
  if (ws_bytes < c.total) {
    set_error("workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)c.total);
    return kWorkspaceTooSmall;
  }
  ac::Geo<T> g2 = make_geo<T>(p, ws, c, p->t2);
  if (fz != nullptr) {
    g2.fz_obs = static_cast<const T*>(fz->obs);
    g2.fz_tr = reinterpret_cast<const l2::TraceFactors<T>*>(ws + c.mfac);
    g2.fz_gmul = fz->gmul;
    g2.fz_norm_obs = fz->norm_obs;
  }
  const int64_t pl = p->L.plane;
  const int64_t ns = p->d.ns;
  const int nt = p->d.nt;
  const bool full = K >= nt;
  const T* cf = reinterpret_cast<const T*>(ws + c.coef);
  T* fa = reinterpret_cast<T*>(ws + c.fa);
  T* fb = reinterpret_cast<T*>(ws + c.fb);
  T* hp = reinterpret_cast<T*>(ws + c.hp);
  T* hd = reinterpret_cast<T*>(ws + c.hd);
  T* la = reinterpret_cast<T*>(ws + c.la);
  T* lb = reinterpret_cast<T*>(ws + c.lb);
  T* g1p = reinterpret_cast<T*>(ws + c.g1);
  T* g2p = reinterpret_cast<T*>(ws + c.g2);
  int* flag = reinterpret_cast<int*>(ws + c.flag);
  const T* wav = static_cast<const T*>(wavelet);
  const T* gp = static_cast<const T*>(grp);
  const T* gu = static_cast<const T*>(gru);
  const T* gw = static_cast<const T*>(grw);

  ADFWI_CUDA_TRY(cudaMemsetAsync(la, 0, 3 * ns * pl * sizeof(T), st));
  ADFWI_CUDA_TRY(cudaMemsetAsync(lb, 0, 3 * ns * pl * sizeof(T), st));
  ADFWI_CUDA_TRY(cudaMemsetAsync(g1p, 0, (size_t)p->t2.ngroups * pl * sizeof(T), st));
  ADFWI_CUDA_TRY(cudaMemsetAsync(g2p, 0, (size_t)p->t2.ngroups * pl * sizeof(T), st));
  if (!full) {
    // the recomputed pressure history is read with its halo by the next step and the adjoint
    rc = zero_frames<T>(hp, (int64_t)K * ns, p->L, st);
    if (rc) return rc;
  }
  if (gp || gu || gw) {
    dim3 sg(std::max(1, std::min(64, (p->t2.ncells + 127) / 128)), p->d.ns);
    ADFWI_LAUNCH(kAux, st, (ac::adj_seed<T><<<sg, 128, 0, st>>>(g2, p->t2.ntiles, ac2::TZ, ac2::TX, gp, gu, gw, la,
                                                                   la + ns * pl, la + 2 * ns * pl)));
  }
  T* lcur = la;
  T* lnxt = lb;
  if (boundary_saving(p)) {
    // The forward left its last state in fa (nt even) or fb; rebuild the states backwards, the
    // pressure ping-ponging between the two buffers' p planes, u and w in place.
    T* sbuf = nt % 2 == 0 ? fa : fb;
    T* pcur = sbuf;
    T* poth = sbuf == fa ? fb : fa;
    T* u = sbuf + ns * pl;
    T* w = sbuf + 2 * ns * pl;
    const int* fidx = reinterpret_cast<const int*>(ws + c.tab) + p->o_fidx;
    const T* bsv = reinterpret_cast<const T*>(ws + c.bsv);
    const int64_t bslot = (int64_t)3 * ns * p->nframe;
    const dim3 gb(32, 8), gr((unsigned)((p->nxp + 31) / 32), (unsigned)((p->nzp + 7) / 8), (unsigned)ns);
    for (int it = nt - 1; it >= 0; --it) {
      const T* slot = it > 0 ? bsv + it * bslot : nullptr;
      ADFWI_LAUNCH(kAux, st, (ac::bs_reverse_uw<T><<<gr, gb, 0, st>>>(g2, p->bbox, fidx, cf, pcur, u, w, slot,
                                                                      p->nframe)));
      ADFWI_LAUNCH(kAux, st, (ac::bs_reverse_p<T><<<gr, gb, 0, st>>>(g2, p->bbox, it, fidx, cf, pcur, u, w, poth, hd,
                                                                     slot, p->nframe, wav)));
      rc = launch_adj<T>(p, g2, it, cf, lcur, lcur + ns * pl, lcur + 2 * ns * pl, lnxt, lnxt + ns * pl,
                         lnxt + 2 * ns * pl, pcur, hd, gp, gu, gw, g1p, g2p, flag, st);
      if (rc) return rc;
      std::swap(lcur, lnxt);
      std::swap(pcur, poth);
    }
    ADFWI_CUDA_TRY(cudaGetLastError());
  }
  const int nseg = boundary_saving(p) ? 0 : (full ? 1 : (nt + K - 1) / K);
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int t0 = full ? 0 : seg * K;
    const int t1 = full ? nt : std::min(nt, t0 + K);
    if (!full) {
      // Recompute the segment from its snapshot, keeping p and the divergence of every step.
      rc = snapshot_load<T>(p->d.snapshot_precision, fa, 3 * ns, pl, ws + c.snap, ws + c.snap_scale,
                            (int64_t)seg * 3 * ns, st);
      if (rc) return rc;
      T* cur = fa;
      T* nxt = fb;
      for (int it = t0; it < t1; ++it) {
        const T* p0 = it == t0 ? fa : hp + (int64_t)(it - 1 - t0) * ns * pl;
        rc = launch_fwd<T>(p, g2, it, 0, cf, wav, p0, cur + ns * pl, cur + 2 * ns * pl,
                           hp + (int64_t)(it - t0) * ns * pl, nxt + ns * pl, nxt + 2 * ns * pl,
                           hd + (int64_t)(it - t0) * ns * pl, nullptr, nullptr, nullptr, nullptr, nullptr, flag, st);
        if (rc) return rc;
        std::swap(cur, nxt);
      }
    }
    for (int it = t1 - 1; it >= t0; --it) {
      rc = launch_adj<T>(p, g2, it, cf, lcur, lcur + ns * pl, lcur + 2 * ns * pl, lnxt, lnxt + ns * pl,
                         lnxt + 2 * ns * pl, hp + (int64_t)(it - t0) * ns * pl, hd + (int64_t)(it - t0) * ns * pl, gp,
                         gu, gw, g1p, g2p, flag, st);
      if (rc) return rc;
      std::swap(lcur, lnxt);
    }
    ADFWI_CUDA_TRY(cudaGetLastError());
  }
  const int64_t n = (int64_t)p->nzp * p->nxp;
  for (int m = 0; m < p->nm; ++m) {  // model m's gradients: the sum over its groups' partial planes
    const int g0 = p->model_grp_beg[m], ng = p->model_grp_beg[m + 1] - g0;
    ADFWI_LAUNCH(kAux, st, (ac::reduce_planes<T><<<grid_blocks(n), 256, 0, st>>>(
                                p->L, ng, 0, 0, p->nzp, p->nxp, g1p + (int64_t)g0 * pl, static_cast<T*>(ga1) + m * n)));
    ADFWI_LAUNCH(kAux, st, (ac::reduce_planes<T><<<grid_blocks(n), 256, 0, st>>>(
                                p->L, ng, 0, 0, p->nzp, p->nxp, g2p + (int64_t)g0 * pl, static_cast<T*>(ga2) + m * n)));
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// Normalised L2 misfit of the records `syn` against `obs` (the misfit of adfwi_l2_misfit) into
// the gradient workspace's factor arrays, and each model's loss: the sum of its traces' norms.
template <typename T>
int l2_loss_impl(const adfwi_acoustic_plan* p, const void* syn, const void* obs, double silent_rel, int flags,
                 double* loss, unsigned char* ws, int64_t ws_bytes, cudaStream_t st) {
  const Carve c = carve(p, true, p->K);
  if (ws_bytes < c.total) {
    set_error("workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)c.total);
    return kWorkspaceTooSmall;
  }
  const int ns = p->d.ns, nt = p->d.nt, nr = p->d.nr;
  auto* stats = reinterpret_cast<l2::TraceStats<T>*>(ws + c.mst);
  auto* gsyn = reinterpret_cast<l2::PeakWord<T>*>(ws + c.mpk);
  auto* gobs = gsyn + ns;
  auto* norms = reinterpret_cast<double*>(ws + c.mnorm);
  auto* fac = reinterpret_cast<l2::TraceFactors<T>*>(ws + c.mfac);
  ADFWI_CUDA_TRY(cudaMemsetAsync(ws + c.mpk, 0, 2 * (size_t)ns * 8, st));  // peaks start at +0
  const dim3 grid = l2::grid(ns, nr);
  const T* sy = static_cast<const T*>(syn);
  const T* ob = static_cast<const T*>(obs);
  ADFWI_LAUNCH(kAux, st, (l2::peaks<T><<<grid, l2::block(), 0, st>>>(ns, nt, nr, sy, ob, stats, gsyn, gobs)));
  ADFWI_LAUNCH(kAux, st, (l2::factors<T><<<grid, l2::block(), 0, st>>>(ns, nt, nr, p->d.dt, silent_rel, flags & 1, sy,
                                                                         ob, stats, gsyn, gobs, fac, norms)));
  for (int m = 0; m < p->nm; ++m) {
    const int s0 = p->model_shot_beg[m], s1 = p->model_shot_beg[m + 1];
    ADFWI_LAUNCH(kAux, st, (l2::sum_norms<<<1, l2::kThreads, 0, st>>>((int64_t)(s1 - s0) * nr,
                                                                       norms + (int64_t)s0 * nr, loss + m)));
  }
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// The misfit's adjoint source of every record sample into adj (ns, nt, nr), times *gmul, from
// the factors l2_loss_impl left in the workspace.
template <typename T>
int l2_sources_impl(const adfwi_acoustic_plan* p, const void* syn, const void* obs, int flags, const double* gmul,
                    void* adj, unsigned char* ws, int64_t ws_bytes, cudaStream_t st) {
  const Carve c = carve(p, true, p->K);
  if (ws_bytes < c.total) {
    set_error("workspace too small: %lld bytes given, %lld needed", (long long)ws_bytes, (long long)c.total);
    return kWorkspaceTooSmall;
  }
  const int ns = p->d.ns, nt = p->d.nt, nr = p->d.nr;
  const auto* fac = reinterpret_cast<const l2::TraceFactors<T>*>(ws + c.mfac);
  ADFWI_LAUNCH(kAux, st, (l2::sources<T><<<l2::grid(ns, nr), l2::block(), 0, st>>>(
                             ns, nt, nr, flags & 1, static_cast<const T*>(syn), static_cast<const T*>(obs), fac, gmul,
                             static_cast<T*>(adj))));
  ADFWI_CUDA_TRY(cudaGetLastError());
  return kOk;
}

// Resident blocks of a persistent step kernel on the current device (`fallback` per SM x 152
// without a GPU).
template <typename K>
int resident_blocks(K kernel, int threads, int smem, int fallback) {
  int dev = 0, sms = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 152 * fallback;
  }
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem) != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return 152 * fallback;
  }
  return sms * occ;
}

template <typename T>
int resident_adj_blocks(bool deep) {
  return resident_blocks(adj_kernel<T>(deep), ac2::VTHREADS, ac2::VecAdjLayout<T>::bytes(vec_adj_stages<T>(deep)),
                         sizeof(T) == 8 ? 1 : (deep ? ac2::VDEEP : ac2::VAMINB));
}
template <typename T>
int resident_fwd_blocks(bool deep) {
  return resident_blocks(fwd_kernel<T>(deep), ac2::VTHREADS, ac2::VecFwdLayout<T>::bytes(vec_stages<T>(deep)),
                         sizeof(T) == 8 ? 1 : (deep ? ac2::VDEEP : ac2::VMINB));
}

// Padded grids at least this wide run the deep-ring variants (one more stage, 2 blocks per SM).
// An empirical rule from per-launch times of both rings (FP32, full history; forward / adjoint
// in us, shallow -> deep): 600 x 1600 padded with 4 / 8 / 16 shots 44.1 -> 41.6 / 77.2 -> 69.1,
// 86.0 -> 73.5 / 130.8 -> 118.0, 161.8 -> 165.8 / 227.6 -> 217.1; every narrower grid measured
// (300 x 700 with 10 / 30 / 60 shots, 400 x 1000 with 8 / 16 / 30, 200 x 400 with 16 / 64,
// up to 144 MB of fields per time level) ran 4-42 % slower with the deep ring. The wide grid's
// kernels read 27 B per cell-update from DRAM against 13.5 B on the 300 x 700 grid (L2 hit
// rate 19 % against 30 %), so they wait longer per stage and profit from the extra stage.
constexpr int kDeepRingCols = 1400;

// Shots per unit for the persistent TMA kernels: balance the units over the resident blocks
// (the block with the most units sets the time) against the per-unit costs (the coefficient
// loads, and the load and flush of the partial accumulator planes), weighted as 1.5 items: the
// weight that reproduces the measured optimum of a sweep of 1, 2, 4 and 8 shots per unit on the
// 600 x 1600 grid with 8 and 32 shots.
int pick_unit_shots(const std::vector<int>& model_shot_beg, int ntiles, int blocks_fwd, int blocks_adj) {
  const int nm = (int)model_shot_beg.size() - 1;
  int maxns = 1;
  for (int m = 0; m < nm; ++m) maxns = std::max(maxns, model_shot_beg[m + 1] - model_shot_beg[m]);
  int best = 1;
  double best_cost = 1e30;
  for (int G = 1; G <= maxns; ++G) {
    int groups = 0;
    for (int m = 0; m < nm; ++m) groups += (model_shot_beg[m + 1] - model_shot_beg[m] + G - 1) / G;
    const long long units = (long long)ntiles * groups;
    const long long pf = (units + blocks_fwd - 1) / blocks_fwd;
    const long long pa = (units + blocks_adj - 1) / blocks_adj;
    const double cost = (double)(pf + 2 * pa) * (G + 1.5);  // the adjoint step takes about twice as long
    if (cost < best_cost - 1e-9) {
      best_cost = cost;
      best = G;
    }
  }
  return best;
}

// Tile the grid and build the receiver tables of that tiling (appended to p->tab).
void build_tiling(adfwi_acoustic_plan* p, Tiling* tl, int tz, int tx, const std::vector<int>& Gm, const int32_t* rcv_z,
                  const int32_t* rcv_x) {
  const adfwi_acoustic_desc& d = p->d;
  std::vector<int32_t>& t = p->tab;
  tl->tz = tz;
  tl->tx = tx;
  tl->tiles_x = (p->nxp + tx - 1) / tx;
  tl->tiles_z = (p->nzp - p->zbeg + tz - 1) / tz;
  tl->ntiles = tl->tiles_x * tl->tiles_z;
  tl->G = 1;
  tl->blocks = 0;
  // shot groups of at most Gm[m] shots of model m, never across two models
  std::vector<int32_t> gb(1, 0), gm;
  p->model_grp_beg.assign(1, 0);
  for (int m = 0; m < p->nm; ++m) {
    const int G = std::max(1, Gm[m]);
    tl->G = std::max(tl->G, G);
    for (int s = p->model_shot_beg[m]; s < p->model_shot_beg[m + 1]; s += G) {
      gb.push_back(std::min(s + G, p->model_shot_beg[m + 1]));
      gm.push_back(m);
    }
    p->model_grp_beg.push_back((int)gm.size());
  }
  tl->ngroups = (int)gm.size();
  tl->o_gb = t.size();
  t.insert(t.end(), gb.begin(), gb.end());
  tl->o_gm = t.size();
  t.insert(t.end(), gm.begin(), gm.end());
  struct R {
    int tile, cell, id;
  };
  std::vector<R> rs(d.nr);
  for (int r = 0; r < d.nr; ++r) {
    int z = rcv_z[r] + d.nabc - p->zbeg, x = rcv_x[r] + d.nabc;
    rs[r].tile = (z / tz) * tl->tiles_x + x / tx;
    rs[r].cell = ((z % tz) << 16) | (x % tx);
    rs[r].id = r;
  }
  std::stable_sort(rs.begin(), rs.end(), [](const R& a, const R& b) {
    return a.tile != b.tile ? a.tile < b.tile : a.cell < b.cell;
  });
  tl->o_trb = t.size();
  {
    std::vector<int32_t> beg(tl->ntiles + 1, 0);
    for (const R& r : rs) beg[r.tile + 1]++;
    for (int q = 0; q < tl->ntiles; ++q) beg[q + 1] += beg[q];
    t.insert(t.end(), beg.begin(), beg.end());
  }
  tl->o_trc = t.size();
  for (const R& r : rs) t.push_back(r.cell);
  tl->o_tri = t.size();
  for (const R& r : rs) t.push_back(r.id);
  std::vector<int32_t> tcb(tl->ntiles + 1, 0), tcc, tcr, cr;
  for (size_t q = 0; q < rs.size(); ++q) {
    bool fresh = q == 0 || rs[q].tile != rs[q - 1].tile || rs[q].cell != rs[q - 1].cell;
    if (fresh) {
      tcb[rs[q].tile + 1]++;
      tcc.push_back(rs[q].cell);
      tcr.push_back((int32_t)cr.size());
    }
    cr.push_back(rs[q].id);
  }
  tcr.push_back((int32_t)cr.size());
  for (int q = 0; q < tl->ntiles; ++q) tcb[q + 1] += tcb[q];
  tl->ncells = (int)tcc.size();
  tl->o_tcb = t.size();
  t.insert(t.end(), tcb.begin(), tcb.end());
  tl->o_tcc = t.size();
  t.insert(t.end(), tcc.begin(), tcc.end());
  tl->o_tcr = t.size();
  t.insert(t.end(), tcr.begin(), tcr.end());
  tl->o_cr = t.size();
  t.insert(t.end(), cr.begin(), cr.end());
}

// ----------------------------------------------------------------------------------------
// Forward solve for callers that cannot allocate device memory.
//
// Its scratch (staged coefficients, wavefield ping-pong buffers, illumination partials and
// geometry tables) lives in one file-scope __device__ array of kStaticScratchBytes, which
// every GPU that loads this library reserves until the process exits. Host code never
// passes the symbol itself to a kernel (on the host it only names a stand-in object):
// the device address is looked up once per device with cudaGetSymbolAddress, on that
// device, by the first call made there.
// ----------------------------------------------------------------------------------------
constexpr int64_t kStaticScratchBytes = int64_t(64) << 20;  // 64 MiB
__device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
std::mutex g_static_mu;
std::vector<void*> g_static_addr;  // device address of g_static_scratch, per device ordinal

int static_scratch_address(void** out) {
  int dev = 0;
  ADFWI_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_static_mu);
  if ((int)g_static_addr.size() <= dev) g_static_addr.resize(dev + 1, nullptr);
  if (g_static_addr[dev] == nullptr) {
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_static_scratch);
    if (e != cudaSuccess || addr == nullptr) {
      set_error("cudaGetSymbolAddress(static scratch) failed on device %d: %s", dev, cudaGetErrorString(e));
      return kCudaError;
    }
    g_static_addr[dev] = addr;
  }
  *out = g_static_addr[dev];
  return kOk;
}

}  // namespace

extern "C" {

int adfwi_acoustic_forward_noalloc(const adfwi_acoustic_plan* p, const void* alpha1, const void* alpha2,
                                   const void* damp, const void* wavelet, void* rec_p, void* rec_u, void* rec_w,
                                   void* fw_p, void* fw_u, void* fw_w, void* stream) {
  ADFWI_CHECK_ARG(p && alpha1 && alpha2 && damp && wavelet, "null argument");
  ADFWI_CHECK_ARG((rec_p && rec_u && rec_w) || (!rec_p && !rec_u && !rec_w), "records: give all three or none");
  ADFWI_CHECK_ARG(p->d.nr > 0 || rec_p == nullptr, "records requested without receivers");
  const int64_t need = carve(p, false, 1).total;
  if (need > kStaticScratchBytes) {
    set_error("adfwi_acoustic_forward_noalloc: this solve needs %lld bytes of scratch but the static scratch "
              "array holds %lld bytes (64 MiB); use adfwi_acoustic_forward with a caller-provided workspace",
              (long long)need, (long long)kStaticScratchBytes);
    return kWorkspaceTooSmall;
  }
  void* ws = nullptr;
  int rc = static_scratch_address(&ws);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  // forward_impl clears every scratch region it accumulates into (coefficient ghosts, field
  // buffers, illumination partials) before the first step, so a previous call's leftovers
  // in the shared array do not leak into this one.
  if (p->d.dtype == ADFWI_F64)
    return forward_impl<double>(p, alpha1, alpha2, damp, wavelet, rec_p, rec_u, rec_w, fw_p, fw_u, fw_w, false, w,
                                kStaticScratchBytes, st);
  return forward_impl<float>(p, alpha1, alpha2, damp, wavelet, rec_p, rec_u, rec_w, fw_p, fw_u, fw_w, false, w,
                             kStaticScratchBytes, st);
}

int adfwi_acoustic_noalloc_status(const adfwi_acoustic_plan* p, int32_t* status, void* stream) {
  ADFWI_CHECK_ARG(p && status, "null argument");
  const Carve c = carve(p, false, 1);
  ADFWI_CHECK_ARG(c.total <= kStaticScratchBytes, "this plan's forward does not fit the static scratch array");
  void* ws = nullptr;
  int rc = static_scratch_address(&ws);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int32_t v = 0;
  ADFWI_CUDA_TRY(cudaMemcpyAsync(&v, static_cast<const unsigned char*>(ws) + c.flag, sizeof(v),
                                 cudaMemcpyDeviceToHost, st));
  ADFWI_CUDA_TRY(cudaStreamSynchronize(st));
  *status = v;
  return kOk;
}

}  // extern "C"

namespace {

int plan_create_impl(const adfwi_acoustic_desc* desc, const int32_t* src_z, const int32_t* src_x,
                     const int32_t* rcv_z, const int32_t* rcv_x, int32_t nmodels, const int32_t* shot_model,
                     adfwi_acoustic_plan** out) {
  ADFWI_CHECK_ARG(desc && out, "null descriptor or output pointer");
  *out = nullptr;
  const adfwi_acoustic_desc& d = *desc;
  ADFWI_CHECK_ARG(nmodels >= 1, "need nmodels >= 1");
  ADFWI_CHECK_ARG(d.ns >= 1, "need ns >= 1");
  std::vector<int> model_shot_beg(nmodels + 1, 0);
  if (shot_model != nullptr) {
    // shots of one model are consecutive, models in order, every model has a shot
    for (int s = 0; s < d.ns; ++s) {
      ADFWI_CHECK_ARG(shot_model[s] >= 0 && shot_model[s] < nmodels && (s == 0 || shot_model[s] >= shot_model[s - 1]),
                      "shot_model must be non-decreasing in [0, nmodels) (shot %d)", s);
      model_shot_beg[shot_model[s] + 1]++;
    }
    for (int m = 0; m < nmodels; ++m) {
      ADFWI_CHECK_ARG(model_shot_beg[m + 1] > 0, "model %d has no shot", m);
      model_shot_beg[m + 1] += model_shot_beg[m];
    }
  } else {
    ADFWI_CHECK_ARG(nmodels == 1, "shot_model is required for several models");
    model_shot_beg[1] = d.ns;
  }
  ADFWI_CHECK_ARG(d.nz >= 1 && d.nx >= 1 && d.nabc >= 2, "need nz, nx >= 1 and nabc >= 2");
  ADFWI_CHECK_ARG(d.ns >= 1 && d.nt >= 1 && d.nr >= 0, "need ns >= 1, nt >= 1, nr >= 0");
  ADFWI_CHECK_ARG(d.dtype == ADFWI_F32 || d.dtype == ADFWI_F64, "dtype must be ADFWI_F32 or ADFWI_F64");
  ADFWI_CHECK_ARG(d.snapshot_precision >= 0 && d.snapshot_precision <= 3, "bad snapshot_precision");
  ADFWI_CHECK_ARG(d.checkpoint_segments >= 1, "checkpoint_segments must be >= 1");
  ADFWI_CHECK_ARG(d.ring_depth >= 0 && d.ring_depth <= 2, "ring_depth must be 0, 1 or 2");
  ADFWI_CHECK_ARG(d.snapshot_every >= ADFWI_SNAP_EVERY_BOUNDARY,
                  "snapshot_every must be >= 0, or ADFWI_SNAP_EVERY_BOUNDARY for boundary saving");
  ADFWI_CHECK_ARG(d.snapshot_every != ADFWI_SNAP_EVERY_BOUNDARY || nmodels == 1,
                  "boundary saving takes a single-model plan");
  ADFWI_CHECK_ARG(src_z && src_x && (d.nr == 0 || (rcv_z && rcv_x)), "null geometry array");
  adfwi_acoustic_plan* p = new (std::nothrow) adfwi_acoustic_plan();
  if (!p) {
    set_error("host allocation failed");
    return kBadArgument;
  }
  p->d = d;
  p->nm = nmodels;
  p->model_shot_beg = model_shot_beg;
  p->nzp = d.nz + 2 * d.nabc;
  p->nxp = d.nx + 2 * d.nabc;
  p->fs = d.free_surface ? d.nabc : 1;
  p->zbeg = d.free_surface ? p->fs - 1 : 0;
  p->elem = d.dtype == ADFWI_F64 ? 8 : 4;
  p->L = make_layout(p->nzp, p->nxp, ac2::TZ, ac2::TX, p->elem);
  p->bsave = d.snapshot_every == ADFWI_SNAP_EVERY_BOUNDARY;
  if (p->bsave) {
    // The interior whose update inverts exactly: the model window, inside every update region,
    // away from the free-surface rows, and one cell short of the frame on the right and at the
    // bottom (the u / w damping averages a cell with its right / lower neighbour). Everything
    // else is the frame that the forward keeps step by step.
    const int i_lo = std::max(d.nabc, p->fs + 1), i_hi = std::min(d.nabc + d.nz - 2, p->nzp - 4);
    const int j_lo = std::max(d.nabc, 2), j_hi = std::min(d.nabc + d.nx - 2, p->nxp - 4);
    p->bbox = ac::BsBox{i_lo, i_hi, j_lo, j_hi};
    std::vector<int32_t>& tb = p->tab;
    p->o_fidx = tb.size();
    tb.resize(tb.size() + (size_t)p->nzp * p->nxp, -1);
    std::vector<int32_t> off;
    for (int i = 0; i < p->nzp; ++i)
      for (int j = 0; j < p->nxp; ++j)
        if (!(i >= i_lo && i <= i_hi && j >= j_lo && j <= j_hi)) {
          tb[p->o_fidx + (size_t)i * p->nxp + j] = (int32_t)off.size();
          off.push_back((int32_t)p->L.off(i, j));
        }
    p->nframe = (int)off.size();
    p->o_foff = tb.size();
    tb.insert(tb.end(), off.begin(), off.end());
  }
  // torch.chunk(wavelet, checkpoint_segments): chunks of ceil(nt / segments) steps.
  const int chunk = (d.nt + d.checkpoint_segments - 1) / d.checkpoint_segments;
  const int nchunks = (d.nt + chunk - 1) / chunk;
  p->last_chunk_start = (nchunks - 1) * chunk;

  // Geometry tables.
  std::vector<int32_t>& t = p->tab;
  p->o_srcz = t.size();
  for (int s = 0; s < d.ns; ++s) {
    int z = src_z[s] + d.nabc, x = src_x[s] + d.nabc;
    if (z < p->zbeg || z >= p->nzp || x < 0 || x >= p->nxp) {
      set_error("source %d at (z=%d, x=%d) lies outside the model", s, src_z[s], src_x[s]);
      delete p;
      return kBadGeometry;
    }
    t.push_back(z);
  }
  p->o_srcx = t.size();
  for (int s = 0; s < d.ns; ++s) t.push_back(src_x[s] + d.nabc);
  for (int r = 0; r < d.nr; ++r) {
    int z = rcv_z[r] + d.nabc, x = rcv_x[r] + d.nabc;
    // u has nxp-1 columns and w has nzp-1 rows (acoustic_kernels.py:241-242, 167-169)
    if (z < p->zbeg || z > p->nzp - 2 || x < 0 || x > p->nxp - 2) {
      set_error("receiver %d at (z=%d, x=%d) lies outside the recordable model", r, rcv_z[r], rcv_x[r]);
      delete p;
      return kBadGeometry;
    }
  }
  // 16 x 64 tiles: units of G shots spread over the resident blocks of the pipelined steps.
  {
    const int ntiles = ((p->nxp + ac2::TX - 1) / ac2::TX) * ((p->nzp - p->zbeg + ac2::TZ - 1) / ac2::TZ);
    // shots per group from the shallow variants' widths whatever the ring, so that the ring
    // changes launch widths and stages only, never the results
    const int blocks = p->elem == 8 ? resident_adj_blocks<double>(false) : resident_adj_blocks<float>(false);
    const int fblocks = p->elem == 8 ? resident_fwd_blocks<double>(false) : resident_fwd_blocks<float>(false);
    p->deep = p->elem == 4 && (d.ring_depth == 2 || (d.ring_depth == 0 && p->nxp >= kDeepRingCols));
    const int run_blocks = p->deep ? resident_adj_blocks<float>(true) : blocks;
    const int run_fblocks = p->deep ? resident_fwd_blocks<float>(true) : fblocks;
    // shots per group of each model: as a plan of that model alone would choose them, so a
    // model's partial sums (and so its results) do not depend on the other models of a batch
    std::vector<int> Gm(p->nm);
    for (int m = 0; m < p->nm; ++m) {
      const std::vector<int> alone = {0, p->model_shot_beg[m + 1] - p->model_shot_beg[m]};
      Gm[m] = d.shots_per_block > 0 ? d.shots_per_block : pick_unit_shots(alone, ntiles, fblocks, blocks);
    }
    build_tiling(p, &p->t2, ac2::TZ, ac2::TX, Gm, rcv_z, rcv_x);
    p->t2.blocks = std::max(1, std::min(run_blocks, p->t2.ntiles * p->t2.ngroups));
    p->t2.fwd_blocks = std::max(1, std::min(run_fblocks, p->t2.ntiles * p->t2.ngroups));
  }
  if (t.empty()) t.push_back(0);

  if (!p->tab_pin.assign(p->tab.data(), p->tab.size() * 4)) {
    delete p;
    return kCudaError;
  }
  p->K = choose_K(p);
  p->nseg = (d.nt + p->K - 1) / p->K;
  *out = p;
  return kOk;
}

}  // namespace

extern "C" {

int adfwi_acoustic_plan_create(const adfwi_acoustic_desc* desc, const int32_t* src_z, const int32_t* src_x,
                               const int32_t* rcv_z, const int32_t* rcv_x, adfwi_acoustic_plan** out) {
  return plan_create_impl(desc, src_z, src_x, rcv_z, rcv_x, 1, nullptr, out);
}

int adfwi_acoustic_plan_create_batched(const adfwi_acoustic_desc* desc, const int32_t* src_z,
                                       const int32_t* src_x, const int32_t* rcv_z, const int32_t* rcv_x,
                                       int32_t nmodels, const int32_t* shot_model, adfwi_acoustic_plan** out) {
  if (shot_model == nullptr) {
    set_error("adfwi_acoustic_plan_create_batched: null shot_model");
    return kBadArgument;
  }
  return plan_create_impl(desc, src_z, src_x, rcv_z, rcv_x, nmodels, shot_model, out);
}

int32_t adfwi_acoustic_plan_models(const adfwi_acoustic_plan* plan) { return plan ? plan->nm : 0; }

void adfwi_acoustic_plan_destroy(adfwi_acoustic_plan* plan) { delete plan; }

int adfwi_acoustic_status(const adfwi_acoustic_plan* p, const void* workspace, int64_t workspace_bytes,
                          int32_t with_gradient, int32_t* status, void* stream) {
  ADFWI_CHECK_ARG(p && workspace && status, "null argument");
  Carve c = carve(p, with_gradient != 0, with_gradient ? p->K : 1);
  ADFWI_CHECK_ARG(workspace_bytes >= c.total, "workspace smaller than the plan's layout");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int32_t v = 0;
  ADFWI_CUDA_TRY(cudaMemcpyAsync(&v, static_cast<const unsigned char*>(workspace) + c.flag, sizeof(v),
                                 cudaMemcpyDeviceToHost, st));
  ADFWI_CUDA_TRY(cudaStreamSynchronize(st));
  *status = v;
  return kOk;
}

int adfwi_acoustic_workspace_bytes(const adfwi_acoustic_plan* p, int32_t with_gradient, int64_t* bytes) {
  ADFWI_CHECK_ARG(p && bytes, "null plan or output pointer");
  *bytes = carve(p, with_gradient != 0, with_gradient ? p->K : 1).total;
  return kOk;
}

int adfwi_acoustic_snapshot_every(const adfwi_acoustic_plan* p, int32_t* steps) {
  ADFWI_CHECK_ARG(p && steps, "null plan or output pointer");
  *steps = p->bsave ? ADFWI_SNAP_EVERY_BOUNDARY : p->K;
  return kOk;
}

int adfwi_acoustic_forward(const adfwi_acoustic_plan* p, const void* alpha1, const void* alpha2, const void* damp,
                           const void* wavelet, void* rec_p, void* rec_u, void* rec_w, void* fw_p, void* fw_u,
                           void* fw_w, int32_t with_gradient, void* workspace, int64_t workspace_bytes,
                           void* stream) {
  ADFWI_CHECK_ARG(p && alpha1 && alpha2 && damp && wavelet && workspace, "null argument");
  ADFWI_CHECK_ARG((rec_p && rec_u && rec_w) || (!rec_p && !rec_u && !rec_w), "records: give all three or none");
  ADFWI_CHECK_ARG(p->d.nr > 0 || rec_p == nullptr, "records requested without receivers");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (p->d.dtype == ADFWI_F64)
    return forward_impl<double>(p, alpha1, alpha2, damp, wavelet, rec_p, rec_u, rec_w, fw_p, fw_u, fw_w,
                                with_gradient != 0, ws, workspace_bytes, st);
  return forward_impl<float>(p, alpha1, alpha2, damp, wavelet, rec_p, rec_u, rec_w, fw_p, fw_u, fw_w,
                             with_gradient != 0, ws, workspace_bytes, st);
}

int adfwi_acoustic_backward(const adfwi_acoustic_plan* p, const void* alpha1, const void* alpha2, const void* damp,
                            const void* wavelet, const void* grad_rec_p, const void* grad_rec_u,
                            const void* grad_rec_w, void* grad_alpha1, void* grad_alpha2, void* workspace,
                            int64_t workspace_bytes, void* stream) {
  ADFWI_CHECK_ARG(p && alpha1 && alpha2 && damp && wavelet && workspace && grad_alpha1 && grad_alpha2,
                  "null argument");
  (void)alpha1;
  (void)alpha2;
  (void)damp;  // the coefficient planes staged by the forward call are reused from the workspace
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (p->d.dtype == ADFWI_F64)
    return backward_impl<double>(p, wavelet, grad_rec_p, grad_rec_u, grad_rec_w, grad_alpha1, grad_alpha2, ws,
                                 workspace_bytes, st);
  return backward_impl<float>(p, wavelet, grad_rec_p, grad_rec_u, grad_rec_w, grad_alpha1, grad_alpha2, ws,
                              workspace_bytes, st);
}

int adfwi_acoustic_l2_loss(const adfwi_acoustic_plan* p, const void* syn, const void* obs, double silent_rel,
                           int32_t flags, double* loss, void* workspace, int64_t workspace_bytes, void* stream) {
  ADFWI_CHECK_ARG(p && syn && obs && loss && workspace, "null argument");
  ADFWI_CHECK_ARG(p->d.nr > 0, "the plan has no receivers");
  ADFWI_CHECK_ARG(silent_rel >= 0.0, "silent_rel must be non-negative");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (p->d.dtype == ADFWI_F64)
    return l2_loss_impl<double>(p, syn, obs, silent_rel, flags, loss, ws, workspace_bytes, st);
  return l2_loss_impl<float>(p, syn, obs, silent_rel, flags, loss, ws, workspace_bytes, st);
}

int adfwi_acoustic_l2_sources(const adfwi_acoustic_plan* p, const void* syn, const void* obs, int32_t flags,
                              const double* grad_scale, void* adj, void* workspace, int64_t workspace_bytes,
                              void* stream) {
  ADFWI_CHECK_ARG(p && syn && obs && grad_scale && adj && workspace, "null argument");
  ADFWI_CHECK_ARG(p->d.nr > 0, "the plan has no receivers");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (p->d.dtype == ADFWI_F64)
    return l2_sources_impl<double>(p, syn, obs, flags, grad_scale, adj, ws, workspace_bytes, st);
  return l2_sources_impl<float>(p, syn, obs, flags, grad_scale, adj, ws, workspace_bytes, st);
}

int adfwi_acoustic_backward_l2(const adfwi_acoustic_plan* p, const void* wavelet, const void* syn, const void* obs,
                               int32_t flags, const double* grad_scale, void* grad_alpha1, void* grad_alpha2,
                               void* workspace, int64_t workspace_bytes, void* stream) {
  ADFWI_CHECK_ARG(p && wavelet && syn && obs && grad_scale && grad_alpha1 && grad_alpha2 && workspace,
                  "null argument");
  ADFWI_CHECK_ARG(p->d.nr > 0, "the plan has no receivers");
  const FusedL2 fz{obs, grad_scale, flags & 1};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  if (p->d.dtype == ADFWI_F64)
    return backward_impl<double>(p, wavelet, syn, nullptr, nullptr, grad_alpha1, grad_alpha2, ws, workspace_bytes, st,
                                 &fz);
  return backward_impl<float>(p, wavelet, syn, nullptr, nullptr, grad_alpha1, grad_alpha2, ws, workspace_bytes, st,
                              &fz);
}

}  // extern "C"
