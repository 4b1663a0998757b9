// TMA-pipelined acoustic forward and adjoint steps (included by acoustic.cu).
//
// Work of one launch = all (tile, shot) items of one time step. A persistent block owns a
// contiguous range of "units" (one 16 x 64 tile x one group of G shots; tile-major), so every
// accumulator a unit produces (illumination, coefficient gradients) belongs to one block and
// is flushed once, deterministically, into the group's partial plane.
//
// Inside a block, warp 16 is the producer: one lane issues, per item, the TMA tile loads of
// every wavefield plane the item reads into the next free pipeline stage and arms the stage's
// `full` mbarrier with the byte count (the per-item source cell and amplitude travel in a
// small header written before the arming arrive). Warps 0-15 are the consumers: they wait
// on `full`, compute, and arrive on the stage's `empty` mbarrier once they no longer read it,
// so the loads of the next items overlap the arithmetic of the current one.
//
// Coefficients are staged once per tile, not per item: the tile-cell coefficients of a
// consumer thread stay in its registers (it owns the same cells for every shot of the tile)
// and the halo coefficients go to a small per-tile shared-memory area. The masked planes
// (zero alpha and unit decay outside each update region) remove every region test from the
// hot loop.
//
// Every wait is bounded (kWaitLimit polls); a wait that runs out raises the device error
// flag and a block-wide abort flag, after which the block skips its remaining work
// (consumers still meet every named barrier, so no thread waits on one that never fills).
#pragma once
#include "tma.cuh"

namespace adfwi {
namespace ac2 {

constexpr int TX = 64;             // tile columns
constexpr int TZ = 16;             // tile rows
constexpr int BOXX = TX + 8;       // TMA box width: columns j0-4 .. j0+TX+3 (16-byte aligned start)
constexpr int EZ = TZ + 3;         // rows i0-1 .. i0+TZ+1
constexpr int WZ = TZ + 6;         // rows i0-3 .. i0+TZ+2
constexpr int EXC = TX + 3;        // p-halo columns j0-1 .. j0+TX+1
constexpr int NEXT = EZ * EXC;     // p-halo cells (1273)
constexpr int SPX = TX + 4;        // p-halo row length in shared memory
constexpr int NCW = 16;            // consumer warps
constexpr int NCONS = NCW * 32;    // consumer threads
constexpr int NTHREADS = NCONS + 32;
constexpr int CPL = TX / 32;       // tile columns per lane (one tile row per consumer warp)
constexpr int KEXT = (NEXT + NCONS - 1) / NCONS;  // p-halo cells per consumer thread
constexpr int MAXSTAGES = 8;
static_assert(TZ == NCW, "one tile row per consumer warp");

__host__ __device__ constexpr int round128(int bytes) { return (bytes + 127) / 128 * 128; }

template <typename T>
struct ItemHeader {
  int sz, sx;
  T sval;
};

struct SmemHeader {
  uint64_t full[MAXSTAGES];
  uint64_t empty[MAXSTAGES];
  int abort_flag;
};

__device__ __forceinline__ unsigned char* aligned_smem(unsigned char* raw) {
  return raw + ((1024u - (smem_u32(raw) & 1023u)) & 1023u);
}
__device__ __forceinline__ bool aborted(const SmemHeader* h) { return *(volatile const int*)&h->abort_flag != 0; }
__device__ __forceinline__ void set_abort(SmemHeader* h, int* flag) {
  raise_flag(flag, kErrWaitTimeout);
  *(volatile int*)&h->abort_flag = 1;
}

struct Maps {
  CUtensorMap a, b, c, d, e;  // forward: u, w, p;  adjoint: lu, lw, lp, ph, dh
};

template <typename T>
struct StepArgs {
  int it, G, ngroups, ntiles, accum_u, stages;
  const T* wav;
  const T* cf;  // coefficient block (masked planes kA1M .. kB3)
  T* o0;        // forward: p1 / adjoint: lp1
  T* o1;        // forward: u1 / adjoint: lu1
  T* o2;        // forward: w1 / adjoint: lw1
  T* d1;        // forward: divergence history (may be null)
  const T* rec_p;  // forward: record outputs (cast away) / adjoint: grad_rec inputs
  const T* rec_u;
  const T* rec_w;
  T* acc0;      // forward: illumination P partials / adjoint: dL/d alpha1 partials
  T* acc1;      // forward: illumination U partials / adjoint: dL/d alpha2 partials
  int* flag;
};

// Producer loop shared by both kernels: per item, arm the stage and load NBOX boxes.
// ymap[b] = {map index, first row relative to i0, byte offset in the stage}
template <typename T, int NBOX>
__device__ __forceinline__ void produce(const Maps& maps, const ac::Geo<T>& g, const StepArgs<T>& a, SmemHeader* h,
                                        ItemHeader<T>* ih, unsigned char* stage0, int stage_bytes, int stage_tx,
                                        const int (&ymap)[NBOX][3], int u_beg, int u_end, bool want_src) {
  const CUtensorMap* mp[5] = {&maps.a, &maps.b, &maps.c, &maps.d, &maps.e};
#pragma unroll
  for (int q = 0; q < NBOX; ++q) prefetch_tensormap(mp[ymap[q][0]]);
  const int S = a.stages;
  int k = 0;
  for (int un = u_beg; un < u_end && !aborted(h); ++un) {
    const int tile = un / a.ngroups, grp = un - tile * a.ngroups;
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    const int x = j0 - 4 + GX;
    const int s_beg = grp * a.G, s_end = min(g.ns, s_beg + a.G);
    bool stop = false;
    for (int sh = s_beg; sh < s_end; ++sh, ++k) {
      const int st = k % S;
      if (k >= S && !mbar_wait(&h->empty[st], ((k / S) - 1) & 1)) {
        set_abort(h, a.flag);
        stop = true;
        break;
      }
      if (want_src) {
        ih[st].sz = g.src_z[sh];
        ih[st].sx = g.src_x[sh];
        ih[st].sval = ac::rmul(g.dt, a.wav[(int64_t)sh * g.nt + a.it]);
      }
      unsigned char* sb = stage0 + st * stage_bytes;
      mbar_arrive_expect_tx(&h->full[st], stage_tx);  // also releases the header writes above
#pragma unroll
      for (int q = 0; q < NBOX; ++q)
        tma_load_3d(sb + ymap[q][2], mp[ymap[q][0]], x, i0 + ymap[q][1] + GZ, sh, &h->full[st]);
    }
    if (stop) break;
  }
  // do not leave the block while a load it issued may still be landing
  for (int q = max(0, k - S); q < k; ++q) mbar_wait(&h->full[q % S], (q / S) & 1);
}

// ---------------------------------------------------------------------------- forward
template <typename T>
struct FwdLayout {
  static constexpr int kE = round128(EZ * BOXX * (int)sizeof(T));
  static constexpr int kW = round128(WZ * BOXX * (int)sizeof(T));
  static constexpr int kStage = 2 * kE + kW;  // U, W, P
  static constexpr int kStageTx = (2 * EZ + WZ) * BOXX * (int)sizeof(T);
  static constexpr int kSP = round128(EZ * SPX * (int)sizeof(T));
  static constexpr int kSO = round128(TZ * TX * (int)sizeof(T));
  static constexpr int kCoef = round128(2 * NEXT * (int)sizeof(T));  // alpha1, 1 - kappa1 on the p halo
  static int bytes(int stages) { return 2048 + stages * kStage + kSP + 2 * kSO + kCoef; }
};

// divergence at p-halo cell (r, c) from the staged u (19-row box) and w (22-row box), in the
// reference's operation order (acoustic_kernels.py:118-127)
template <typename T>
__device__ __forceinline__ T fwd_div(const ac::Geo<T>& g, const T* U, const T* W, int r, int c) {
  const int cc = c + 3;
  const T* ur = U + r * BOXX + cc;
  T t1 = ac::rsub(ac::radd(ac::rsub(ur[0], ur[-1]), W[(r + 2) * BOXX + cc]), W[(r + 1) * BOXX + cc]);
  T t2 = ac::rsub(ac::radd(ac::rsub(ur[1], ur[-2]), W[(r + 3) * BOXX + cc]), W[r * BOXX + cc]);
  return ac::radd(ac::rmul(g.c1, t1), ac::rmul(g.c2, t2));
}

template <typename T>
__global__ void __launch_bounds__(NTHREADS, sizeof(T) == 4 ? 2 : 1)
    fwd_step_tma(const __grid_constant__ Maps maps, ac::Geo<T> g, StepArgs<T> a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = aligned_smem(smem_raw);
  using LY = FwdLayout<T>;
  const int S = a.stages;
  SmemHeader* h = reinterpret_cast<SmemHeader*>(smem);
  ItemHeader<T>* ih = reinterpret_cast<ItemHeader<T>*>(smem + 512);
  unsigned char* stage0 = smem + 1024;
  T* SP = reinterpret_cast<T*>(stage0 + S * LY::kStage);
  T* SOU = reinterpret_cast<T*>(stage0 + S * LY::kStage + LY::kSP);
  T* SOW = reinterpret_cast<T*>(stage0 + S * LY::kStage + LY::kSP + LY::kSO);
  T* CA1 = reinterpret_cast<T*>(stage0 + S * LY::kStage + LY::kSP + 2 * LY::kSO);  // alpha1 (p halo)
  T* CB1 = CA1 + NEXT;                                                              // 1 - kappa1 (p halo)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], NCONS);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  const int nunits = a.ntiles * a.ngroups;
  const int per = (nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(nunits, u_beg + per);

  if (warp == NCW) {
    if (lane == 0) {
      const int ymap[3][3] = {{0, -1, 0}, {1, -3, LY::kE}, {2, -1, LY::kE + LY::kW}};
      produce<T, 3>(maps, g, a, h, ih, stage0, LY::kStage, LY::kStageTx, ymap, u_beg, u_end, true);
    }
    return;
  }

  const Layout L = g.L;
  const int64_t PL = L.plane;
  const T* cf = a.cf;
  T* rec_p = const_cast<T*>(a.rec_p);
  T* rec_u = const_cast<T*>(a.rec_u);
  T* rec_w = const_cast<T*>(a.rec_w);
  // per-thread cells: p-halo cells e = tid + NCONS*q; tile cells (row warp, columns lane + 32m)
  int ecell[KEXT];  // (r_eval << 8 | c) of a valid halo cell, -1 otherwise; bit 15: mirrored row fs-1
  T a2u[CPL], b2[CPL], a2w[CPL], b3[CPL];
  bool pin[CPL], win[CPL], inb[CPL];
  int k = 0, prev_tile = -1;
  for (int un = u_beg; un < u_end; ++un) {
    const int tile = un / a.ngroups, grp = un - tile * a.ngroups;
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    const int s_beg = grp * a.G, s_end = min(g.ns, s_beg + a.G);
    if (tile != prev_tile) {
      named_sync(1, NCONS);  // the previous tile's items are done with the halo coefficients
#pragma unroll
      for (int q = 0; q < KEXT; ++q) {
        const int e = tid + NCONS * q;
        ecell[q] = -1;
        if (e < NEXT) {
          CA1[e] = T(0);
          CB1[e] = T(0);
          const int r = e / EXC, c = e - r * EXC;
          const int i = i0 - 1 + r, j = j0 - 1 + c;
          if (i >= g.zbeg && i < L.nzp && j >= 0 && j < L.nxp) {
            const bool fsm = g.fsurf && i == g.fs - 1;  // p[fs-1] = -p[fs+1] (acoustic_kernels.py:135-136)
            const int re = fsm ? r + 2 : r;
            const int64_t o = L.off(i0 - 1 + re, j);
            CA1[e] = cf[ac::kA1M * PL + o];
            CB1[e] = cf[ac::kB1 * PL + o];
            ecell[q] = (re << 8) | c | (fsm ? (1 << 15) : 0);
          }
        }
      }
#pragma unroll
      for (int m = 0; m < CPL; ++m) {
        const int i = i0 + warp, j = j0 + lane + 32 * m;
        inb[m] = i < L.nzp && j < L.nxp;
        const int ie = (g.fsurf && i == g.fs - 1) ? g.fs : i;  // w[fs-1] = w[fs] (163-164)
        const int64_t o = L.off(i, j), oe = L.off(ie, j);
        a2u[m] = cf[ac::kA2U * PL + o];
        b2[m] = cf[ac::kB2 * PL + o];
        a2w[m] = cf[ac::kA2W * PL + oe];
        b3[m] = cf[ac::kB3 * PL + oe];
        pin[m] = inb[m] && ac::in_p(g, i, j);
        win[m] = inb[m] && ac::in_window(g, i, j);
      }
      prev_tile = tile;
    }
    const int rb = g.tile_rcv_beg[tile], re_ = g.tile_rcv_beg[tile + 1];
    const int64_t go = (int64_t)grp * PL;
    T acc_p[CPL], acc_u[CPL];
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
      const int64_t o = go + L.off(i0 + warp, j0 + lane + 32 * m);
      acc_p[m] = (a.acc0 && win[m]) ? a.acc0[o] : T(0);
      acc_u[m] = (a.acc0 && win[m] && a.accum_u) ? a.acc1[o] : T(0);
    }
    for (int sh = s_beg; sh < s_end; ++sh, ++k) {
      const int st = k % S;
      bool ready = !aborted(h);
      if (ready && !mbar_wait(&h->full[st], (k / S) & 1)) {
        set_abort(h, a.flag);
        ready = false;
      }
      const T* U = reinterpret_cast<const T*>(stage0 + st * LY::kStage);
      const T* W = reinterpret_cast<const T*>(stage0 + st * LY::kStage + LY::kE);
      const T* P = reinterpret_cast<const T*>(stage0 + st * LY::kStage + LY::kE + LY::kW);
      const int sz = ih[st].sz, sx = ih[st].sx;
      const bool src_in = sz >= i0 - 1 && sz <= i0 + TZ + 1 && sx >= j0 - 1 && sx <= j0 + TX + 1;
      const int src_cell = src_in ? (((sz - (i0 - 1)) << 8) | (sx - (j0 - 1))) : -2;
      const T sval = ih[st].sval;
      named_sync(1, NCONS);  // the previous item's receiver gather is done with SP / SOU / SOW
      if (ready) {
#pragma unroll
        for (int q = 0; q < KEXT; ++q) {
          const int e = tid + NCONS * q;
          if (e < NEXT) {
            T v = T(0);
            if (ecell[q] >= 0) {
              const int re = (ecell[q] >> 8) & 0x7f, c = ecell[q] & 0xff;
              v = ac::rsub(ac::rmul(CB1[e], P[re * BOXX + c + 3]), ac::rmul(CA1[e], fwd_div(g, U, W, re, c)));
              if (((re << 8) | c) == src_cell) v = ac::radd(v, sval);
              if (ecell[q] & (1 << 15)) v = -v;
            }
            const int r = e / EXC;
            SP[r * SPX + (e - r * EXC)] = v;
          }
        }
      }
      named_sync(1, NCONS);
      const int64_t so = (int64_t)sh * PL;
      const int li = warp, i = i0 + li, r = li + 1;
#pragma unroll
      for (int m = 0; m < CPL; ++m) {
        const int lj = lane + 32 * m, j = j0 + lj, c = lj + 1;
        if (!ready) continue;
        const T* spr = SP + r * SPX + c;
        const T pv = spr[0];
        const int oc = r * BOXX + lj + 4;
        const T dpx = ac::radd(ac::rmul(g.c1, ac::rsub(spr[1], spr[0])), ac::rmul(g.c2, ac::rsub(spr[2], spr[-1])));
        const T un = ac::rsub(ac::rmul(b2[m], U[oc]), ac::rmul(a2u[m], dpx));
        const int rr = (g.fsurf && i == g.fs - 1) ? r + 1 : r;
        const T* spw = SP + rr * SPX + c;
        const T dpz =
            ac::radd(ac::rmul(g.c1, ac::rsub(spw[SPX], spw[0])), ac::rmul(g.c2, ac::rsub(spw[2 * SPX], spw[-SPX])));
        const T wn = ac::rsub(ac::rmul(b3[m], W[(rr + 2) * BOXX + lj + 4]), ac::rmul(a2w[m], dpz));
        SOU[li * TX + lj] = un;
        SOW[li * TX + lj] = wn;
        if (inb[m]) {
          const int64_t o = so + L.off(i, j);
          a.o0[o] = pv;
          a.o1[o] = un;
          a.o2[o] = wn;
          if (a.d1 != nullptr) a.d1[o] = pin[m] ? fwd_div(g, U, W, r, c) : T(0);
          if (win[m]) {
            acc_p[m] += pv * pv;
            acc_u[m] += un * un;
          }
        }
      }
      mbar_arrive(&h->empty[st]);
      if (re_ > rb) {  // only tiles with receivers gather (uniform across the block)
        named_sync(1, NCONS);
        if (ready && rec_p != nullptr && warp == 0) {
          const int64_t rowbase = ((int64_t)sh * g.nt + a.it) * g.nr;
          for (int q = rb + lane; q < re_; q += 32) {
            const int cell = g.trcv_cell[q];
            const int ci = cell >> 16, cj = cell & 0xffff;
            const int64_t o = rowbase + g.trcv_id[q];
            rec_p[o] = SP[(ci + 1) * SPX + cj + 1];
            rec_u[o] = SOU[ci * TX + cj];
            rec_w[o] = SOW[ci * TX + cj];
          }
        }
      }
    }
    if (a.acc0 != nullptr) {
#pragma unroll
      for (int m = 0; m < CPL; ++m) {
        if (!win[m]) continue;
        const int64_t o = go + L.off(i0 + warp, j0 + lane + 32 * m);
        a.acc0[o] = acc_p[m];
        if (a.accum_u) a.acc1[o] = acc_u[m];
      }
    }
  }
}

// ---------------------------------------------------------------------------- adjoint
// Stage: lambda_u (19-row box), lambda_w (22), lambda_p (19), forward p after the step (19),
// forward divergence of the step (19). Scratch: q_u, q_w (masked -alpha2 lambda), q_p
// (masked -alpha1 lambda_p_mid) on their halos, and the three output tiles.
template <typename T>
struct AdjLayout {
  static constexpr int kE = round128(EZ * BOXX * (int)sizeof(T));
  static constexpr int kW = round128(WZ * BOXX * (int)sizeof(T));
  static constexpr int kStage = 4 * kE + kW;
  static constexpr int kStageTx = (4 * EZ + WZ) * BOXX * (int)sizeof(T);
  static constexpr int kQP = round128(EZ * SPX * (int)sizeof(T));
  static constexpr int kSO = round128(TZ * TX * (int)sizeof(T));
  // per-tile coefficients: -alpha2 on the u and w regions, alpha1 and 1 - kappa1 on the p halo
  static constexpr int kCoef = round128((EZ * (TX + 6) + WZ * (TX + 3) + 2 * EZ * (TX + 3)) * (int)sizeof(T));
  static int bytes(int stages) { return 2048 + stages * kStage + kE + kW + kQP + 3 * kSO + kCoef; }
};

constexpr int NU = EZ * (TX + 6);  // u-region cells: rows i0-1.., columns j0-3 .. j0+TX+2 (1330)
constexpr int NW = WZ * EXC;       // w-region cells: rows i0-3.., columns j0-1 .. j0+TX+1 (1474)
constexpr int KU = (NU + NCONS - 1) / NCONS;
constexpr int KW = (NW + NCONS - 1) / NCONS;

template <typename T>
__global__ void __launch_bounds__(NTHREADS, sizeof(T) == 4 ? 2 : 1)
    adj_step_tma(const __grid_constant__ Maps maps, ac::Geo<T> g, StepArgs<T> a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = aligned_smem(smem_raw);
  using LY = AdjLayout<T>;
  const int S = a.stages;
  SmemHeader* h = reinterpret_cast<SmemHeader*>(smem);
  ItemHeader<T>* ih = reinterpret_cast<ItemHeader<T>*>(smem + 512);
  unsigned char* stage0 = smem + 1024;
  unsigned char* scr = stage0 + S * LY::kStage;
  T* QU = reinterpret_cast<T*>(scr);
  T* QW = reinterpret_cast<T*>(scr + LY::kE);
  T* QP = reinterpret_cast<T*>(scr + LY::kE + LY::kW);
  T* OP = reinterpret_cast<T*>(scr + LY::kE + LY::kW + LY::kQP);
  T* OU = OP + LY::kSO / (int)sizeof(T);
  T* OW = OU + LY::kSO / (int)sizeof(T);
  T* CQU = reinterpret_cast<T*>(scr + LY::kE + LY::kW + LY::kQP + 3 * LY::kSO);  // -alpha2 (u region)
  T* CQW = CQU + NU;                                                              // -alpha2 (w region)
  T* CA1 = CQW + NW;                                                              // alpha1 (p halo)
  T* CB1 = CA1 + NEXT;                                                            // 1 - kappa1 (p halo)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], NCONS);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  const int nunits = a.ntiles * a.ngroups;
  const int per = (nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(nunits, u_beg + per);

  if (warp == NCW) {
    if (lane == 0) {
      const int ymap[5][3] = {{0, -1, 0},
                              {1, -3, LY::kE},
                              {2, -1, LY::kE + LY::kW},
                              {3, -1, 2 * LY::kE + LY::kW},
                              {4, -1, 3 * LY::kE + LY::kW}};
      produce<T, 5>(maps, g, a, h, ih, stage0, LY::kStage, LY::kStageTx, ymap, u_beg, u_end, false);
    }
    return;
  }

  const Layout L = g.L;
  const int64_t PL = L.plane;
  const T* cf = a.cf;
  int ecell[KEXT];       // (r << 8 | c) of a valid p-halo cell, -1 otherwise; bit 14: row fs-1; bit 15: row fs+1
  T b2[CPL], b3[CPL];
  bool uin[CPL], win_[CPL], inb[CPL];
  int k = 0, prev_tile = -1;
  bool special = false;  // the tile holds receivers or the free-surface row: outputs pass through shared memory
  for (int un = u_beg; un < u_end; ++un) {
    const int tile = un / a.ngroups, grp = un - tile * a.ngroups;
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    const int s_beg = grp * a.G, s_end = min(g.ns, s_beg + a.G);
    const int cb = g.tile_cell_beg[tile], ce = g.tile_cell_beg[tile + 1];
    if (tile != prev_tile) {
      named_sync(1, NCONS);  // the previous tile's items are done with the coefficient arrays
      for (int e = tid; e < NU; e += NCONS) {
        const int r = e / (TX + 6), c = e - r * (TX + 6);
        CQU[e] = -cf[ac::kA2U * PL + L.off(i0 - 1 + r, j0 - 3 + c)];
      }
      for (int e = tid; e < NW; e += NCONS) {
        const int r = e / EXC, c = e - r * EXC;
        CQW[e] = -cf[ac::kA2W * PL + L.off(i0 - 3 + r, j0 - 1 + c)];
      }
#pragma unroll
      for (int q = 0; q < KEXT; ++q) {
        const int e = tid + NCONS * q;
        ecell[q] = -1;
        if (e < NEXT) {
          CA1[e] = T(0);
          CB1[e] = T(1);
          const int r = e / EXC, c = e - r * EXC;
          const int i = i0 - 1 + r, j = j0 - 1 + c;
          if (i >= g.zbeg && i < L.nzp && j >= 0 && j < L.nxp) {
            const int64_t o = L.off(i, j);
            CA1[e] = cf[ac::kA1M * PL + o];
            CB1[e] = cf[ac::kB1 * PL + o];
            int fl = 0;
            if (g.fsurf && i == g.fs - 1) fl |= 1 << 14;
            if (g.fsurf && i == g.fs + 1 && r >= 2) fl |= 1 << 15;
            ecell[q] = (r << 8) | c | fl;
          }
        }
      }
#pragma unroll
      for (int m = 0; m < CPL; ++m) {
        const int i = i0 + warp, j = j0 + lane + 32 * m;
        inb[m] = i < L.nzp && j < L.nxp;
        const int64_t o = L.off(i, j);
        b2[m] = cf[ac::kB2 * PL + o];
        b3[m] = cf[ac::kB3 * PL + o];
        uin[m] = inb[m] && ac::in_u(g, i, j);
        win_[m] = inb[m] && ac::in_w(g, i, j);
      }
      special = (ce > cb) || (g.fsurf && i0 <= g.fs && g.fs - 1 <= i0 + TZ - 1);
      prev_tile = tile;
    }
    const int64_t go = (int64_t)grp * PL;
    T ag1[KEXT], ag2[CPL];
#pragma unroll
    for (int q = 0; q < KEXT; ++q) {
      ag1[q] = T(0);
      if (ecell[q] >= 0) {
        const int r = (ecell[q] >> 8) & 0x3f, c = ecell[q] & 0xff;
        if (r >= 1 && r <= TZ && c >= 1 && c <= TX) ag1[q] = a.acc0[go + L.off(i0 - 1 + r, j0 - 1 + c)];
      }
    }
#pragma unroll
    for (int m = 0; m < CPL; ++m) ag2[m] = inb[m] ? a.acc1[go + L.off(i0 + warp, j0 + lane + 32 * m)] : T(0);
    const bool inject = a.it >= 1 && (a.rec_p != nullptr || a.rec_u != nullptr || a.rec_w != nullptr) && ce > cb;
    for (int sh = s_beg; sh < s_end; ++sh, ++k) {
      const int st = k % S;
      bool ready = !aborted(h);
      if (ready && !mbar_wait(&h->full[st], (k / S) & 1)) {
        set_abort(h, a.flag);
        ready = false;
      }
      const unsigned char* sb = stage0 + st * LY::kStage;
      const T* LU = reinterpret_cast<const T*>(sb);
      const T* LW = reinterpret_cast<const T*>(sb + LY::kE);
      const T* LP = reinterpret_cast<const T*>(sb + LY::kE + LY::kW);
      const T* PH = reinterpret_cast<const T*>(sb + 2 * LY::kE + LY::kW);
      const T* DH = reinterpret_cast<const T*>(sb + 3 * LY::kE + LY::kW);
      named_sync(1, NCONS);  // the previous item is done with QU / QW / QP / output tiles
      if (ready) {
        for (int e = tid; e < NU; e += NCONS) {
          const int r = e / (TX + 6), c = e - r * (TX + 6);
          QU[r * BOXX + c + 1] = CQU[e] * LU[r * BOXX + c + 1];
        }
        for (int e = tid; e < NW; e += NCONS) {
          const int r = e / EXC, c = e - r * EXC;
          QW[r * BOXX + c + 3] = CQW[e] * LW[r * BOXX + c + 3];
        }
      }
      named_sync(1, NCONS);
      const int64_t so = (int64_t)sh * PL;
      if (ready) {
        // lambda_p after the transposes of the u / w updates' differences of p
        // (acoustic_kernels.py:143-146, 155-158); halo column c sits at stage column c + 3
        auto lp_mid = [&](int r, int c) -> T {
          const T* qu = QU + r * BOXX + c + 3;
          const T* qw = QW + (r + 2) * BOXX + c + 3;
          return LP[r * BOXX + c + 3] + g.c1 * (qu[-1] - qu[0]) + g.c2 * (qu[-2] - qu[1]) +
                 g.c1 * (qw[-BOXX] - qw[0]) + g.c2 * (qw[-2 * BOXX] - qw[BOXX]);
        };
#pragma unroll
        for (int q = 0; q < KEXT; ++q) {
          const int e = tid + NCONS * q;
          if (e < NEXT) {
            T v = T(0);
            if (ecell[q] >= 0) {
              const int r = (ecell[q] >> 8) & 0x3f, c = ecell[q] & 0xff;
              if (!(ecell[q] & (1 << 14))) {  // the mirrored row fs-1 carries no sensitivity
                v = lp_mid(r, c);
                if (ecell[q] & (1 << 15)) v -= lp_mid(r - 2, c);  // adjoint of p[fs-1] = -p[fs+1]
              }
              if (r >= 1 && r <= TZ && c >= 1 && c <= TX) {
                const T lpo = CB1[e] * v;
                ag1[q] -= v * DH[r * BOXX + c + 3];
                if (special) {
                  OP[(r - 1) * TX + c - 1] = lpo;
                } else if (i0 - 1 + r < L.nzp && j0 - 1 + c < L.nxp) {
                  a.o0[so + L.off(i0 - 1 + r, j0 - 1 + c)] = lpo;
                }
              }
            }
            const int rr = e / EXC;
            QP[rr * SPX + (e - rr * EXC)] = -CA1[e] * v;
          }
        }
      }
      named_sync(1, NCONS);
      const int li = warp, i = i0 + li, r = li + 1;
#pragma unroll
      for (int m = 0; m < CPL; ++m) {
        const int lj = lane + 32 * m, j = j0 + lj, c = lj + 1;
        if (!ready) continue;
        const int oc = r * BOXX + lj + 4;
        const T luin = LU[oc], lwin = LW[(r + 2) * BOXX + lj + 4];
        const T* qp = QP + r * SPX + c;
        // transposes of the p update's differences of u and w (acoustic_kernels.py:119-126)
        const T luo = b2[m] * luin + g.c1 * (qp[0] - qp[1]) + g.c2 * (qp[-1] - qp[2]);
        const T lwo = b3[m] * lwin + g.c1 * (qp[0] - qp[SPX]) + g.c2 * (qp[-SPX] - qp[2 * SPX]);
        const T* ph = PH + oc;
        if (uin[m]) ag2[m] -= luin * (g.c1 * (ph[1] - ph[0]) + g.c2 * (ph[2] - ph[-1]));
        if (win_[m]) ag2[m] -= lwin * (g.c1 * (ph[BOXX] - ph[0]) + g.c2 * (ph[2 * BOXX] - ph[-BOXX]));
        if (special) {
          OU[li * TX + lj] = luo;
          OW[li * TX + lj] = lwo;
        } else if (inb[m]) {
          const int64_t o = so + L.off(i, j);
          a.o1[o] = luo;
          a.o2[o] = lwo;
        }
      }
      mbar_arrive(&h->empty[st]);
      if (special) {
        named_sync(1, NCONS);
        if (ready && inject && warp == 0) {
          // dL/d records of step it-1 enter the state after step it-1 (acoustic_kernels.py:167-169)
          const int64_t rowbase = ((int64_t)sh * g.nt + (a.it - 1)) * g.nr;
          for (int q = cb + lane; q < ce; q += 32) {
            const int cell = g.tcell_cell[q];
            const int ci = cell >> 16, cj = cell & 0xffff;
            T ap = T(0), au = T(0), aw = T(0);
            for (int mm = g.tcell_rbeg[q]; mm < g.tcell_rbeg[q + 1]; ++mm) {
              const int64_t o = rowbase + g.cell_rcv[mm];
              if (a.rec_p) ap += a.rec_p[o];
              if (a.rec_u) au += a.rec_u[o];
              if (a.rec_w) aw += a.rec_w[o];
            }
            OP[ci * TX + cj] += ap;
            OU[ci * TX + cj] += au;
            OW[ci * TX + cj] += aw;
          }
        }
        named_sync(1, NCONS);
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
          const int lj = lane + 32 * m, j = j0 + lj;
          if (!ready || !inb[m]) continue;
          T wv = OW[li * TX + lj];
          if (g.fsurf && i == g.fs - 1) wv = T(0);  // adjoint of w[fs-1] = w[fs]
          if (g.fsurf && i == g.fs && li >= 1) wv += OW[(li - 1) * TX + lj];
          const int64_t o = so + L.off(i, j);
          a.o0[o] = OP[li * TX + lj];
          a.o1[o] = OU[li * TX + lj];
          a.o2[o] = wv;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < KEXT; ++q) {
      if (ecell[q] >= 0) {
        const int r = (ecell[q] >> 8) & 0x3f, c = ecell[q] & 0xff;
        if (r >= 1 && r <= TZ && c >= 1 && c <= TX) a.acc0[go + L.off(i0 - 1 + r, j0 - 1 + c)] = ag1[q];
      }
    }
#pragma unroll
    for (int m = 0; m < CPL; ++m)
      if (inb[m]) a.acc1[go + L.off(i0 + warp, j0 + lane + 32 * m)] = ag2[m];
  }
}

}  // namespace ac2
}  // namespace adfwi
