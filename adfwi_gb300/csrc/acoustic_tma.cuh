// TMA-pipelined acoustic forward / adjoint steps (included by acoustic.cu).
//
// Work of one launch = all (tile, shot) items of one time step. A persistent block owns a
// contiguous range of "units" (one tile x one group of G shots; tile-major), so every
// accumulator a unit produces (illumination, coefficient gradients) belongs to one block
// and is flushed once, deterministically, into the group's partial plane.
//
// Inside a block, warp 8 is the producer: one lane issues, per item, the TMA tile loads of
// every plane the item reads into the next free pipeline stage and arms the stage's
// `full` mbarrier with the byte count. Warps 0-7 are the consumers: they wait on `full`,
// compute, and arrive on the stage's `empty` mbarrier when they no longer read it, so the
// loads of the next items overlap the arithmetic of the current one. Every wait is bounded
// (kWaitLimit polls); a wait that runs out raises the device error flag and a block-wide
// abort flag, after which the block skips its remaining work (consumers still meet every
// named barrier, so no thread is left waiting on one that never fills).
#pragma once
#include "tma.cuh"

namespace adfwi {
namespace ac2 {

constexpr int TX = 64;             // tile columns
constexpr int TZ = 16;             // tile rows
constexpr int BOXX = TX + 8;       // TMA box width: columns j0-4 .. j0+TX+3 (16-byte aligned start)
constexpr int EZ = TZ + 3;         // rows i0-1 .. i0+TZ+1
constexpr int WZ = TZ + 6;         // rows i0-3 .. i0+TZ+2
constexpr int SPX = TX + 4;        // p-halo row length in shared memory (67 used)
constexpr int NCW = 16;            // consumer warps
constexpr int NCONS = NCW * 32;    // consumer threads
constexpr int NTHREADS = NCONS + 32;
constexpr int RPW = TZ / NCW;      // tile rows per consumer warp
constexpr int CPL = TX / 32;       // tile columns per lane
constexpr int NSLOT = 2;           // coefficient slots (tile changes are double-buffered)
constexpr int MAXSTAGES = 8;

__host__ __device__ constexpr int round128(int bytes) { return (bytes + 127) / 128 * 128; }

// Per-item scalars the producer hands to the consumers with the stage.
template <typename T>
struct ItemHeader {
  int sz, sx;
  T sval;
};

// ---------------------------------------------------------------------------- forward
template <typename T>
struct FwdLayout {
  static constexpr int kE = round128(EZ * BOXX * (int)sizeof(T));  // one 19-row box
  static constexpr int kW = round128(WZ * BOXX * (int)sizeof(T));  // the 22-row w box
  static constexpr int kStage = 2 * kE + kW;                       // U, W, P
  static constexpr int kStageTx = (2 * EZ + WZ) * BOXX * (int)sizeof(T);
  static constexpr int kSlot = 3 * kE;                             // A1, A2, D
  static constexpr int kSlotTx = 3 * EZ * BOXX * (int)sizeof(T);
  static constexpr int kSP = round128(EZ * SPX * (int)sizeof(T));
  static constexpr int kSO = round128(TZ * TX * (int)sizeof(T));
  // 1 KB header (barriers, abort flag, item headers) + up to 1 KB to align the base
  static int bytes(int stages) { return 2048 + NSLOT * kSlot + stages * kStage + kSP + 2 * kSO; }
};

struct Maps {
  CUtensorMap u, w, p, coef;  // coef: planes 0 = alpha1, 1 = alpha2, 2 = damp
};

template <typename T>
struct FwdArgs {
  int it, G, ngroups, ntiles, accum_u, stages;
  const T* wav;
  T* p1;
  T* u1;
  T* w1;
  T* d1;
  T* rec_p;
  T* rec_u;
  T* rec_w;
  T* ill_p;
  T* ill_u;
  int* flag;
};

template <typename T>
__device__ __forceinline__ T v2_divergence(const ac::Geo<T>& g, const T* U, const T* W, int r, int c) {
  const int cc = c + 3;
  T t1 = ac::rsub(ac::radd(ac::rsub(U[r * BOXX + cc], U[r * BOXX + cc - 1]), W[(r + 2) * BOXX + cc]),
                  W[(r + 1) * BOXX + cc]);
  T t2 = ac::rsub(ac::radd(ac::rsub(U[r * BOXX + cc + 1], U[r * BOXX + cc - 2]), W[(r + 3) * BOXX + cc]),
                  W[r * BOXX + cc]);
  return ac::radd(ac::rmul(g.c1, t1), ac::rmul(g.c2, t2));
}

template <typename T>
__device__ __forceinline__ T v2_eval_p(const ac::Geo<T>& g, const T* U, const T* W, const T* P, const T* A1,
                                       const T* D, int i, int j, int r, int c, int sz, int sx, T sval) {
  const int o = r * BOXX + c + 3;
  T v = P[o];
  if (ac::in_p(g, i, j)) {
    T k1 = ac::rmul(D[o], g.dt);
    v = ac::rsub(ac::rmul(ac::rsub(T(1), k1), v), ac::rmul(A1[o], v2_divergence(g, U, W, r, c)));
  }
  if (i == sz && j == sx) v = ac::radd(v, sval);
  return v;
}

// Shared-memory map of the pipelined kernels: header | coefficient slots | stages | scratch.
struct SmemHeader {
  uint64_t full[MAXSTAGES];
  uint64_t empty[MAXSTAGES];
  uint64_t cfull[NSLOT];
  uint64_t cempty[NSLOT];
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

template <typename T>
__global__ void __launch_bounds__(NTHREADS, sizeof(T) == 4 ? 2 : 1) fwd_step_tma(const __grid_constant__ Maps maps, ac::Geo<T> g,
                                                          FwdArgs<T> a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = aligned_smem(smem_raw);
  using LY = FwdLayout<T>;
  const int S = a.stages;
  SmemHeader* h = reinterpret_cast<SmemHeader*>(smem);
  ItemHeader<T>* ih = reinterpret_cast<ItemHeader<T>*>(smem + 512);
  unsigned char* slot0 = smem + 1024;
  unsigned char* stage0 = slot0 + NSLOT * LY::kSlot;
  T* SP = reinterpret_cast<T*>(stage0 + S * LY::kStage);
  T* SOU = reinterpret_cast<T*>(stage0 + S * LY::kStage + LY::kSP);
  T* SOW = reinterpret_cast<T*>(stage0 + S * LY::kStage + LY::kSP + LY::kSO);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], NCONS);
    }
    for (int s = 0; s < NSLOT; ++s) {
      mbar_init(&h->cfull[s], 1);
      mbar_init(&h->cempty[s], NCONS);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();

  const int nunits = a.ntiles * a.ngroups;
  const int per = (nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(nunits, u_beg + per);

  if (warp == NCW) {  // ------------------------------------------------------- producer
    if (lane == 0) {
      prefetch_tensormap(&maps.u);
      prefetch_tensormap(&maps.w);
      prefetch_tensormap(&maps.p);
      prefetch_tensormap(&maps.coef);
      int k = 0, cgen = 0, prev_tile = -1;
      for (int un = u_beg; un < u_end && !aborted(h); ++un) {
        const int tile = un / a.ngroups, grp = un - tile * a.ngroups;
        const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
        const int x = j0 - 4 + GX, ye = i0 - 1 + GZ, yw = i0 - 3 + GZ;
        if (tile != prev_tile) {
          const int cs = cgen % NSLOT;
          if (cgen >= NSLOT && !mbar_wait(&h->cempty[cs], ((cgen / NSLOT) - 1) & 1)) {
            set_abort(h, a.flag);
            break;
          }
          unsigned char* cb = slot0 + cs * LY::kSlot;
          mbar_arrive_expect_tx(&h->cfull[cs], LY::kSlotTx);
          tma_load_3d(cb, &maps.coef, x, ye, 0, &h->cfull[cs]);
          tma_load_3d(cb + LY::kE, &maps.coef, x, ye, 1, &h->cfull[cs]);
          tma_load_3d(cb + 2 * LY::kE, &maps.coef, x, ye, 2, &h->cfull[cs]);
          ++cgen;
          prev_tile = tile;
        }
        const int s_beg = grp * a.G, s_end = min(g.ns, s_beg + a.G);
        for (int sh = s_beg; sh < s_end; ++sh, ++k) {
          const int st = k % S;
          if (k >= S && !mbar_wait(&h->empty[st], ((k / S) - 1) & 1)) {
            set_abort(h, a.flag);
            break;
          }
          ih[st].sz = g.src_z[sh];
          ih[st].sx = g.src_x[sh];
          ih[st].sval = ac::rmul(g.dt, a.wav[(int64_t)sh * g.nt + a.it]);
          unsigned char* sb = stage0 + st * LY::kStage;
          mbar_arrive_expect_tx(&h->full[st], LY::kStageTx);  // releases the header writes above
          tma_load_3d(sb, &maps.u, x, ye, sh, &h->full[st]);
          tma_load_3d(sb + LY::kE, &maps.w, x, yw, sh, &h->full[st]);
          tma_load_3d(sb + LY::kE + LY::kW, &maps.p, x, ye, sh, &h->full[st]);
        }
      }
      // do not leave the block while a load it issued may still be landing
      for (int q = max(0, k - S); q < k; ++q) mbar_wait(&h->full[q % S], (q / S) & 1);
      for (int q = max(0, cgen - NSLOT); q < cgen; ++q) mbar_wait(&h->cfull[q % NSLOT], (q / NSLOT) & 1);
    }
    return;
  }

  // --------------------------------------------------------------------- consumers
  const Layout L = g.L;
  int k = 0, cgen = 0, prev_tile = -1;
  const T* A1 = nullptr;
  const T* A2 = nullptr;
  const T* D = nullptr;
  for (int un = u_beg; un < u_end; ++un) {
    const int tile = un / a.ngroups, grp = un - tile * a.ngroups;
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    const int s_beg = grp * a.G, s_end = min(g.ns, s_beg + a.G);
    if (tile != prev_tile) {
      if (prev_tile >= 0) mbar_arrive(&h->cempty[(cgen - 1) % NSLOT]);  // done with the old tile's slot
      const int cs = cgen % NSLOT;
      if (!aborted(h) && !mbar_wait(&h->cfull[cs], (cgen / NSLOT) & 1)) set_abort(h, a.flag);
      const unsigned char* cb = slot0 + cs * LY::kSlot;
      A1 = reinterpret_cast<const T*>(cb);
      A2 = reinterpret_cast<const T*>(cb + LY::kE);
      D = reinterpret_cast<const T*>(cb + 2 * LY::kE);
      ++cgen;
      prev_tile = tile;
    }
    const int rb = g.tile_rcv_beg[tile], re = g.tile_rcv_beg[tile + 1];
    // Illumination partials of this unit: read now, so the load overlaps the unit's items.
    const int64_t go = (int64_t)grp * L.plane;
    T acc_p[RPW][CPL], acc_u[RPW][CPL];
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
      const int i = i0 + warp * RPW + q;
#pragma unroll
      for (int m = 0; m < CPL; ++m) {
        const int j = j0 + lane + 32 * m;
        const bool w = a.ill_p != nullptr && i < L.nzp && j < L.nxp && ac::in_window(g, i, j);
        acc_p[q][m] = w ? a.ill_p[go + L.off(i, j)] : T(0);
        acc_u[q][m] = (w && a.accum_u) ? a.ill_u[go + L.off(i, j)] : T(0);
      }
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
      const T sval = ih[st].sval;
      named_sync(1, NCONS);  // the previous item's receiver gather has finished with SP / SOU / SOW
      if (ready) {
        for (int e = tid; e < EZ * (TX + 3); e += NCONS) {
          const int r = e / (TX + 3), c = e - r * (TX + 3);
          const int i = i0 - 1 + r, j = j0 - 1 + c;
          T v = T(0);
          if (i >= g.zbeg && i < L.nzp && j >= 0 && j < L.nxp) {
            if (g.fsurf && i == g.fs - 1)
              v = -v2_eval_p(g, U, W, P, A1, D, i + 2, j, r + 2, c, sz, sx, sval);
            else
              v = v2_eval_p(g, U, W, P, A1, D, i, j, r, c, sz, sx, sval);
          }
          SP[r * SPX + c] = v;
        }
      }
      named_sync(1, NCONS);
      const int64_t so = (int64_t)sh * L.plane;
#pragma unroll
      for (int q = 0; q < RPW; ++q) {
        const int li = warp * RPW + q;
        const int i = i0 + li;
        const int r = li + 1;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
          const int lj = lane + 32 * m;
          const int j = j0 + lj;
          const int c = lj + 1;
          if (!ready) continue;
          const T pv = SP[r * SPX + c];
          const int oc = r * BOXX + lj + 4;  // offset of (i, j) in a 19-row box
          T uo = U[oc], un = uo;
          if (ac::in_u(g, i, j)) {
            T k2 = ac::rmul(ac::rmul(T(0.5), ac::radd(D[oc], D[oc + 1])), g.dt);
            T dpx = ac::radd(ac::rmul(g.c1, ac::rsub(SP[r * SPX + c + 1], SP[r * SPX + c])),
                             ac::rmul(g.c2, ac::rsub(SP[r * SPX + c + 2], SP[r * SPX + c - 1])));
            un = ac::rsub(ac::rmul(ac::rsub(T(1), k2), uo), ac::rmul(A2[oc], dpx));
          }
          const int ie = (g.fsurf && i == g.fs - 1) ? g.fs : i;
          const int rr = r + (ie - i);
          const int oe = rr * BOXX + lj + 4;
          T wo = W[(rr + 2) * BOXX + lj + 4], wn = wo;
          if (ac::in_w(g, ie, j)) {
            T k3 = ac::rmul(ac::rmul(T(0.5), ac::radd(D[oe], D[oe + BOXX])), g.dt);
            T dpz = ac::radd(ac::rmul(g.c1, ac::rsub(SP[(rr + 1) * SPX + c], SP[rr * SPX + c])),
                             ac::rmul(g.c2, ac::rsub(SP[(rr + 2) * SPX + c], SP[(rr - 1) * SPX + c])));
            wn = ac::rsub(ac::rmul(ac::rsub(T(1), k3), wo), ac::rmul(A2[oe], dpz));
          }
          T dv = T(0);
          if (a.d1 != nullptr && ac::in_p(g, i, j)) dv = v2_divergence(g, U, W, r, c);
          SOU[li * TX + lj] = un;
          SOW[li * TX + lj] = wn;
          if (i < L.nzp && j < L.nxp) {
            const int64_t o = so + L.off(i, j);
            a.p1[o] = pv;
            a.u1[o] = un;
            a.w1[o] = wn;
            if (a.d1 != nullptr) a.d1[o] = dv;
            if (ac::in_window(g, i, j)) {
              acc_p[q][m] += pv * pv;
              acc_u[q][m] += un * un;
            }
          }
        }
      }
      mbar_arrive(&h->empty[st]);  // this thread no longer reads the stage
      named_sync(1, NCONS);        // SOU / SOW complete for the receiver gather
      if (ready && a.rec_p != nullptr && warp == 0) {
        const int64_t rowbase = ((int64_t)sh * g.nt + a.it) * g.nr;
        for (int q = rb + lane; q < re; q += 32) {
          const int cell = g.trcv_cell[q];
          const int li = cell >> 16, lj = cell & 0xffff;
          const int64_t o = rowbase + g.trcv_id[q];
          a.rec_p[o] = SP[(li + 1) * SPX + lj + 1];
          a.rec_u[o] = SOU[li * TX + lj];
          a.rec_w[o] = SOW[li * TX + lj];
        }
      }
    }
    if (a.ill_p != nullptr) {
#pragma unroll
      for (int q = 0; q < RPW; ++q) {
        const int i = i0 + warp * RPW + q;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
          const int j = j0 + lane + 32 * m;
          if (i < L.nzp && j < L.nxp && ac::in_window(g, i, j)) {
            a.ill_p[go + L.off(i, j)] = acc_p[q][m];
            if (a.accum_u) a.ill_u[go + L.off(i, j)] = acc_u[q][m];
          }
        }
      }
    }
  }
}

}  // namespace ac2
}  // namespace adfwi
