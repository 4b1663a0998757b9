// Vectorised acoustic forward step (included by acoustic.cu after acoustic_tma.cuh).
//
// Same work, pipeline and results as fwd_step_tma (the TMA producer warp, the stage ring
// and the 16 x 64 tiles are shared), with the arithmetic reorganised to cut instructions
// per cell-update: every consumer thread owns four adjacent columns and moves them with
// 16-byte shared / global accesses, its per-tile coefficients sit in registers (loaded once
// per tile with vector loads, zeroed outside the grid so no cell test remains in the loop),
// the divergence history is written by the halo pass that computes it, and the new-p halo
// is double-buffered so an item needs one barrier.
//
// A block is one producer warp and one group of eight consumer warps that takes every item of
// the block's units in ring order (a second consumer group on the same ring could wait on a
// stage two phases ahead of its last fill, where an mbarrier parity wait passes falsely).
// Two or more blocks share an SM, so one block's barrier waits overlap another's work.
//
// Per item the consumer group runs:
//   halo pass  (180 threads): p after the step on rows i0-1 .. i0+17 and box columns
//              j0-4 .. j0+67 (2 rows x 4 columns per thread; columns j0-4 .. j0-2 and
//              j0+66, j0+67 are computed but never read);
//   tile pass  (256 threads): u and w after the step on the 16 x 64 tile (1 row x 4 columns
//              per thread), the three stores and the illumination;
//   receivers  (tiles holding receivers only): the consumers arrive on the stage's `stored`
//              mbarrier instead of `empty`, and the 31 idle lanes of the producer warp (the
//              relay) gather p, u, w of the item from the global stores just made and release
//              the stage, so a receiver tile costs the consumers nothing extra.
// The operation order of every cell value is the reference's (acoustic_kernels.py:115-160),
// with explicitly rounded arithmetic as in fwd_step_tma, so the records are bit-identical.
#pragma once

namespace adfwi {
namespace ac2 {

constexpr int VG = 256;                      // threads of a consumer group
constexpr int VTHREADS = VG + 32;            // the consumer group + the producer warp
#ifndef ADFWI_VEC_MINB
#define ADFWI_VEC_MINB 3
#endif
constexpr int VMINB = ADFWI_VEC_MINB;        // resident blocks per SM of the shallow-ring forward
constexpr int VDEEP = 2;                     // resident blocks per SM of the deep-ring variants
constexpr int CGE = BOXX / 4;                // four-column groups across the box (18)
constexpr int ERP = (EZ + 1) / 2;            // row pairs of the p halo (10)
constexpr int EXT_TASKS = ERP * CGE;         // halo tasks (180)
constexpr int CGT = TX / 4;                  // four-column groups across the tile (16)
static_assert(TZ * CGT == VG, "one tile task per group thread");
static_assert(EXT_TASKS <= VG, "one halo task per group thread at most");
static_assert(BOXX % 4 == 0 && (BOXX * 4) % 16 == 0, "16-byte aligned box rows");

// Shared memory of the vectorised kernels: 128-byte alignment suffices (plain TMA boxes, no
// swizzle); the 1024-byte header (mbarriers, item headers) comes first.
__device__ __forceinline__ unsigned char* aligned_smem128(unsigned char* raw) {
  return raw + ((128u - (smem_u32(raw) & 127u)) & 127u);
}
constexpr int kVecSmemFixed = 1024 + 128;
constexpr int RC = 3;  // receiver cells a relay lane keeps in registers for a unit (31 RC per tile)

__device__ __forceinline__ void ld4(const float* p, float (&r)[4]) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  r[0] = q.x, r[1] = q.y, r[2] = q.z, r[3] = q.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&r)[4]) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  const double2 b = *reinterpret_cast<const double2*>(p + 2);
  r[0] = a.x, r[1] = a.y, r[2] = b.x, r[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&r)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&r)[4]) {
  *reinterpret_cast<double2*>(p) = make_double2(r[0], r[1]);
  *reinterpret_cast<double2*>(p + 2) = make_double2(r[2], r[3]);
}

// read-only (non-coherent path) loads of data that no thread writes during the launch
__device__ __forceinline__ void ldg4(const float* p, float (&r)[4]) {
  const float4 q = __ldg(reinterpret_cast<const float4*>(p));
  r[0] = q.x, r[1] = q.y, r[2] = q.z, r[3] = q.w;
}
__device__ __forceinline__ void ldg4(const double* p, double (&r)[4]) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p + 2));
  r[0] = a.x, r[1] = a.y, r[2] = b.x, r[3] = b.y;
}

// twelve consecutive values (three 16-byte groups)
template <typename T>
__device__ __forceinline__ void ld12(const T* p, T (&r)[12]) {
  T x[4], y[4], z[4];
  ld4(p, x);
  ld4(p + 4, y);
  ld4(p + 8, z);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    r[q] = x[q];
    r[4 + q] = y[q];
    r[8 + q] = z[q];
  }
}

template <typename T>
struct VecFwdLayout {
  static constexpr int kE = round128(EZ * BOXX * (int)sizeof(T));
  static constexpr int kW = round128(WZ * BOXX * (int)sizeof(T));
  static constexpr int kStage = 2 * kE + kW;  // U, W, P boxes
  static constexpr int kStageTx = (2 * EZ + WZ) * BOXX * (int)sizeof(T);
  static constexpr int kSP = kE;  // new p on the halo (box columns)
  static constexpr int kGroup = 2 * kSP;
  static int bytes(int stages) { return kVecSmemFixed + stages * kStage + kGroup; }
};

// Relay lanes (lanes 1..31 of the producer warp). For every item of the block's units whose
// tile `relayed(tile)` holds, wait until the consumers have stored the item (their VG arrivals
// on the stage's `stored` mbarrier, release / acquire at CTA scope, so the item's global stores
// are visible here), release the stage to the producer with VG arrivals on `empty`, and run
// `work(tile, shot)`, which touches global memory only (`prep(tile)` runs once per relayed
// unit first). The relay cannot fall two `stored` phases behind: the producer refills a stage
// only after the relay's arrival on `empty`.
template <typename T, typename Pred, typename Prep, typename Work>
__device__ __forceinline__ void relay(const ac::Geo<T>& g, const StepArgs<T>& a, SmemHeader* h, int u_beg,
                                      int u_end, int lane, Pred relayed, Prep prep, Work work) {
  const int S = a.stages;
  unsigned par = 0;  // parity of each stage's next `stored` phase
  int k = 0;
  for (int un = u_beg; un < u_end && !aborted(h); ++un) {
    const int grp = un / a.ntiles, tile = un - grp * a.ntiles;
    const int s_beg = g.grp_beg[grp], s_end = g.grp_beg[grp + 1];
    if (!relayed(tile)) {
      k += s_end - s_beg;
      continue;
    }
    prep(tile);
    for (int sh = s_beg; sh < s_end; ++sh, ++k) {
      const int st = k % S;
      if (!mbar_wait(&h->stored[st], (par >> st) & 1u)) {
        set_abort(h, a.flag);
        return;
      }
      par ^= 1u << st;
      if (lane == 1) mbar_arrive_cnt(&h->empty[st], VG);
      work(tile, sh);
    }
  }
}

// MB: resident blocks per SM the variant is compiled for (VMINB: shallow ring; VDEEP: fewer
// blocks with more registers and one stage more, for grids whose fields do not stay in L2).
template <typename T, int MB>
__global__ void __launch_bounds__(VTHREADS, MB)
    fwd_step_vec(const __grid_constant__ Maps maps, ac::Geo<T> g, StepArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = aligned_smem128(smem_raw);
  using LY = VecFwdLayout<T>;
  const int S = a.stages;
  SmemHeader* h = reinterpret_cast<SmemHeader*>(smem);
  ItemHeader<T>* ih = reinterpret_cast<ItemHeader<T>*>(smem + 512);
  unsigned char* stage0 = smem + 1024;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], VG);
      mbar_init(&h->stored[s], VG);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  griddep_launch_dependents();
  griddep_wait();
  const int nunits = a.ntiles * a.ngroups;
  const int per = (nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(nunits, u_beg + per);
  const bool recording = a.rec_p != nullptr;

  if (warp == VG / 32) {
    if (lane == 0) {
      const int ymap[3][3] = {{0, -1, 0}, {1, -3, LY::kE}, {2, -1, LY::kE + LY::kW}};
      produce<T, 3>(maps, g, a, h, ih, stage0, LY::kStage, LY::kStageTx, ymap, u_beg, u_end, true);
    } else if (recording) {
      // records of step it (acoustic_kernels.py:167-169) from the item's stored p, u, w; a lane
      // keeps the cells and ids of its receivers rb + lane - 1 + 31 m (m < RC) for the unit
      const Layout L = g.L;
      T* rp = const_cast<T*>(a.rec_p);
      T* ru = const_cast<T*>(a.rec_u);
      T* rw = const_cast<T*>(a.rec_w);
      int64_t coff[RC] = {};
      int rid[RC] = {}, rn = 0, rb = 0, re = 0, i0 = 0, j0 = 0;
      relay(g, a, h, u_beg, u_end, lane, [&](int tile) { return g.tile_rcv_beg[tile + 1] > g.tile_rcv_beg[tile]; },
            [&](int tile) {
              rb = g.tile_rcv_beg[tile];
              re = g.tile_rcv_beg[tile + 1];
              i0 = g.zbeg + (tile / g.tiles_x) * TZ;
              j0 = (tile % g.tiles_x) * TX;
              rn = 0;
#pragma unroll
              for (int m = 0; m < RC; ++m) {
                const int q = rb + lane - 1 + 31 * m;
                if (q < re) {
                  const int cell = g.trcv_cell[q];
                  coff[m] = L.off(i0 + (cell >> 16), j0 + (cell & 0xffff));
                  rid[m] = g.trcv_id[q];
                  rn = m + 1;
                }
              }
            },
            [&](int tile, int sh) {
              const int64_t rowbase = ((int64_t)sh * g.nt + a.it) * g.nr, so = (int64_t)sh * L.plane;
              T vp[RC], vu[RC], vw[RC];
#pragma unroll
              for (int m = 0; m < RC; ++m)
                if (m < rn) {
                  vp[m] = a.o0[so + coff[m]];
                  vu[m] = a.o1[so + coff[m]];
                  vw[m] = a.o2[so + coff[m]];
                }
#pragma unroll
              for (int m = 0; m < RC; ++m)
                if (m < rn) {
                  rp[rowbase + rid[m]] = vp[m];
                  ru[rowbase + rid[m]] = vu[m];
                  rw[rowbase + rid[m]] = vw[m];
                }
              for (int q = rb + lane - 1 + 31 * RC; q < re; q += 31) {  // more than 31 RC receivers in the tile
                const int cell = g.trcv_cell[q];
                const int64_t o = rowbase + g.trcv_id[q], c = so + L.off(i0 + (cell >> 16), j0 + (cell & 0xffff));
                rp[o] = a.o0[c];
                ru[o] = a.o1[c];
                rw[o] = a.o2[c];
              }
            });
    }
    return;
  }

  const int gt = tid;
  constexpr int bar = 1;
  unsigned char* gs = stage0 + S * LY::kStage;
  T* SPB0 = reinterpret_cast<T*>(gs);
  T* SPB1 = reinterpret_cast<T*>(gs + LY::kSP);
  const Layout L = g.L;
  const int64_t PL = L.plane;

  // halo task: rows 2*erp, 2*erp+1 of the p halo, box columns 4*ecg .. 4*ecg+3
  const bool has_ext = gt < EXT_TASKS;
  const int erp = gt / CGE, ecg = gt - erp * CGE;
  // tile task: tile row tli, tile columns 4*tcg .. 4*tcg+3
  const int tli = gt / CGT, tcg = gt - tli * CGT;

  T ca1[2][4], cb1[2][4];  // halo coefficients at the evaluated rows, zero outside the grid
  int eve[2];              // evaluated box row of halo row 2*erp+q (-1: no such row)
  bool eneg[2];            // mirrored row fs-1: p = -p(fs+1)
  unsigned epin[2];        // p-region bits of the tile cells of halo row 2*erp+q (divergence history)
  T a2u[4], b2[4], a2w[4], b3[4];
  unsigned twin = 0;       // illumination-window bits of the tile cells
  bool trow = false, tfs = false;
  int prev_tile = -1, prev_model = -1, sel = 0, k = 0;

  for (int un = u_beg; un < u_end; ++un) {
    const int sgrp = un / a.ntiles, tile = un - sgrp * a.ntiles;
    const int s_beg = g.grp_beg[sgrp], s_end = g.grp_beg[sgrp + 1];
    const int model = g.grp_model[sgrp];
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    if (tile != prev_tile || model != prev_model) {
      const T* cf = a.cf + (int64_t)model * a.cf_stride;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int r = 2 * erp + q;
        eve[q] = -1;
        eneg[q] = false;
        epin[q] = 0;
        if (!has_ext || r >= EZ) continue;
        const int i = i0 - 1 + r;
        const bool mir = g.fsurf && i == g.fs - 1;  // p[fs-1] = -p[fs+1] (acoustic_kernels.py:135-136)
        const int re = mir ? r + 2 : r;
        eve[q] = re;
        eneg[q] = mir;
        const int jb = j0 - 4 + 4 * ecg;
        const int64_t o = L.off(i0 - 1 + re, jb);
        ld4(cf + ac::kA1M * PL + o, ca1[q]);
        ld4(cf + ac::kB1 * PL + o, cb1[q]);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int j = jb + c;
          if (!(i >= g.zbeg && i < L.nzp && j >= 0 && j < L.nxp)) {
            ca1[q][c] = T(0);
            cb1[q][c] = T(0);
          }
          if (ac::in_p(g, i, j) && i < L.nzp && j < L.nxp) epin[q] |= 1u << c;
        }
      }
      {
        const int i = i0 + tli, jb = j0 + 4 * tcg;
        trow = i < L.nzp;
        tfs = g.fsurf && i == g.fs - 1;  // w[fs-1] = w[fs] (acoustic_kernels.py:163-164)
        const int ie = tfs ? g.fs : i;
        ld4(cf + ac::kA2U * PL + L.off(i, jb), a2u);
        ld4(cf + ac::kB2 * PL + L.off(i, jb), b2);
        ld4(cf + ac::kA2W * PL + L.off(ie, jb), a2w);
        ld4(cf + ac::kB3 * PL + L.off(ie, jb), b3);
        twin = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (trow && jb + c < L.nxp && ac::in_window(g, i, jb + c)) twin |= 1u << c;
      }
      prev_tile = tile;
      prev_model = model;
    }
    const int rb = g.tile_rcv_beg[tile], re_ = g.tile_rcv_beg[tile + 1];
    const int64_t go = (int64_t)sgrp * PL;
    const int64_t ot = L.off(i0 + tli, j0 + 4 * tcg);  // this thread's tile cells
    // the unit's illumination sums continue the partial planes' running sums
    T accp[4] = {T(0), T(0), T(0), T(0)}, accu[4] = {T(0), T(0), T(0), T(0)};
    if (a.acc0 != nullptr && twin) {
      ld4(a.acc0 + go + ot, accp);
      if (a.accum_u) ld4(a.acc1 + go + ot, accu);
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
      T* SP = sel ? SPB1 : SPB0;
      const int64_t so = (int64_t)sh * PL;
      // ---- halo pass: p after the step
      if (ready && has_ext) {
        const int sz = ih[st].sz, sx = ih[st].sx;
        const T sval = ih[st].sval;
        const int jb = j0 - 4 + 4 * ecg;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int re = eve[q];
          if (re < 0) continue;
          const int r = 2 * erp + q;
          T uu[12], w0[4], w1[4], w2[4], w3[4], pp[4];
          ld12(U + re * BOXX + 4 * ecg - 4, uu);
          const T* wr = W + re * BOXX + 4 * ecg;
          ld4(wr, w0);
          ld4(wr + BOXX, w1);
          ld4(wr + 2 * BOXX, w2);
          ld4(wr + 3 * BOXX, w3);
          ld4(P + re * BOXX + 4 * ecg, pp);
          T dv[4], v[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            // divergence in the reference's operation order (acoustic_kernels.py:118-127)
            const T t1 = ac::rsub(ac::radd(ac::rsub(uu[4 + c], uu[3 + c]), w2[c]), w1[c]);
            const T t2 = ac::rsub(ac::radd(ac::rsub(uu[5 + c], uu[2 + c]), w3[c]), w0[c]);
            dv[c] = ac::radd(ac::rmul(g.c1, t1), ac::rmul(g.c2, t2));
            v[c] = ac::rsub(ac::rmul(cb1[q][c], pp[c]), ac::rmul(ca1[q][c], dv[c]));
          }
          if (sz == i0 - 1 + re) {
            const int sc = sx - jb;
#pragma unroll
            for (int c = 0; c < 4; ++c)
              if (sc == c) v[c] = ac::radd(v[c], sval);
          }
          if (eneg[q]) {
#pragma unroll
            for (int c = 0; c < 4; ++c) v[c] = -v[c];
          }
          st4(SP + r * BOXX + 4 * ecg, v);
          if (a.d1 != nullptr && r >= 1 && r <= TZ && ecg >= 1 && ecg <= CGT && i0 - 1 + r < L.nzp) {
            T dd[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) dd[c] = (epin[q] >> c) & 1u ? dv[c] : T(0);
            st4(a.d1 + so + L.off(i0 - 1 + r, jb), dd);
          }
        }
      }
      named_sync(bar, VG);
      // ---- tile pass: u, w after the step, stores, illumination
      if (ready && trow) {
        const int r = tli + 1, b = 4 * tcg + 4;
        T ss[12], uo[4], un[4], wn[4];
        ld12(SP + r * BOXX + 4 * tcg, ss);
        ld4(U + r * BOXX + b, uo);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const T dpx = ac::radd(ac::rmul(g.c1, ac::rsub(ss[5 + c], ss[4 + c])),
                                 ac::rmul(g.c2, ac::rsub(ss[6 + c], ss[3 + c])));
          un[c] = ac::rsub(ac::rmul(b2[c], uo[c]), ac::rmul(a2u[c], dpx));
        }
        const int rr = tfs ? r + 1 : r;
        T zm[4], z0[4], z1[4], z2[4], wo[4];
        ld4(SP + (rr - 1) * BOXX + b, zm);
        ld4(SP + rr * BOXX + b, z0);
        ld4(SP + (rr + 1) * BOXX + b, z1);
        ld4(SP + (rr + 2) * BOXX + b, z2);
        ld4(W + (rr + 2) * BOXX + b, wo);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const T dpz = ac::radd(ac::rmul(g.c1, ac::rsub(z1[c], z0[c])), ac::rmul(g.c2, ac::rsub(z2[c], zm[c])));
          wn[c] = ac::rsub(ac::rmul(b3[c], wo[c]), ac::rmul(a2w[c], dpz));
        }
        T pv[4] = {ss[4], ss[5], ss[6], ss[7]};
        st4(a.o0 + so + ot, pv);
        st4(a.o1 + so + ot, un);
        st4(a.o2 + so + ot, wn);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if ((twin >> c) & 1u) {
            accp[c] += pv[c] * pv[c];
            accu[c] += un[c] * un[c];
          }
        }
      }
      // a receiver tile's item goes through the relay lanes, which record it from the stores
      mbar_arrive(recording && re_ > rb ? &h->stored[st] : &h->empty[st]);
      sel ^= 1;
    }
    if (a.acc0 != nullptr && twin) {
      st4(a.acc0 + go + ot, accp);
      if (a.accum_u) st4(a.acc1 + go + ot, accu);
    }
  }
}


// ---------------------------------------------------------------------------- adjoint
// Vectorised reverse step: the same transposed update as adj_step_tma, organised like
// fwd_step_vec (one consumer group per block, four adjacent columns per task, register
// coefficients). Stage: lambda_u (19-row box), lambda_w (22), lambda_p (19), forward p after
// the step (19), forward divergence of the step (19). Per item:
//   A  (738 tasks, <= 3 per thread): q_u = -alpha2 lambda_u and q_w = -alpha2 lambda_w on the
//      whole box (masked alpha2, zero outside the u / w regions);
//   B  (180 threads, 2 halo rows x 4 columns): lambda_p before the transposed p update,
//      its free-surface folds, dL/d alpha1 at the tile cells, the new lambda_p of the tile
//      and q_p = -alpha1 lambda_p on the halo;
//   C  (256 threads, 1 tile row x 4 columns): the new lambda_u / lambda_w and dL/d alpha2;
//   D  (tiles holding the free-surface rows, or receivers of u / w): the new tile passes through
//      shared memory (lambda_u / lambda_w in the space of q_u / q_w, dead after B), where the
//      dL/d records of step it-1 are injected and the free-surface fold of lambda_w applied,
//      before the stores.
// Tiles whose receivers record p only take the ordinary path: the consumers arrive on the
// stage's `stored` mbarrier, and the relay lanes of the producer warp add the dL/d p-records
// to the stored lambda_p (a read-modify-write of the item's own output, in the order the
// shared-memory path adds them) and release the stage.
#ifndef ADFWI_VEC_ADJ_MINB
#define ADFWI_VEC_ADJ_MINB 3
#endif
constexpr int VAMINB = ADFWI_VEC_ADJ_MINB;
constexpr int QU_TASKS = EZ * CGE;               // 342
constexpr int QW_TASKS = WZ * CGE;               // 396
constexpr int Q_TASKS = QU_TASKS + QW_TASKS;     // 738
constexpr int Q_ROUNDS = (Q_TASKS + VG - 1) / VG;  // 3

template <typename T>
struct VecAdjLayout {
  static constexpr int kE = round128(EZ * BOXX * (int)sizeof(T));
  static constexpr int kW = round128(WZ * BOXX * (int)sizeof(T));
  static constexpr int kStage = 4 * kE + kW;  // LU, LW, LP, PH, DH boxes
  static constexpr int kStageTx = (4 * EZ + WZ) * BOXX * (int)sizeof(T);
  static constexpr int kSO = round128(TZ * TX * (int)sizeof(T));
  // scratch: QU (EZ rows), QW (WZ rows), QP (EZ rows) in box columns. A receiver /
  // free-surface tile keeps its new lambda_p in the stage's DH box (each cell overwrites its
  // own, already consumed, divergence) and its new lambda_u / lambda_w in the QU / QW space
  // (dead after B); such a tile releases its stage only after D.
  static constexpr int kScratch = kE + kW + kE;
  static_assert(2 * kSO <= kE + kW, "OU and OW fit in the QU / QW space");
  static int bytes(int stages) { return kVecSmemFixed + stages * kStage + kScratch; }
};

// An adjoint tile whose outputs pass through shared memory (phase D).
template <typename T>
__device__ __forceinline__ bool adj_smem_tile(const ac::Geo<T>& g, const StepArgs<T>& a, int tile) {
  const int i0 = g.zbeg + (tile / g.tiles_x) * TZ;
  const bool rcv = g.tile_cell_beg[tile + 1] > g.tile_cell_beg[tile];
  return (g.fsurf && i0 <= g.fs && g.fs - 1 <= i0 + TZ - 1) || (rcv && (a.rec_u != nullptr || a.rec_w != nullptr));
}
// An adjoint tile whose dL/d p-records the relay lanes inject.
template <typename T>
__device__ __forceinline__ bool adj_relay_tile(const ac::Geo<T>& g, const StepArgs<T>& a, int tile) {
  return a.it >= 1 && a.rec_p != nullptr && g.tile_cell_beg[tile + 1] > g.tile_cell_beg[tile] &&
         !adj_smem_tile(g, a, tile);
}

template <typename T, int MB>
__global__ void __launch_bounds__(VTHREADS, MB)
    adj_step_vec(const __grid_constant__ Maps maps, ac::Geo<T> g, StepArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = aligned_smem128(smem_raw);
  using LY = VecAdjLayout<T>;
  const int S = a.stages;
  SmemHeader* h = reinterpret_cast<SmemHeader*>(smem);
  ItemHeader<T>* ih = reinterpret_cast<ItemHeader<T>*>(smem + 512);
  unsigned char* stage0 = smem + 1024;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], VG);
      mbar_init(&h->stored[s], VG);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  griddep_launch_dependents();
  griddep_wait();
  const int nunits = a.ntiles * a.ngroups;
  const int per = (nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(nunits, u_beg + per);

  if (warp == VG / 32) {
    if (lane == 0) {
      const int ymap[5][3] = {{0, -1, 0},
                              {1, -3, LY::kE},
                              {2, -1, LY::kE + LY::kW},
                              {3, -1, 2 * LY::kE + LY::kW},
                              {4, -1, 3 * LY::kE + LY::kW}};
      produce<T, 5>(maps, g, a, h, ih, stage0, LY::kStage, LY::kStageTx, ymap, u_beg, u_end, false);
    } else if (a.it >= 1 && a.rec_p != nullptr) {
      // dL/d p-records of step it-1 enter lambda_p after step it-1 (acoustic_kernels.py:167-169),
      // added to the item's stored lambda_p. A lane keeps its receiver cells cb + lane - 1 + 31 m
      // (m < RC) with their receiver for the unit and issues every load of an item before its
      // arithmetic, so that an item costs the relay one round trip (the relay paces the
      // receiver tiles' blocks: work added here lengthens the launch). Cells with several
      // receivers, and tiles of more than 31 RC receiver cells, walk the tables per item.
      const Layout L = g.L;
      int64_t coff[RC] = {};
      int rid[RC] = {}, cn = 0, cb = 0, ce = 0, i0 = 0, j0 = 0;
      bool walk = false;
      const T gmul = ac::fused_scale(g);
      relay(g, a, h, u_beg, u_end, lane, [&](int tile) { return adj_relay_tile(g, a, tile); },
            [&](int tile) {
              cb = g.tile_cell_beg[tile];
              ce = g.tile_cell_beg[tile + 1];
              i0 = g.zbeg + (tile / g.tiles_x) * TZ;
              j0 = (tile % g.tiles_x) * TX;
              cn = 0;
              walk = ce - cb > 31 * RC;
#pragma unroll
              for (int m = 0; m < RC; ++m) {
                const int q = cb + lane - 1 + 31 * m;
                if (q < ce) {
                  const int cell = g.tcell_cell[q], m0 = g.tcell_rbeg[q];
                  coff[m] = L.off(i0 + (cell >> 16), j0 + (cell & 0xffff));
                  rid[m] = g.cell_rcv[m0];
                  if (g.tcell_rbeg[q + 1] - m0 != 1) walk = true;
                  cn = m + 1;
                }
              }
            },
            [&](int tile, int sh) {
              const int64_t so = (int64_t)sh * L.plane;
              if (!walk) {
                ac::RecPIn<T> in[RC];
                T o[RC];
#pragma unroll
                for (int m = 0; m < RC; ++m)
                  if (m < cn) {
                    in[m] = ac::grad_rec_p_load(g, a.rec_p, sh, a.it - 1, rid[m]);
                    o[m] = a.o0[so + coff[m]];
                  }
#pragma unroll
                for (int m = 0; m < RC; ++m)
                  if (m < cn) {
                    T ap = T(0);
                    ap += ac::grad_rec_p_value(g, in[m], a.it - 1, gmul);
                    a.o0[so + coff[m]] = o[m] + ap;
                  }
              } else {
                for (int q = cb + lane - 1; q < ce; q += 31) {
                  const int cell = g.tcell_cell[q];
                  T ap = T(0);
                  for (int mm = g.tcell_rbeg[q]; mm < g.tcell_rbeg[q + 1]; ++mm)
                    ap += ac::grad_rec_p(g, a.rec_p, sh, a.it - 1, g.cell_rcv[mm], gmul);
                  T* o = a.o0 + so + L.off(i0 + (cell >> 16), j0 + (cell & 0xffff));
                  *o = *o + ap;
                }
              }
            });
    }
    return;
  }

  constexpr int bar = 1;
  const int gt = tid;
  unsigned char* scr = stage0 + S * LY::kStage;
  T* QU = reinterpret_cast<T*>(scr);
  T* QW = reinterpret_cast<T*>(scr + LY::kE);
  T* QP = reinterpret_cast<T*>(scr + LY::kE + LY::kW);
  T* OU = QU;  // reuses the q_u / q_w space
  T* OW = reinterpret_cast<T*>(scr + LY::kSO);
  const Layout L = g.L;
  const int64_t PL = L.plane;

  const bool has_ext = gt < EXT_TASKS;
  const int erp = gt / CGE, ecg = gt - erp * CGE;
  const int tli = gt / CGT, tcg = gt - tli * CGT;

  unsigned evalid[2];      // halo cells inside the grid (and at or below zbeg)
  int ekind[2];            // 0: ordinary row, 1: row fs-1 (no sensitivity), 2: row fs+1 (fold of fs-1), -1: none
  unsigned tin = 0, tu = 0, tw = 0;  // tile cells inside the grid / the u region / the w region
  bool trow = false, special = false;
  int prev_tile = -1, k = 0;

  for (int un = u_beg; un < u_end; ++un) {
    const int sgrp = un / a.ntiles, tile = un - sgrp * a.ntiles;
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    const int s_beg = g.grp_beg[sgrp], s_end = g.grp_beg[sgrp + 1];
    const T* cf = a.cf + (int64_t)g.grp_model[sgrp] * a.cf_stride;
    const int cb = g.tile_cell_beg[tile], ce = g.tile_cell_beg[tile + 1];
    if (tile != prev_tile) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int r = 2 * erp + q;
        ekind[q] = -1;
        evalid[q] = 0;
        if (!has_ext || r >= EZ) continue;
        const int i = i0 - 1 + r, jb = j0 - 4 + 4 * ecg;
        ekind[q] = (g.fsurf && i == g.fs - 1) ? 1 : ((g.fsurf && i == g.fs + 1 && r >= 2) ? 2 : 0);
#pragma unroll
        for (int c = 0; c < 4; ++c)
          if (i >= g.zbeg && i < L.nzp && jb + c >= 0 && jb + c < L.nxp) evalid[q] |= 1u << c;
      }
      {
        const int i = i0 + tli, jb = j0 + 4 * tcg;
        trow = i < L.nzp;
        tin = tu = tw = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int j = jb + c;
          if (trow && j < L.nxp) {
            tin |= 1u << c;
            if (ac::in_u(g, i, j)) tu |= 1u << c;
            if (ac::in_w(g, i, j)) tw |= 1u << c;
          }
        }
      }
      special = adj_smem_tile(g, a, tile);
      prev_tile = tile;
    }
    const int64_t go = (int64_t)sgrp * PL;
    // the unit's gradient partials continue the partial planes' running sums
    T ag1[2][4], ag2[4];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int c = 0; c < 4; ++c) ag1[q][c] = T(0);
#pragma unroll
    for (int c = 0; c < 4; ++c) ag2[c] = T(0);
    const bool ext_tile_col = has_ext && ecg >= 1 && ecg <= CGT;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int r = 2 * erp + q;
      if (ext_tile_col && r >= 1 && r <= TZ && i0 - 1 + r < L.nzp)
        ld4(a.acc0 + go + L.off(i0 - 1 + r, j0 - 4 + 4 * ecg), ag1[q]);
    }
    if (trow) ld4(a.acc1 + go + L.off(i0 + tli, j0 + 4 * tcg), ag2);
    const bool inject = a.it >= 1 && (a.rec_p != nullptr || a.rec_u != nullptr || a.rec_w != nullptr) && ce > cb;
    for (int sh = s_beg; sh < s_end; ++sh, ++k) {
      const int st = k % S;
      // the coefficients of A (re-read per item through the read-only path, so they need no
      // registers across items) are requested before the stage wait
      T cq[Q_ROUNDS][4];
#pragma unroll
      for (int q = 0; q < Q_ROUNDS; ++q) {
        const int t = gt + q * VG;
        if (t < QU_TASKS) {
          const int r = t / CGE, cg = t - r * CGE;
          ldg4(cf + ac::kA2U * PL + L.off(i0 - 1 + r, j0 - 4 + 4 * cg), cq[q]);
        } else if (t < Q_TASKS) {
          const int tt = t - QU_TASKS, r = tt / CGE, cg = tt - r * CGE;
          ldg4(cf + ac::kA2W * PL + L.off(i0 - 3 + r, j0 - 4 + 4 * cg), cq[q]);
        }
      }
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
      T* OP = const_cast<T*>(DH);  // new lambda_p of a special tile, at the cell's own DH slot
      const int64_t so = (int64_t)sh * PL;
      // ---- A: q_u, q_w
      if (ready) {
#pragma unroll
        for (int q = 0; q < Q_ROUNDS; ++q) {
          const int t = gt + q * VG;
          if (t < Q_TASKS) {
            const bool isu = t < QU_TASKS;
            const int tt = isu ? t : t - QU_TASKS, r = tt / CGE, cg = tt - r * CGE;
            const int o = r * BOXX + 4 * cg;
            T x[4];
            ld4((isu ? LU : LW) + o, x);
#pragma unroll
            for (int c = 0; c < 4; ++c) x[c] = -cq[q][c] * x[c];
            st4((isu ? QU : QW) + o, x);
          }
        }
      }
      named_sync(bar, VG);
      // ---- B: lambda_p, dL/d alpha1, q_p
      if (ready && has_ext) {
        auto lp_mid = [&](int r, T (&out)[4]) {
          T qu[12], w0[4], w1[4], w2[4], w3[4], lp[4];
          ld12(QU + r * BOXX + 4 * ecg - 4, qu);
          const T* qw = QW + r * BOXX + 4 * ecg;
          ld4(qw, w0);
          ld4(qw + BOXX, w1);
          ld4(qw + 2 * BOXX, w2);
          ld4(qw + 3 * BOXX, w3);
          ld4(LP + r * BOXX + 4 * ecg, lp);
#pragma unroll
          for (int c = 0; c < 4; ++c)
            out[c] = lp[c] + g.c1 * (qu[3 + c] - qu[4 + c]) + g.c2 * (qu[2 + c] - qu[5 + c]) +
                     g.c1 * (w1[c] - w2[c]) + g.c2 * (w0[c] - w3[c]);
        };
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int kind = ekind[q];
          if (kind < 0) continue;
          const int r = 2 * erp + q;
          const int64_t oc = L.off(i0 - 1 + r, j0 - 4 + 4 * ecg);
          T ca1[4], cb1[4];
          ldg4(cf + ac::kA1M * PL + oc, ca1);
          ldg4(cf + ac::kB1 * PL + oc, cb1);
          T v[4] = {T(0), T(0), T(0), T(0)};
          if (kind != 1) {  // the mirrored row fs-1 carries no sensitivity
            lp_mid(r, v);
            if (kind == 2) {  // adjoint of p[fs-1] = -p[fs+1]
              T m2[4];
              lp_mid(r - 2, m2);
#pragma unroll
              for (int c = 0; c < 4; ++c) v[c] -= m2[c];
            }
          }
#pragma unroll
          for (int c = 0; c < 4; ++c)
            if (!((evalid[q] >> c) & 1u)) v[c] = T(0);
          if (r >= 1 && r <= TZ && ecg >= 1 && ecg <= CGT) {
            T dh[4], lpo[4];
            ld4(DH + r * BOXX + 4 * ecg, dh);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              lpo[c] = cb1[c] * v[c];
              if ((evalid[q] >> c) & 1u) ag1[q][c] -= v[c] * dh[c];
            }
            if (special)
              st4(OP + r * BOXX + 4 * ecg, lpo);
            else if (i0 - 1 + r < L.nzp)
              st4(a.o0 + so + L.off(i0 - 1 + r, j0 - 4 + 4 * ecg), lpo);
          }
          T qp[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) qp[c] = -ca1[c] * v[c];
          st4(QP + r * BOXX + 4 * ecg, qp);
        }
      }
      named_sync(bar, VG);
      // ---- C: lambda_u, lambda_w, dL/d alpha2
      if (ready && trow) {
        const int r = tli + 1, b = 4 * tcg + 4;
        T lu[4], lw[4], luo[4], lwo[4], b2[4], b3[4];
        {
          const int64_t oc = L.off(i0 + tli, j0 + 4 * tcg);
          ldg4(cf + ac::kB2 * PL + oc, b2);
          ldg4(cf + ac::kB3 * PL + oc, b3);
        }
        ld4(LU + r * BOXX + b, lu);
        ld4(LW + (r + 2) * BOXX + b, lw);
        {
          // transposes of the p update's differences of u and w (acoustic_kernels.py:119-126)
          T qh[12], qz[4], qz1[4], qz2[4];
          ld12(QP + r * BOXX + b - 4, qh);
          ld4(QP + (r - 1) * BOXX + b, qz);
          ld4(QP + (r + 1) * BOXX + b, qz1);
          ld4(QP + (r + 2) * BOXX + b, qz2);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            luo[c] = b2[c] * lu[c] + g.c1 * (qh[4 + c] - qh[5 + c]) + g.c2 * (qh[3 + c] - qh[6 + c]);
            lwo[c] = b3[c] * lw[c] + g.c1 * (qh[4 + c] - qz1[c]) + g.c2 * (qz[c] - qz2[c]);
            if (!((tin >> c) & 1u)) luo[c] = lwo[c] = T(0);
          }
        }
        {
          T ph[12], pz[4], pz1[4], pz2[4];
          ld12(PH + r * BOXX + b - 4, ph);
          ld4(PH + (r - 1) * BOXX + b, pz);
          ld4(PH + (r + 1) * BOXX + b, pz1);
          ld4(PH + (r + 2) * BOXX + b, pz2);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if ((tu >> c) & 1u) ag2[c] -= lu[c] * (g.c1 * (ph[5 + c] - ph[4 + c]) + g.c2 * (ph[6 + c] - ph[3 + c]));
            if ((tw >> c) & 1u) ag2[c] -= lw[c] * (g.c1 * (pz1[c] - ph[4 + c]) + g.c2 * (pz2[c] - pz[c]));
          }
        }
        if (special) {
          st4(OU + tli * TX + 4 * tcg, luo);
          st4(OW + tli * TX + 4 * tcg, lwo);
        } else {
          const int64_t o = so + L.off(i0 + tli, j0 + 4 * tcg);
          st4(a.o1 + o, luo);
          st4(a.o2 + o, lwo);
        }
      }
      // an ordinary tile that injects (p receivers only: adj_relay_tile) hands the item to the relay
      if (!special) mbar_arrive(inject ? &h->stored[st] : &h->empty[st]);
      // ---- D: tiles with receivers or the free-surface rows
      if (special) {
        named_sync(bar, VG);
        if (ready && inject && gt < 32) {
          // dL/d records of step it-1 enter the state after step it-1 (acoustic_kernels.py:167-169)
          const int64_t rowbase = ((int64_t)sh * g.nt + (a.it - 1)) * g.nr;
          for (int q = cb + lane; q < ce; q += 32) {
            const int cell = g.tcell_cell[q];
            const int ci = cell >> 16, cj = cell & 0xffff;
            T ap = T(0), au = T(0), aw = T(0);
            for (int mm = g.tcell_rbeg[q]; mm < g.tcell_rbeg[q + 1]; ++mm) {
              const int64_t o = rowbase + g.cell_rcv[mm];
              if (a.rec_p) ap += ac::grad_rec_p(g, a.rec_p, sh, a.it - 1, g.cell_rcv[mm], ac::fused_scale(g));
              if (a.rec_u) au += a.rec_u[o];
              if (a.rec_w) aw += a.rec_w[o];
            }
            OP[(ci + 1) * BOXX + cj + 4] += ap;
            OU[ci * TX + cj] += au;
            OW[ci * TX + cj] += aw;
          }
        }
        named_sync(bar, VG);
        if (ready && trow) {
          const int i = i0 + tli;
          T op[4], ou[4], ow[4];
          ld4(OP + (tli + 1) * BOXX + 4 * tcg + 4, op);
          ld4(OU + tli * TX + 4 * tcg, ou);
          ld4(OW + tli * TX + 4 * tcg, ow);
          if (g.fsurf && i == g.fs - 1) {  // adjoint of w[fs-1] = w[fs]
#pragma unroll
            for (int c = 0; c < 4; ++c) ow[c] = T(0);
          }
          if (g.fsurf && i == g.fs && tli >= 1) {
            T up[4];
            ld4(OW + (tli - 1) * TX + 4 * tcg, up);
#pragma unroll
            for (int c = 0; c < 4; ++c) ow[c] += up[c];
          }
#pragma unroll
          for (int c = 0; c < 4; ++c)
            if (!((tin >> c) & 1u)) op[c] = ou[c] = ow[c] = T(0);
          const int64_t o = so + L.off(i, j0 + 4 * tcg);
          st4(a.o0 + o, op);
          st4(a.o1 + o, ou);
          st4(a.o2 + o, ow);
        }
        mbar_arrive(&h->empty[st]);  // OP (in the DH box) is read
        named_sync(bar, VG);  // OU / OW are read before the next item's A rewrites q_u / q_w
      }
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int r = 2 * erp + q;
      if (ext_tile_col && r >= 1 && r <= TZ && i0 - 1 + r < L.nzp)
        st4(a.acc0 + go + L.off(i0 - 1 + r, j0 - 4 + 4 * ecg), ag1[q]);
    }
    if (trow) st4(a.acc1 + go + L.off(i0 + tli, j0 + 4 * tcg), ag2);
  }
}

}  // namespace ac2
}  // namespace adfwi
