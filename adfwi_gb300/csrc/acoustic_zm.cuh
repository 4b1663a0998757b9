// Z-streamed acoustic forward step (included by acoustic.cu after acoustic_tma.cuh).
//
// A unit of work is a column strip of 120 grid columns x a range [z0, z1) of rows x a group of
// G shots. A block marches down the strip's rows, one shot after the other: per step it takes a
// chunk of R = 8 new rows of u, w and p (TMA boxes 136 columns wide, columns j0-8 .. j0+127,
// into a ring of NCH chunks), computes the new pressure on the 8 rows that the chunk completes
// (one row per consumer warp, four adjacent columns per lane, columns j0-4 .. j0+123) into a
// ring of p rows, and then the new u and w three rows further up, where the new pressure
// rows above and below are already in the ring. Every input row crosses HBM once per unit and
// no row is recomputed (a tile of a 2-D decomposition re-reads and recomputes its halo rows):
//
//   step s (chunk rows rb = z0-8+8s .. rb+7 just landed):
//     p pass   rows rb-1 .. rb+6 (warp w: row rb-1+w)  needs w rows up to rb+7, u / p rows rb-1..
//     barrier
//     u/w pass rows rb-4 .. rb+3 (warp w: row rb-4+w) needs new p rows up to rb+5
//     release chunk s-1 (its last rows were read by this step for the last time)
//
// Step 0 only loads (rows z0-8 .. z0-1: the stencil halo above the range); the last step
// reaches row z1-1 of the u/w pass. The ring holds the chunks s-1 and s being read while the
// next ones are in flight. Lanes 1 .. 30 own the strip's 120 output columns; lanes 0 and 31
// compute the pressure of the strip's halo columns (j0-4 .. j0-1, j0+120 .. j0+123).
//
// Receivers are recorded by the warp that finishes their row (the row's receiver list in
// the strip, read back from the p ring and the global u / w stores); the illumination sums
// are read-modify-writes of the unit's shot-group partial planes (one warp per row for
// every shot of the group, so the order of the sums is fixed).
//
// The operation order of every cell value is the reference's (acoustic_kernels.py:115-160),
// with explicitly rounded arithmetic, as in fwd_step_vec: records are bit-identical.
#pragma once

namespace adfwi {
namespace zm {

using ac2::aborted;
using ac2::ld12;
using ac2::ld4;
using ac2::ldg4;
using ac2::st4;

constexpr int SW = 120;           // output columns of a strip
constexpr int BW = 136;           // staged row: columns j0-8 .. j0+127
constexpr int R = 8;              // rows per step = consumer warps
constexpr int PR = 32;            // rows of the new-p ring
constexpr int CG = 32 * R;        // consumer threads
constexpr int THREADS = CG + 32;  // + the producer warp
static_assert(PR >= 16 && (PR & (PR - 1)) == 0, "p ring: a power of two of at least two steps");

template <typename T>
struct FwdLayout {
  static constexpr int kNch = sizeof(T) == 8 ? 3 : 6;  // chunks of the input ring
  static constexpr int kRow = BW * (int)sizeof(T);
  static constexpr int kField = R * kRow;
  static constexpr int kChunk = 3 * kField;  // u, w, p
  static constexpr int kRing = kNch * kChunk;
  static constexpr int kP = PR * kRow;
  static int bytes() { return 1024 + 128 + kRing + kP; }
};

struct Units {
  int nstrips, nzr, lz, G, ngroups, nunits;
  const int* rrow_beg;  // per strip: nzp+1 offsets of its receiver rows into rcol / rid
  const int* rcol;      // receiver column within the strip (0 .. SW-1)
  const int* rid;       // receiver index
};

struct UnitPos {
  int strip, j0, z0, z1, s_beg, s_end, S;
};

template <typename T>
__device__ __forceinline__ UnitPos unit_pos(const ac::Geo<T>& g, const Units& U, int un) {
  UnitPos p;
  const int zr = un % U.nzr, t = un / U.nzr;
  p.strip = t % U.nstrips;
  const int grp = t / U.nstrips;
  p.j0 = p.strip * SW;
  p.z0 = g.zbeg + zr * U.lz;
  p.z1 = min(g.L.nzp, p.z0 + U.lz);
  p.s_beg = grp * U.G;
  p.s_end = min(g.ns, p.s_beg + U.G);
  p.S = (p.z1 - p.z0 + 4 + R - 1) / R;  // steps with work; chunks = S + 1
  return p;
}

// Producer lane: the chunks of every (unit, shot) of the block in order.
template <typename T>
__device__ __forceinline__ void zm_produce(const ac2::Maps& maps, const ac::Geo<T>& g, const Units& U,
                                           const ac2::StepArgs<T>& a, ac2::SmemHeader* h, unsigned char* ring,
                                           int u_beg, int u_end) {
  using LY = FwdLayout<T>;
  constexpr int NCH = LY::kNch;
  prefetch_tensormap(&maps.a);
  prefetch_tensormap(&maps.b);
  prefetch_tensormap(&maps.c);
  int k = 0;
  bool stop = false;
  for (int un = u_beg; un < u_end && !stop; ++un) {
    const UnitPos P = unit_pos(g, U, un);
    for (int sh = P.s_beg; sh < P.s_end && !stop; ++sh) {
      for (int c = 0; c <= P.S; ++c, ++k) {
        const int slot = k % NCH;
        if (aborted(h) || (k >= NCH && !mbar_wait(&h->empty[slot], ((k / NCH) - 1) & 1))) {
          ac2::set_abort(h, a.flag);
          stop = true;
          break;
        }
        unsigned char* sb = ring + slot * LY::kChunk;
        mbar_arrive_expect_tx(&h->full[slot], LY::kChunk);
        const int x = P.j0 - 8 + GX, y = P.z0 - R + R * c + GZ;
        tma_load_3d(sb, &maps.a, x, y, sh, &h->full[slot]);
        tma_load_3d(sb + LY::kField, &maps.b, x, y, sh, &h->full[slot]);
        tma_load_3d(sb + 2 * LY::kField, &maps.c, x, y, sh, &h->full[slot]);
      }
    }
  }
  // do not leave the block while a load it issued may still be landing
  for (int q = max(0, k - NCH); q < k; ++q) mbar_wait(&h->full[q % NCH], (q / NCH) & 1);
}

#ifndef ADFWI_ZM_MINB
#define ADFWI_ZM_MINB 2
#endif
// Every global value a step reads besides the staged rows (the coefficients of the warp's rows
// and the illumination partials) is loaded one step ahead, right after its previous use, so
// no step waits on an L2 round trip.
template <typename T>
__global__ void __launch_bounds__(THREADS, ADFWI_ZM_MINB)
    fwd_zmarch(const __grid_constant__ ac2::Maps maps, ac::Geo<T> g, ac2::StepArgs<T> a, Units U) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = ac2::aligned_smem128(smem_raw);
  using LY = FwdLayout<T>;
  constexpr int NCH = LY::kNch;
  ac2::SmemHeader* h = reinterpret_cast<ac2::SmemHeader*>(smem);
  unsigned char* ring = smem + 1024;
  T* PRING = reinterpret_cast<T*>(ring + LY::kRing);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < NCH; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], R);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  griddep_launch_dependents();
  griddep_wait();
  const int per = (U.nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(U.nunits, u_beg + per);

  if (warp == R) {
    if (lane == 0) zm_produce<T>(maps, g, U, a, h, ring, u_beg, u_end);
    return;
  }

  const Layout L = g.L;
  const int64_t PL = L.plane;
  const T* cf = a.cf;
  const bool own = lane >= 1 && lane <= 30;  // lane owns output columns of the strip
  const bool recording = a.rec_p != nullptr;
  constexpr int bar = 1;
  int k = 0;
  for (int un = u_beg; un < u_end; ++un) {
    const UnitPos P = unit_pos(g, U, un);
    const int jb = P.j0 - 4 + 4 * lane;  // this lane's four columns
    const int64_t go = (int64_t)(un / U.nzr / U.nstrips) * PL;
    unsigned win = 0, pin_cols = 0;  // columns in the illumination window / in the p region's x range
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = jb + c;
      if (j >= g.nabc && j < g.nabc + g.nx) win |= 1u << c;
      if (j >= 2 && j <= L.nxp - 3) pin_cols |= 1u << c;
    }
    // rows of this warp in step s: p pass z0-9+8s+warp, u/w pass z0-12+8s+warp
    auto p_row = [&](int s) { return P.z0 - R - 1 + R * s + warp; };
    auto u_row = [&](int s) { return P.z0 - R - 4 + R * s + warp; };
    auto p_eval = [&](int i) { return (g.fsurf && i == g.fs - 1) ? i + 2 : i; };  // p[fs-1] = -p[fs+1]
    auto w_eval = [&](int i) { return (g.fsurf && i == g.fs - 1) ? g.fs : i; };   // w[fs-1] = w[fs]
    auto illum_row = [&](int i) { return own && win && i >= P.z0 && i < P.z1 && i >= g.nabc && i < g.nabc + g.nz; };
    // values of the warp's rows of the next step, loaded one step ahead
    T ca[4], cb[4], a2u[4], b2[4], a2w[4], b3[4], accp[4], accu[4];
    auto fetch = [&](int s) {
      const int ip = p_row(s), iu = u_row(s);
      if (ip >= P.z0 - 1) {
        const int64_t oc = L.off(p_eval(ip), jb);
        ldg4(cf + ac::kA1M * PL + oc, ca);
        ldg4(cf + ac::kB1 * PL + oc, cb);
        if (a.acc0 != nullptr && illum_row(ip)) ld4(a.acc0 + go + L.off(ip, jb), accp);
      }
      if (own && iu >= P.z0 && iu < P.z1) {
        ldg4(cf + ac::kA2U * PL + L.off(iu, jb), a2u);
        ldg4(cf + ac::kB2 * PL + L.off(iu, jb), b2);
        ldg4(cf + ac::kA2W * PL + L.off(w_eval(iu), jb), a2w);
        ldg4(cf + ac::kB3 * PL + L.off(w_eval(iu), jb), b3);
        if (a.accum_u && a.acc1 != nullptr && illum_row(iu)) ld4(a.acc1 + go + L.off(iu, jb), accu);
      }
    };
    for (int sh = P.s_beg; sh < P.s_end; ++sh) {
      const int kbase = k;
      const int sz = g.src_z[sh], sx = g.src_x[sh];
      const T sval = ac::rmul(g.dt, a.wav[(int64_t)sh * g.nt + a.it]);
      const int64_t so = (int64_t)sh * PL;
      // staged row r (grid row) of field f of this z-march
      auto srow = [&](int f, int r) -> const T* {
        const int q = r - (P.z0 - R);
        const int slot = (kbase + q / R) % NCH;
        return reinterpret_cast<const T*>(ring + slot * LY::kChunk + f * LY::kField + (q % R) * LY::kRow);
      };
      auto prow = [&](int r) -> T* { return PRING + ((r + 4 * PR) & (PR - 1)) * BW; };
      for (int s = 0; s <= P.S; ++s, ++k) {
        const int slot = k % NCH;
        if (s == 0) fetch(1);
        bool ready = !aborted(h);
        if (ready && !mbar_wait(&h->full[slot], (k / NCH) & 1)) {
          ac2::set_abort(h, a.flag);
          ready = false;
        }
        if (s == 0) {
          // the halo chunk above the range: nothing completes yet. The barrier keeps a warp that
          // starts this z-march from writing p-ring rows that a slower warp still reads in the
          // last step of the previous one.
          named_sync(bar, CG);
          continue;
        }
        const bool more = s < P.S;
        // ---- p pass: new pressure on row z0-9+8s+warp
        {
          const int i = p_row(s);
          if (ready && i >= P.z0 - 1) {
            const bool mir = g.fsurf && i == g.fs - 1;
            const int re = p_eval(i);
            T uu[12], w0[4], w1[4], w2[4], w3[4], pp[4];
            ld12(srow(0, re) + 4 * lane, uu);
            ld4(srow(1, re - 2) + 4 + 4 * lane, w0);
            ld4(srow(1, re - 1) + 4 + 4 * lane, w1);
            ld4(srow(1, re) + 4 + 4 * lane, w2);
            ld4(srow(1, re + 1) + 4 + 4 * lane, w3);
            ld4(srow(2, re) + 4 + 4 * lane, pp);
            T dv[4], v[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              // divergence in the reference's operation order (acoustic_kernels.py:118-127)
              const T t1 = ac::rsub(ac::radd(ac::rsub(uu[4 + c], uu[3 + c]), w2[c]), w1[c]);
              const T t2 = ac::rsub(ac::radd(ac::rsub(uu[5 + c], uu[2 + c]), w3[c]), w0[c]);
              dv[c] = ac::radd(ac::rmul(g.c1, t1), ac::rmul(g.c2, t2));
              v[c] = ac::rsub(ac::rmul(cb[c], pp[c]), ac::rmul(ca[c], dv[c]));
            }
            if (sz == re) {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (sx == jb + c) v[c] = ac::radd(v[c], sval);
            }
            if (mir) {
#pragma unroll
              for (int c = 0; c < 4; ++c) v[c] = -v[c];
            }
            st4(prow(i) + 4 + 4 * lane, v);
            if (own && i >= P.z0 && i < P.z1) {
              const int64_t o = so + L.off(i, jb);
              st4(a.o0 + o, v);
              if (a.d1 != nullptr) {
                const bool prow_in = i >= g.fs + 1 && i <= L.nzp - 3;
                T dd[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) dd[c] = prow_in && ((pin_cols >> c) & 1u) ? dv[c] : T(0);
                st4(a.d1 + o, dd);
              }
              if (a.acc0 != nullptr && illum_row(i)) {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                  if ((win >> c) & 1u) accp[c] += v[c] * v[c];
                st4(a.acc0 + go + L.off(i, jb), accp);
              }
            }
          }
          // the next step's p-pass values (the registers are free now)
          if (more) {
            const int in_ = p_row(s + 1);
            if (in_ >= P.z0 - 1) {
              const int64_t oc = L.off(p_eval(in_), jb);
              ldg4(cf + ac::kA1M * PL + oc, ca);
              ldg4(cf + ac::kB1 * PL + oc, cb);
              if (a.acc0 != nullptr && illum_row(in_)) ld4(a.acc0 + go + L.off(in_, jb), accp);
            }
          }
        }
        named_sync(bar, CG);
        // ---- u / w pass: new u and w on row z0-12+8s+warp
        {
          const int i = u_row(s);
          if (ready && own && i >= P.z0 && i < P.z1) {
            const int ie = w_eval(i);
            T ss[12], uo[4], un_[4], wn[4];
            ld12(prow(i) + 4 * lane, ss);
            ld4(srow(0, i) + 4 + 4 * lane, uo);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const T dpx = ac::radd(ac::rmul(g.c1, ac::rsub(ss[5 + c], ss[4 + c])),
                                     ac::rmul(g.c2, ac::rsub(ss[6 + c], ss[3 + c])));
              un_[c] = ac::rsub(ac::rmul(b2[c], uo[c]), ac::rmul(a2u[c], dpx));
            }
            T zm_[4], z0[4], z1[4], z2[4], wo[4];
            ld4(prow(ie - 1) + 4 + 4 * lane, zm_);
            ld4(prow(ie) + 4 + 4 * lane, z0);
            ld4(prow(ie + 1) + 4 + 4 * lane, z1);
            ld4(prow(ie + 2) + 4 + 4 * lane, z2);
            ld4(srow(1, ie) + 4 + 4 * lane, wo);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              const T dpz = ac::radd(ac::rmul(g.c1, ac::rsub(z1[c], z0[c])), ac::rmul(g.c2, ac::rsub(z2[c], zm_[c])));
              wn[c] = ac::rsub(ac::rmul(b3[c], wo[c]), ac::rmul(a2w[c], dpz));
            }
            const int64_t o = so + L.off(i, jb);
            st4(a.o1 + o, un_);
            st4(a.o2 + o, wn);
            if (a.accum_u && a.acc1 != nullptr && illum_row(i)) {
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if ((win >> c) & 1u) accu[c] += un_[c] * un_[c];
              st4(a.acc1 + go + L.off(i, jb), accu);
            }
          }
          // records of step it at this row (acoustic_kernels.py:167-169)
          if (ready && recording && i >= P.z0 && i < P.z1) {
            const int* rb_ = U.rrow_beg + (int64_t)P.strip * (L.nzp + 1);
            const int q0 = rb_[i], q1 = rb_[i + 1];
            if (q1 > q0) {
              __syncwarp();  // the row's u / w stores of the other lanes are visible
              const int64_t rowbase = ((int64_t)sh * g.nt + a.it) * g.nr;
              T* rp = const_cast<T*>(a.rec_p);
              T* ru = const_cast<T*>(a.rec_u);
              T* rw = const_cast<T*>(a.rec_w);
              const T* pr = prow(i);
              for (int q = q0 + lane; q < q1; q += 32) {
                const int c = U.rcol[q], id = U.rid[q];
                const int64_t o = so + L.off(i, P.j0 + c);
                rp[rowbase + id] = pr[c + 8];
                ru[rowbase + id] = a.o1[o];
                rw[rowbase + id] = a.o2[o];
              }
            }
          }
          if (more) {
            const int in_ = u_row(s + 1);
            if (own && in_ >= P.z0 && in_ < P.z1) {
              ldg4(cf + ac::kA2U * PL + L.off(in_, jb), a2u);
              ldg4(cf + ac::kB2 * PL + L.off(in_, jb), b2);
              ldg4(cf + ac::kA2W * PL + L.off(w_eval(in_), jb), a2w);
              ldg4(cf + ac::kB3 * PL + L.off(w_eval(in_), jb), b3);
              if (a.accum_u && a.acc1 != nullptr && illum_row(in_)) ld4(a.acc1 + go + L.off(in_, jb), accu);
            }
          }
        }
        // chunk s-1 is read for the last time by this step
        __syncwarp();
        if (lane == 0) mbar_arrive(&h->empty[(kbase + s - 1) % NCH]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&h->empty[(kbase + P.S) % NCH]);
    }
  }
}

// ================================================================================ adjoint
// Z-streamed reverse step: the exact transpose of fwd_zmarch's step (and of adj_step_vec), on
// the same strips. Staged per chunk: lambda_u, lambda_w after the step and the forward pressure
// after the step; lambda_p after the step and the forward divergence of the step are read
// pointwise, one step ahead like the coefficients. Per step s:
//
//   q pass   rows rb .. rb+7 (the chunk's rows): q_u = -alpha2 lambda_u, q_w = -alpha2 lambda_w
//   barrier
//   v pass   rows rb-1 .. rb+6: v = lambda_p + transposed x / z differences of q_u (this row)
//            and q_w (rows i-2 .. i+1), with the free-surface folds; dL/d alpha1 -= v x
//            divergence; the new lambda_p = (1 - kappa1) v; q_p = -alpha1 v into the q_p ring
//   barrier
//   u/w pass rows rb-4 .. rb+3: new lambda_u / lambda_w from q_p (rows i-1 .. i+2) and
//            dL/d alpha2 -= lambda_u Dx(p) + lambda_w Dz(p) from the staged forward pressure
//
// Step 0 runs the q pass of the halo chunk only. dL/d records of step it-1 enter the new state
// after the stores of the row that holds them (one lane per receiver cell, several receivers of
// a cell summed in receiver order). The coefficient-gradient partials are read-modify-writes of
// the unit's shot-group planes.
template <typename T>
struct AdjLayout {
  static constexpr int kNch = sizeof(T) == 8 ? 3 : 5;
  static constexpr int kRow = BW * (int)sizeof(T);
  static constexpr int kField = R * kRow;
  static constexpr int kChunk = 3 * kField;  // lambda_u, lambda_w, p
  static constexpr int kRing = kNch * kChunk;
  static constexpr int kQ = 16 * kRow;       // q_u or q_w ring (16 rows)
  static constexpr int kQP = PR * kRow;      // q_p ring
  static int bytes() { return 1024 + 128 + kRing + 2 * kQ + kQP; }
};

template <typename T>
__device__ __forceinline__ void zm_produce_adj(const ac2::Maps& maps, const ac::Geo<T>& g, const Units& U,
                                               const ac2::StepArgs<T>& a, ac2::SmemHeader* h, unsigned char* ring,
                                               int u_beg, int u_end) {
  using LY = AdjLayout<T>;
  constexpr int NCH = LY::kNch;
  prefetch_tensormap(&maps.a);
  prefetch_tensormap(&maps.b);
  prefetch_tensormap(&maps.c);
  int k = 0;
  bool stop = false;
  for (int un = u_beg; un < u_end && !stop; ++un) {
    const UnitPos P = unit_pos(g, U, un);
    for (int sh = P.s_beg; sh < P.s_end && !stop; ++sh) {
      for (int c = 0; c <= P.S; ++c, ++k) {
        const int slot = k % NCH;
        if (aborted(h) || (k >= NCH && !mbar_wait(&h->empty[slot], ((k / NCH) - 1) & 1))) {
          ac2::set_abort(h, a.flag);
          stop = true;
          break;
        }
        unsigned char* sb = ring + slot * LY::kChunk;
        mbar_arrive_expect_tx(&h->full[slot], LY::kChunk);
        const int x = P.j0 - 8 + GX, y = P.z0 - R + R * c + GZ;
        tma_load_3d(sb, &maps.a, x, y, sh, &h->full[slot]);
        tma_load_3d(sb + LY::kField, &maps.b, x, y, sh, &h->full[slot]);
        tma_load_3d(sb + 2 * LY::kField, &maps.c, x, y, sh, &h->full[slot]);
      }
    }
  }
  for (int q = max(0, k - NCH); q < k; ++q) mbar_wait(&h->full[q % NCH], (q / NCH) & 1);
}

#ifndef ADFWI_ZM_ADJ_MINB
#define ADFWI_ZM_ADJ_MINB 2
#endif
template <typename T>
__global__ void __launch_bounds__(THREADS, ADFWI_ZM_ADJ_MINB)
    adj_zmarch(const __grid_constant__ ac2::Maps maps, ac::Geo<T> g, ac2::StepArgs<T> a, Units U,
               const T* __restrict__ lp_in, const T* __restrict__ dh_in) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = ac2::aligned_smem128(smem_raw);
  using LY = AdjLayout<T>;
  constexpr int NCH = LY::kNch;
  enum { LU = 0, LW = 1, PH = 2 };
  ac2::SmemHeader* h = reinterpret_cast<ac2::SmemHeader*>(smem);
  unsigned char* ring = smem + 1024;
  T* QU = reinterpret_cast<T*>(ring + LY::kRing);
  T* QW = reinterpret_cast<T*>(ring + LY::kRing + LY::kQ);
  T* QP = reinterpret_cast<T*>(ring + LY::kRing + 2 * LY::kQ);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < NCH; ++s) {
      mbar_init(&h->full[s], 1);
      mbar_init(&h->empty[s], R);
    }
    h->abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  griddep_launch_dependents();
  griddep_wait();
  const int per = (U.nunits + gridDim.x - 1) / gridDim.x;
  const int u_beg = blockIdx.x * per, u_end = min(U.nunits, u_beg + per);

  if (warp == R) {
    if (lane == 0) zm_produce_adj<T>(maps, g, U, a, h, ring, u_beg, u_end);
    return;
  }

  const Layout L = g.L;
  const int64_t PL = L.plane;
  const T* cf = a.cf;
  const bool own = lane >= 1 && lane <= 30;
  const bool inject = a.it >= 1 && (a.rec_p != nullptr || a.rec_u != nullptr || a.rec_w != nullptr);
  constexpr int bar = 1;
  auto q16 = [&](T* base, int r) -> T* { return base + ((r + 64) & 15) * BW; };
  auto qprow = [&](int r) -> T* { return QP + ((r + 4 * PR) & (PR - 1)) * BW; };
  int k = 0;
  for (int un = u_beg; un < u_end; ++un) {
    const UnitPos P = unit_pos(g, U, un);
    const int jb = P.j0 - 4 + 4 * lane;
    const int64_t go = (int64_t)(un / U.nzr / U.nstrips) * PL;
    unsigned cin = 0;  // this lane's columns inside the grid
#pragma unroll
    for (int c = 0; c < 4; ++c)
      if (jb + c >= 0 && jb + c < L.nxp) cin |= 1u << c;
    auto q_row = [&](int s) { return P.z0 - R + R * s + warp; };
    auto v_row = [&](int s) { return P.z0 - R - 1 + R * s + warp; };
    auto u_row = [&](int s) { return P.z0 - R - 4 + R * s + warp; };
    // values of the warp's rows of the next step, loaded one step ahead
    T a2u[4], a2w[4], ca1[4], cb1[4], lpv[4], dhv[4], acc1v[4], b2[4], b3[4], acc2v[4];
    for (int sh = P.s_beg; sh < P.s_end; ++sh) {
      const int kbase = k;
      const int64_t so = (int64_t)sh * PL;
      const int64_t rowbase = ((int64_t)sh * g.nt + (a.it - 1)) * g.nr;
      auto srow = [&](int f, int r) -> const T* {
        const int q = r - (P.z0 - R);
        const int slot = (kbase + q / R) % NCH;
        return reinterpret_cast<const T*>(ring + slot * LY::kChunk + f * LY::kField + (q % R) * LY::kRow);
      };
      auto fetch_q = [&](int s) {
        const int r = q_row(s);
        ldg4(cf + ac::kA2U * PL + L.off(r, jb), a2u);
        ldg4(cf + ac::kA2W * PL + L.off(r, jb), a2w);
      };
      auto fetch_v = [&](int s) {
        const int i = v_row(s);
        if (i >= P.z0 - 1) {
          const int64_t oc = L.off(i, jb);
          ldg4(cf + ac::kA1M * PL + oc, ca1);
          ldg4(cf + ac::kB1 * PL + oc, cb1);
          ldg4(lp_in + so + oc, lpv);
          if (own && i >= P.z0 && i < P.z1) {
            ldg4(dh_in + so + oc, dhv);
            ld4(a.acc0 + go + oc, acc1v);
          }
        }
      };
      auto fetch_u = [&](int s) {
        const int i = u_row(s);
        if (own && i >= P.z0 && i < P.z1) {
          const int64_t oc = L.off(i, jb);
          ldg4(cf + ac::kB2 * PL + oc, b2);
          ldg4(cf + ac::kB3 * PL + oc, b3);
          ld4(a.acc1 + go + oc, acc2v);
        }
      };
      // v = lambda_p + transposed differences of q_u / q_w at row r (acoustic_kernels.py:115-127)
      auto lp_mid = [&](int r, const T (&lp)[4], T (&out)[4]) {
        T qu[12], w0[4], w1[4], w2[4], w3[4];
        ld12(q16(QU, r) + 4 * lane, qu);
        ld4(q16(QW, r - 2) + 4 + 4 * lane, w0);
        ld4(q16(QW, r - 1) + 4 + 4 * lane, w1);
        ld4(q16(QW, r) + 4 + 4 * lane, w2);
        ld4(q16(QW, r + 1) + 4 + 4 * lane, w3);
#pragma unroll
        for (int c = 0; c < 4; ++c)
          out[c] = lp[c] + g.c1 * (qu[3 + c] - qu[4 + c]) + g.c2 * (qu[2 + c] - qu[5 + c]) + g.c1 * (w1[c] - w2[c]) +
                   g.c2 * (w0[c] - w3[c]);
      };
      // dL/d records of step it-1 at row i, added to the stored state of the row (one lane per
      // receiver cell; the entries of a cell are consecutive)
      auto inject_row = [&](int i, const T* rec, T* field) {
        const int* rb_ = U.rrow_beg + (int64_t)P.strip * (L.nzp + 1);
        const int q0 = rb_[i], q1 = rb_[i + 1];
        if (q1 <= q0) return;
        __syncwarp();
        for (int q = q0 + lane; q < q1; q += 32) {
          const int c = U.rcol[q];
          if (q > q0 && U.rcol[q - 1] == c) continue;  // not the cell's first entry
          T add = T(0);
          for (int m = q; m < q1 && U.rcol[m] == c; ++m) add += rec[rowbase + U.rid[m]];
          T* o = field + so + L.off(i, P.j0 + c);
          *o = *o + add;
        }
        __syncwarp();
      };
      fetch_q(0);
      fetch_v(1);
      fetch_u(1);
      for (int s = 0; s <= P.S; ++s, ++k) {
        const int slot = k % NCH;
        bool ready = !aborted(h);
        if (ready && !mbar_wait(&h->full[slot], (k / NCH) & 1)) {
          ac2::set_abort(h, a.flag);
          ready = false;
        }
        const bool more = s < P.S;
        // ---- q pass: the chunk's rows
        {
          const int r = q_row(s);
          if (ready) {
            T lu[4], lw[4], qu[4], qw[4];
            ld4(srow(LU, r) + 4 + 4 * lane, lu);
            ld4(srow(LW, r) + 4 + 4 * lane, lw);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              qu[c] = -a2u[c] * lu[c];
              qw[c] = -a2w[c] * lw[c];
            }
            st4(q16(QU, r) + 4 + 4 * lane, qu);
            st4(q16(QW, r) + 4 + 4 * lane, qw);
          }
          if (more) fetch_q(s + 1);
        }
        named_sync(bar, CG);
        if (s == 0) continue;  // the halo chunk: q rows only
        // ---- v pass
        {
          const int i = v_row(s);
          if (ready && i >= P.z0 - 1) {
            const int kind = (g.fsurf && i == g.fs - 1) ? 1 : ((g.fsurf && i == g.fs + 1) ? 2 : 0);
            T v[4] = {T(0), T(0), T(0), T(0)};
            if (kind != 1) {  // the mirrored row fs-1 carries no sensitivity
              lp_mid(i, lpv, v);
              if (kind == 2) {  // adjoint of p[fs-1] = -p[fs+1]
                T lpm[4], m2[4];
                ldg4(lp_in + so + L.off(i - 2, jb), lpm);
                lp_mid(i - 2, lpm, m2);
#pragma unroll
                for (int c = 0; c < 4; ++c) v[c] -= m2[c];
              }
            }
            const bool rin = i >= g.zbeg && i < L.nzp;
#pragma unroll
            for (int c = 0; c < 4; ++c)
              if (!(rin && ((cin >> c) & 1u))) v[c] = T(0);
            if (own && i >= P.z0 && i < P.z1) {
              T lpo[4];
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                lpo[c] = cb1[c] * v[c];
                if (rin && ((cin >> c) & 1u)) acc1v[c] -= v[c] * dhv[c];
              }
              const int64_t oc = L.off(i, jb);
              st4(a.acc0 + go + oc, acc1v);
              st4(a.o0 + so + oc, lpo);
            }
            T qp[4];
#pragma unroll
            for (int c = 0; c < 4; ++c) qp[c] = -ca1[c] * v[c];
            st4(qprow(i) + 4 + 4 * lane, qp);
            if (inject && a.rec_p != nullptr && i >= P.z0 && i < P.z1) inject_row(i, a.rec_p, const_cast<T*>(a.o0));
          }
          if (more) fetch_v(s + 1);
        }
        named_sync(bar, CG);
        // ---- u / w pass
        {
          const int i = u_row(s);
          if (ready && i >= P.z0 && i < P.z1) {
            if (own) {
              unsigned tin = 0, tu = 0, tw = 0;
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                const int j = jb + c;
                if (i < L.nzp && j < L.nxp) {
                  tin |= 1u << c;
                  if (ac::in_u(g, i, j)) tu |= 1u << c;
                  if (ac::in_w(g, i, j)) tw |= 1u << c;
                }
              }
              const int64_t oc = L.off(i, jb);
              T lu[4], lw[4], luo[4], lwo[4];
              ld4(srow(LU, i) + 4 + 4 * lane, lu);
              ld4(srow(LW, i) + 4 + 4 * lane, lw);
              auto lw_new = [&](int r, const T (&b3r)[4], const T (&lwr)[4], T (&out)[4]) {
                T qh[4], qz[4], qz1[4], qz2[4];
                ld4(qprow(r) + 4 + 4 * lane, qh);
                ld4(qprow(r - 1) + 4 + 4 * lane, qz);
                ld4(qprow(r + 1) + 4 + 4 * lane, qz1);
                ld4(qprow(r + 2) + 4 + 4 * lane, qz2);
#pragma unroll
                for (int c = 0; c < 4; ++c) out[c] = b3r[c] * lwr[c] + g.c1 * (qh[c] - qz1[c]) + g.c2 * (qz[c] - qz2[c]);
              };
              {
                // transposes of the p update's differences of u and w (acoustic_kernels.py:119-126)
                T qh[12];
                ld12(qprow(i) + 4 * lane, qh);
#pragma unroll
                for (int c = 0; c < 4; ++c)
                  luo[c] = b2[c] * lu[c] + g.c1 * (qh[4 + c] - qh[5 + c]) + g.c2 * (qh[3 + c] - qh[6 + c]);
                lw_new(i, b3, lw, lwo);
              }
#pragma unroll
              for (int c = 0; c < 4; ++c)
                if (!((tin >> c) & 1u)) luo[c] = lwo[c] = T(0);
              if (g.fsurf && i == g.fs - 1) {  // adjoint of w[fs-1] = w[fs]: row fs-1 hands its share to row fs
#pragma unroll
                for (int c = 0; c < 4; ++c) lwo[c] = T(0);
              }
              if (g.fsurf && i == g.fs) {
                T b3m[4], lwm_in[4], lwm[4];
                ldg4(cf + ac::kB3 * PL + L.off(i - 1, jb), b3m);
                ld4(srow(LW, i - 1) + 4 + 4 * lane, lwm_in);
                lw_new(i - 1, b3m, lwm_in, lwm);
#pragma unroll
                for (int c = 0; c < 4; ++c)
                  if ((tin >> c) & 1u) lwo[c] += lwm[c];
              }
              {
                T ph[12], pz[4], pz1[4], pz2[4];
                ld12(srow(PH, i) + 4 * lane, ph);
                ld4(srow(PH, i - 1) + 4 + 4 * lane, pz);
                ld4(srow(PH, i + 1) + 4 + 4 * lane, pz1);
                ld4(srow(PH, i + 2) + 4 + 4 * lane, pz2);
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                  if ((tu >> c) & 1u) acc2v[c] -= lu[c] * (g.c1 * (ph[5 + c] - ph[4 + c]) + g.c2 * (ph[6 + c] - ph[3 + c]));
                  if ((tw >> c) & 1u) acc2v[c] -= lw[c] * (g.c1 * (pz1[c] - ph[4 + c]) + g.c2 * (pz2[c] - pz[c]));
                }
                st4(a.acc1 + go + oc, acc2v);
              }
              st4(a.o1 + so + oc, luo);
              st4(a.o2 + so + oc, lwo);
            }
            if (inject) {
              if (a.rec_u != nullptr) inject_row(i, a.rec_u, a.o1);
              if (a.rec_w != nullptr) inject_row(i, a.rec_w, a.o2);
            }
          }
          if (more) fetch_u(s + 1);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&h->empty[(kbase + s - 1) % NCH]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&h->empty[(kbase + P.S) % NCH]);
    }
  }
}

}  // namespace zm
}  // namespace adfwi
