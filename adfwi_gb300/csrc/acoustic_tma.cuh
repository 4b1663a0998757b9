// TMA pipeline shared by the acoustic step kernels (included by acoustic.cu; the kernels
// themselves are in acoustic_vec.cuh).
//
// Work of one launch = all (tile, shot) items of one time step. A persistent block owns a
// contiguous range of "units" (one 16 x 64 tile x one group of at most G shots; group-major:
// unit u is tile u mod ntiles of group u / ntiles, so a block walks neighbouring tiles of one
// group and reads their shared halo columns from L2 -- 2 % faster than tile-major on the
// 600 x 1600 grid, the same elsewhere), so every accumulator a unit produces (illumination,
// coefficient gradients) belongs to one block and is flushed once, deterministically, into the
// group's partial plane. The shots of a group
// share one velocity model: a batched plan solves several models of one grid shape in the same
// launches, each with its own coefficient block and its own groups.
//
// Inside a block, one producer warp has one lane issue, per item, the TMA tile loads of
// every wavefield plane the item reads into the next free pipeline stage and arm the stage's
// `full` mbarrier with the byte count (the per-item source cell and amplitude travel in a
// small header written before the arming arrive). The consumer warps wait on `full`,
// compute, and arrive on the stage's `empty` mbarrier once they no longer read it, so the
// loads of the next items overlap the arithmetic of the current one. Items of tiles holding
// receivers go through the producer warp's other 31 lanes (the relay): the consumers arrive
// on the stage's `stored` mbarrier instead, and the relay releases the stage (`empty`) and does
// the receiver work on the item's global outputs, off the consumers' path.
//
// Every wait is bounded (kWaitNs of elapsed time); a wait that runs out raises the device
// error flag and a block-wide abort flag, after which the block skips its remaining work
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
constexpr int MAXSTAGES = 8;

__host__ __device__ constexpr int round128(int bytes) { return (bytes + 127) / 128 * 128; }

template <typename T>
struct ItemHeader {
  int sz, sx;
  T sval;
};

struct SmemHeader {
  uint64_t full[MAXSTAGES];
  uint64_t empty[MAXSTAGES];
  uint64_t stored[MAXSTAGES];  // consumers -> relay lanes: the item's outputs are in global memory
  int abort_flag;
};
static_assert(sizeof(SmemHeader) <= 512, "the item headers start 512 bytes into shared memory");

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
  const T* cf;  // coefficient block of model 0 (masked planes kA1M .. kB3); model m at cf + m * cf_stride
  int64_t cf_stride;
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
    const int grp = un / a.ntiles, tile = un - grp * a.ntiles;
    const int i0 = g.zbeg + (tile / g.tiles_x) * TZ, j0 = (tile % g.tiles_x) * TX;
    const int x = j0 - 4 + GX;
    const int s_beg = g.grp_beg[grp], s_end = g.grp_beg[grp + 1];
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

}  // namespace ac2
}  // namespace adfwi
