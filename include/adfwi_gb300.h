/*
 * adfwi_gb300 -- C ABI of the GB300 (sm_103a) propagator hot path of ADFWI.
 *
 * Every entry point is stream-ordered on the caller's CUDA stream, allocates no
 * device memory (the caller passes a workspace whose size the library reports),
 * returns 0 on success or a negative status, and records a message retrievable
 * with adfwi_last_error(). Device arrays are dense row-major; `dtype` selects
 * float32 or float64 for every floating-point array of a call.
 *
 * Reference interfaces replaced (paths inside liufeng2317/ADFWI):
 *   acoustic: ADFWI/propagator/acoustic_kernels.py:179 forward_kernel(...) as called from
 *             ADFWI/propagator/acoustic_propagator.py:147-156, plus the autograd backward
 *             through torch.utils.checkpoint at acoustic_kernels.py:268-278;
 *   elastic:  ADFWI/propagator/elastic_kernels.py:917 forward_kernel(...) as called from
 *             ADFWI/propagator/elastic_propagator.py:132-141, plus its autograd backward
 *             (elastic_kernels.py:975-1008).
 */
#ifndef ADFWI_GB300_H
#define ADFWI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADFWI_F32 0
#define ADFWI_F64 1

/* Storage of the checkpoint snapshots kept for the gradient (stencils stay in dtype). */
#define ADFWI_SNAP_NATIVE 0 /* same type as the wavefields */
#define ADFWI_SNAP_BF16 1   /* bfloat16 with one max-abs scale per snapshot, shot and field */
#define ADFWI_SNAP_FP16 2   /* float16 with one max-abs scale per snapshot, shot and field */
#define ADFWI_SNAP_FP24 3   /* float32 rounded to a 15-bit mantissa, 3 bytes per value, no scale */

/* adfwi_acoustic_desc.snapshot_every: boundary saving instead of snapshots. The forward keeps
 * p, u, w of the absorbing frame (every cell outside the damping-free interior of the model)
 * after every step; the adjoint rebuilds the interior states backwards by inverting the update
 * and restores the frame. Replaces the reference's planned boundary-saving time step
 * (ADFWI/propagator/acoustic_kernels_bs.py:40-54, 202-313); the damping must vanish in the
 * model's interior (true of the reference's PML, Gerjan and sin^2 frames). Single-model plans
 * only. The backward rebuilds the states in the workspace it was given, consuming the forward's
 * last state: run the forward again before another backward. */
#define ADFWI_SNAP_EVERY_BOUNDARY (-1)

/* Status codes. */
#define ADFWI_OK 0
#define ADFWI_ERR_ARGUMENT (-1)
#define ADFWI_ERR_GEOMETRY (-2)
#define ADFWI_ERR_WORKSPACE (-3)
#define ADFWI_ERR_CUDA (-4)
#define ADFWI_ERR_UNSUPPORTED (-5)

/* ------------------------------------------------------------------------- */
/* Acoustic (p, u, w) 4th-order staggered grid with PML damping.              */
/* ------------------------------------------------------------------------- */

typedef struct adfwi_acoustic_desc {
  int32_t nz, nx;             /* model cells before padding                                  */
  int32_t nabc;               /* absorbing cells on every side (grid = nz+2nabc x nx+2nabc)  */
  int32_t free_surface;       /* 0 / 1                                                       */
  int32_t ns;                 /* shots of this solve (one source each)                       */
  int32_t nt;                 /* time steps                                                  */
  int32_t nr;                 /* receivers, shared by all shots                              */
  int32_t dtype;              /* ADFWI_F32 / ADFWI_F64                                       */
  int32_t checkpoint_segments;/* reference chunk count; only shapes forward_wavefield_u/w    */
  int32_t snapshot_every;     /* steps between snapshots for the gradient; 0 = automatic;    */
                              /* ADFWI_SNAP_EVERY_BOUNDARY = boundary saving                 */
  int32_t snapshot_precision; /* ADFWI_SNAP_*                                                */
  int32_t shots_per_block;    /* shots handled by one thread block; 0 = automatic            */
  double dt;                  /* time step (s)                                               */
  int64_t memory_budget;      /* byte cap for the gradient workspace; 0 = no cap             */
  int32_t ring_depth;         /* TMA ring of the step kernels: 0 = automatic, 1 = shallow    */
                              /* (3 blocks / SM), 2 = deep (2 blocks / SM, one stage more);  */
                              /* results do not depend on it                                 */
  int32_t reserved;           /* 0                                                           */
} adfwi_acoustic_desc;

typedef struct adfwi_acoustic_plan adfwi_acoustic_plan; /* opaque */

/* Build a plan from the descriptor and HOST arrays of grid coordinates in model cells
 * (before padding): src_z/src_x (ns), rcv_z/rcv_x (nr). Replaces the geometry handling of
 * acoustic_propagator.py:84-99 and the "+nabc" index shift of acoustic_kernels.py:233-237. */
int adfwi_acoustic_plan_create(const adfwi_acoustic_desc* desc, const int32_t* src_z,
                               const int32_t* src_x, const int32_t* rcv_z,
                               const int32_t* rcv_x, adfwi_acoustic_plan** plan);
void adfwi_acoustic_plan_destroy(adfwi_acoustic_plan* plan);

/* Batched plan: `nmodels` velocity models of one grid shape solved in the same launches (no
 * counterpart in the reference, whose propagator solves one model per call; this is what the
 * continuous-batching server packs requests into). shot_model (HOST, ns) gives each shot's
 * model, non-decreasing, every model with at least one shot; receivers are shared. The
 * forward / backward of a batched plan take alpha1, alpha2, damp as (nmodels, nz+2nabc,
 * nx+2nabc) arrays, write fw_p/u/w as (nmodels, nz, nx) and grad_alpha1/2 as (nmodels,
 * nz+2nabc, nx+2nabc); records stay (ns, nt, nr) in shot order. Per shot the arithmetic is
 * that of a single-model plan. */
int adfwi_acoustic_plan_create_batched(const adfwi_acoustic_desc* desc, const int32_t* src_z,
                                       const int32_t* src_x, const int32_t* rcv_z,
                                       const int32_t* rcv_x, int32_t nmodels,
                                       const int32_t* shot_model, adfwi_acoustic_plan** plan);
/* Models of a plan (1 for adfwi_acoustic_plan_create). */
int32_t adfwi_acoustic_plan_models(const adfwi_acoustic_plan* plan);

/* Workspace bytes for a forward solve (with_gradient = 0) or for a forward solve that keeps
 * what adfwi_acoustic_backward needs (with_gradient = 1). Used for HBM-budget admission. */
int adfwi_acoustic_workspace_bytes(const adfwi_acoustic_plan* plan, int32_t with_gradient,
                                   int64_t* bytes);

/* Segment length (steps between snapshots) the plan uses in gradient mode. */
int adfwi_acoustic_snapshot_every(const adfwi_acoustic_plan* plan, int32_t* steps);

/* Forward solve: replaces forward_kernel (acoustic_kernels.py:179-301).
 *   alpha1 = rho c^2 dt/dz, alpha2 = dt/(rho dz), damp: (nz+2nabc, nx+2nabc)
 *   wavelet: (ns, nt); rec_p/u/w: (ns, nt, nr) outputs;
 *   fw_p/u/w: (nz, nx) outputs (forward_wavefield_* of the reference, with its
 *   accumulation order), any of them may be NULL.
 * With with_gradient = 1 the workspace keeps the snapshots for adjoint_acoustic_backward. */
int adfwi_acoustic_forward(const adfwi_acoustic_plan* plan, const void* alpha1, const void* alpha2,
                           const void* damp, const void* wavelet, void* rec_p, void* rec_u,
                           void* rec_w, void* fw_p, void* fw_u, void* fw_w, int32_t with_gradient,
                           void* workspace, int64_t workspace_bytes, void* stream);

/* Adjoint (reverse-time) solve after a with_gradient forward on the same workspace and the
 * same coefficients: replaces the autograd backward through acoustic_kernels.py:268-278.
 * grad_rec_*: dL/d rec_* (ns, nt, nr), NULL means zero. Outputs dL/d alpha1 and
 * dL/d alpha2 (nz+2nabc, nx+2nabc), overwritten. */
int adfwi_acoustic_backward(const adfwi_acoustic_plan* plan, const void* alpha1,
                            const void* alpha2, const void* damp, const void* wavelet,
                            const void* grad_rec_p, const void* grad_rec_u,
                            const void* grad_rec_w, void* grad_alpha1, void* grad_alpha2,
                            void* workspace, int64_t workspace_bytes, void* stream);

/* The normalised L2 misfit on a plan's records: replaces the reference's misfit evaluation
 * ADFWI/fwi/misfit/L2.py:26-29 on the traces normalised at ADFWI/fwi/acoustic_fwi.py:149-150
 * and the hand-off of its autograd gradient to the propagator's backward.
 * adfwi_acoustic_l2_loss, after a with_gradient forward on the workspace: syn = the forward's
 * p records, obs (ns, nt, nr); writes each model's loss (nmodels device doubles; the misfit of
 * adfwi_l2_misfit, same flags and silent_rel, dt of the plan) and keeps the per-trace factors in
 * the workspace. Then either
 *   adfwi_acoustic_l2_sources writes the adjoint source times *grad_scale (one device double;
 *   exactly the unscaled source when it is 1) into adj (ns, nt, nr), for
 *   adfwi_acoustic_backward's grad_rec_p; or
 *   adfwi_acoustic_backward_l2 runs the adjoint with that source formed inside the adjoint step
 *   as it is injected (no (ns, nt, nr) array; slower per step on GB300, where the extra work
 *   lands on the lanes that inject the receivers),
 * giving dL/d alpha1 and dL/d alpha2 like adfwi_acoustic_backward. The source values of both are
 * bit-identical to adfwi_l2_misfit's adj. */
int adfwi_acoustic_l2_loss(const adfwi_acoustic_plan* plan, const void* syn, const void* obs,
                           double silent_rel, int32_t flags, double* loss, void* workspace,
                           int64_t workspace_bytes, void* stream);
int adfwi_acoustic_l2_sources(const adfwi_acoustic_plan* plan, const void* syn, const void* obs,
                              int32_t flags, const double* grad_scale, void* adj, void* workspace,
                              int64_t workspace_bytes, void* stream);
int adfwi_acoustic_backward_l2(const adfwi_acoustic_plan* plan, const void* wavelet, const void* syn,
                               const void* obs, int32_t flags, const double* grad_scale,
                               void* grad_alpha1, void* grad_alpha2, void* workspace,
                               int64_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* Elastic velocity-stress (vx, vz, txx, tzz, txz), 4th / 6th order staggered grid. */
/* ------------------------------------------------------------------------- */

typedef struct adfwi_elastic_desc {
  int32_t nz, nx;             /* model cells before padding                                     */
  int32_t nabc;               /* absorbing cells (left, right, bottom; top too without a free surface) */
  int32_t free_surface;       /* 0 / 1                                                          */
  int32_t ns, nt, nr;         /* shots, time steps, receivers                                   */
  int32_t dtype;              /* ADFWI_F32 / ADFWI_F64                                          */
  int32_t fd_order;           /* 4 or 6                                                         */
  int32_t pml;                /* 1: split-field PML (bcx, bcz); 0: multiplicative layer (damp)  */
  int32_t checkpoint_segments;/* reference chunk count; shapes the forward_wavefield_* maps      */
  int32_t snapshot_every;     /* steps between gradient snapshots; 0 = automatic                */
  int32_t snapshot_precision; /* ADFWI_SNAP_*                                                   */
  int32_t reserved;
  double dt, dx, dz;
  double fdc[3];              /* staggered coefficients (DiffCoef, float32-rounded), fd_order/2 used */
  int64_t memory_budget;      /* byte cap for the gradient workspace; 0 = no cap                */
} adfwi_elastic_desc;

typedef struct adfwi_elastic_plan adfwi_elastic_plan; /* opaque */

/* Plan from HOST geometry in model cells (before padding) and the moment tensors (ns x 3 x 3,
 * row-major doubles). Replaces elastic_propagator.py:81-96 and elastic_kernels.py:955-959. */
int adfwi_elastic_plan_create(const adfwi_elastic_desc* desc, const int32_t* src_z,
                              const int32_t* src_x, const int32_t* rcv_z, const int32_t* rcv_x,
                              const double* moment_tensor, adfwi_elastic_plan** plan);
void adfwi_elastic_plan_destroy(adfwi_elastic_plan* plan);
int adfwi_elastic_workspace_bytes(const adfwi_elastic_plan* plan, int32_t with_gradient,
                                  int64_t* bytes);
int adfwi_elastic_snapshot_every(const adfwi_elastic_plan* plan, int32_t* steps);

/* Forward solve: replaces elastic_kernels.py:917-1037 forward_kernel.
 * coef[10] = padded C11, C13, C15, C33, C35, C55, bx, bz, bcx, bcz (pml = 1) or
 * coef[9] = ... bx, bz, damp (pml = 0), each dense with its own padded shape given in
 * shapes[2*q], shapes[2*q+1] (the reference's padding keeps bx (nz, nx-1), bz (nz-1, nx) and
 * C55 (nz-2, nx-2) smaller). wavelet: (ns, nt). rec: 5 x (ns, nt, nr) for txx, tzz, txz, vx, vz.
 * fw: 5 x (nz, nx) forward_wavefield_* maps, or NULL. */
int adfwi_elastic_forward(const adfwi_elastic_plan* plan, const void* const* coef,
                          const int32_t* shapes, const void* wavelet, void* rec, void* fw,
                          int32_t with_gradient, void* workspace, int64_t workspace_bytes,
                          void* stream);

/* Adjoint solve after a with_gradient forward on the same workspace: replaces the autograd
 * backward through elastic_kernels.py:975-1008. grad_rec: 5 x (ns, nt, nr) or NULL.
 * grad_coef[8]: outputs dL/d(C11, C13, C15, C33, C35, C55, bx, bz) with the shapes of the
 * first 8 coefficient inputs (entries may be NULL). */
int adfwi_elastic_backward(const adfwi_elastic_plan* plan, const void* wavelet,
                           const void* grad_rec, void* const* grad_coef, const int32_t* shapes,
                           void* workspace, int64_t workspace_bytes, void* stream);

/* Device status of the last solve run in `workspace` (same with_gradient as that solve):
 * 0 = clean, 1 = a bounded pipeline wait inside a kernel ran out (results invalid).
 * Waits for the stream. */
int adfwi_acoustic_status(const adfwi_acoustic_plan* plan, const void* workspace,
                          int64_t workspace_bytes, int32_t with_gradient, int32_t* status,
                          void* stream);

/* Self-test of the bounded waits behind adfwi_acoustic_status (no reference counterpart: the
 * reference's PyTorch loop has no device-side waits). One block waits, through the pipelined
 * kernels' wait loop, on an mbarrier phase that nothing completes; after limit_ns (at most 2 s)
 * it gives up, writes 1 (wait timed out) to the DEVICE int *flag and exits, leaving the context
 * usable. Stream-ordered; the caller zeroes *flag first. */
int adfwi_wait_selftest(int64_t limit_ns, int32_t* flag, void* stream);

/* ------------------------------------------------------------------------- */
/* Normalised L2 trace misfit and its adjoint source.                          */
/* ------------------------------------------------------------------------- */

/* Workspace bytes of adfwi_l2_misfit for ns shots and nr receivers. */
int adfwi_l2_misfit_workspace_bytes(int32_t dtype, int32_t ns, int32_t nr, int64_t* bytes);

/* loss = sum over traces (s, r) of sqrt(sum_t (obs/max|obs| - syn/max|syn|)^2 dt) and
 * adj = dL/dsyn, for records syn, obs of shape (ns, nt, nr). Replaces the reference's
 * misfit evaluation ADFWI/fwi/misfit/L2.py:26-29 on the traces normalised at
 * ADFWI/fwi/acoustic_fwi.py:149-150, and its autograd backward. `loss` is ONE device double;
 * every sum is FP64 in a fixed order (deterministic). flags bit 0: normalise obs (else obs is
 * used as given). Traces whose peak is at most silent_rel times their gather's peak count as
 * zero (silent_rel = 0 keeps the reference's rule, under which an all-zero trace divides by
 * zero). Stream-ordered; allocates nothing. */
int adfwi_l2_misfit(int32_t dtype, int32_t ns, int32_t nt, int32_t nr, double dt, double silent_rel,
                    int32_t flags, const void* syn, const void* obs, void* adj, double* loss,
                    void* workspace, int64_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* Gaussian smoothing of model planes (gradient processor).                    */
/* ------------------------------------------------------------------------- */

/* Workspace bytes of adfwi_smooth2d for an (nz, nx) plane. */
int adfwi_smooth2d_workspace_bytes(int32_t nz, int32_t nx, int32_t span, int64_t* bytes);

/* out = smooth2d(in, span) of ADFWI/propagator/gradient_process.py:32-49 (used by
 * GradProcessor.forward, 91-134): 'same'-size convolution of the FP64 (nz, nx) plane `in` with a
 * normalised Gaussian of standard deviation `span` sampled every 2 cells over [-2 span,
 * 2 span], divided by the convolution of a plane of ones. Device arrays; stream-ordered;
 * allocates nothing. */
int adfwi_smooth2d(int32_t nz, int32_t nx, int32_t span, const double* in, double* out, void* workspace,
                   int64_t workspace_bytes, void* stream);

/* Forward solve that allocates nothing, for callers that cannot call cudaMalloc: hosts whose
 * device memory is entirely owned by another allocator or pool, sandboxed plug-ins that may
 * not grow their footprint after start-up, or code running where an allocation would break
 * a pre-planned memory budget. It has no counterpart in the reference (whose PyTorch path
 * allocates through the caching allocator on every step).
 * Same arguments and results as adfwi_acoustic_forward without the gradient mode and
 * without the workspace: the scratch is a static device array of 64 MiB inside the
 * library, reserved on every GPU that loads the library until the process exits. A solve
 * whose scratch (adfwi_acoustic_workspace_bytes(plan, 0, ...)) exceeds 64 MiB is rejected
 * with ADFWI_ERR_WORKSPACE and a message. The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) on that device; make that first call
 * before any stream capture. All calls share the one array and it keeps the last call's
 * contents: the call clears what it accumulates into, but two calls whose work overlaps on
 * the GPU (for example on two streams) race on it and must be serialised by the caller. */
int adfwi_acoustic_forward_noalloc(const adfwi_acoustic_plan* plan, const void* alpha1,
                                   const void* alpha2, const void* damp, const void* wavelet,
                                   void* rec_p, void* rec_u, void* rec_w, void* fw_p, void* fw_u,
                                   void* fw_w, void* stream);

/* Device status of the last adfwi_acoustic_forward_noalloc call made with `plan` on the
 * current device: 0 = clean, 1 = a bounded pipeline wait inside a kernel ran out (the records
 * and wavefields of that call are invalid). The allocation-free forward keeps its error flag in
 * the library's static scratch array, whose address callers never see, so this is the way to
 * read it (the counterpart of adfwi_acoustic_status for workspace solves). Waits for the
 * stream; a later allocation-free call on the device overwrites the flag. */
int adfwi_acoustic_noalloc_status(const adfwi_acoustic_plan* plan, int32_t* status, void* stream);

/* ------------------------------------------------------------------------- */
/* Errors and build information.                                             */
/* ------------------------------------------------------------------------- */

/* Launch accounting and per-kernel-class device time (used by the benchmark's roofline).
 * adfwi_profile_start resets the session counters; with timed = 1 every launch of the library
 * is bracketed by CUDA events on its stream until adfwi_profile_stop, which waits for the
 * events and fills up to max_out entries (one per kernel class that launched). */
typedef struct adfwi_kernel_stat {
  char name[32];
  int64_t launches;
  int64_t timed_launches;
  double total_ms;
} adfwi_kernel_stat;
int adfwi_profile_start(int32_t timed);
int adfwi_profile_stop(adfwi_kernel_stat* out, int32_t max_out, int32_t* n_out);
/* Cumulative number of kernel launches issued by this library in this process. */
int64_t adfwi_launch_count(void);

/* Copy the calling thread's last error message into buf (NUL-terminated); returns its length. */
int adfwi_last_error(char* buf, size_t n);

/* Library version string. */
const char* adfwi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* ADFWI_GB300_H */
