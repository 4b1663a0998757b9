"""Acoustic solve: native plan wrapper and the autograd Function around the CUDA library.

``AcousticSolve.apply(alpha1, alpha2, damp, wavelet, plan)`` replaces the reference's
``forward_kernel`` time loop (ADFWI/propagator/acoustic_kernels.py:179-301) and its
autograd backward through ``torch.utils.checkpoint`` (268-278): the forward runs the CUDA
time loop, the backward runs the hand-written adjoint and returns dL/d alpha1 and
dL/d alpha2; PyTorch autograd then carries them through alpha = f(pad(vp), pad(rho)).
"""
import ctypes

import numpy as np
import torch

from . import _native as N

# snapshot_every value of boundary saving: the forward keeps the absorbing frame of every step
# and the adjoint rebuilds the interior states backwards (no snapshots, no recomputation)
BOUNDARY_SAVING = -1

_SNAP = {"native": N.SNAP_NATIVE, "f32": N.SNAP_NATIVE, "fp32": N.SNAP_NATIVE, "float32": N.SNAP_NATIVE,
         "bf16": N.SNAP_BF16, "bfloat16": N.SNAP_BF16, "fp16": N.SNAP_FP16, "float16": N.SNAP_FP16,
         "fp24": N.SNAP_FP24, "f24": N.SNAP_FP24}


def snapshot_code(precision):
    if isinstance(precision, int):
        return precision
    try:
        return _SNAP[str(precision).lower()]
    except KeyError:
        raise ValueError("snapshot precision must be one of native, bf16, fp16, fp24") from None


def dtype_code(dtype):
    if dtype == torch.float32:
        return N.F32
    if dtype == torch.float64:
        return N.F64
    raise ValueError("adfwi_gb300 propagators support float32 and float64, got %s" % dtype)


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).astype(np.int32))


class AcousticPlan(object):
    """Geometry tables and launch configuration of one acoustic solve shape (host object)."""

    def __init__(self, *, nz, nx, nabc, free_surface, src_z, src_x, rcv_z, rcv_x, nt, dt, dtype,
                 checkpoint_segments=1, snapshot_every=0, snapshot_precision="native",
                 shots_per_block=0, memory_budget=0, shot_model=None, ring_depth=0):
        """``shot_model`` (ns ints, non-decreasing) makes a batched plan: several velocity models of
        this grid shape solved in the same launches, shot s on model shot_model[s]; its
        coefficient inputs and its illumination / gradient outputs then carry a leading model
        axis (nmodels, ...)."""
        self.lib = N.lib()
        self.src_z, self.src_x = _i32(src_z), _i32(src_x)
        self.rcv_z, self.rcv_x = _i32(rcv_z), _i32(rcv_x)
        self.ns, self.nr, self.nt = len(self.src_z), len(self.rcv_z), int(nt)
        self.nz, self.nx, self.nabc = int(nz), int(nx), int(nabc)
        self.dtype = dtype
        d = N.AcousticDesc()
        d.nz, d.nx, d.nabc, d.free_surface = self.nz, self.nx, self.nabc, int(bool(free_surface))
        d.ns, d.nt, d.nr, d.dtype = self.ns, self.nt, self.nr, dtype_code(dtype)
        d.checkpoint_segments = int(checkpoint_segments)
        d.snapshot_every = int(snapshot_every or 0)
        d.snapshot_precision = snapshot_code(snapshot_precision)
        d.shots_per_block = int(shots_per_block or 0)
        d.dt = float(dt)
        d.memory_budget = int(memory_budget or 0)
        d.ring_depth = int(ring_depth)
        self.desc = d
        h = ctypes.c_void_p()
        geo = (ctypes.byref(d), self.src_z.ctypes.data_as(ctypes.c_void_p),
               self.src_x.ctypes.data_as(ctypes.c_void_p), self.rcv_z.ctypes.data_as(ctypes.c_void_p),
               self.rcv_x.ctypes.data_as(ctypes.c_void_p))
        if shot_model is None:
            self.nm, self.batched = 1, False
            N.check(self.lib.adfwi_acoustic_plan_create(*geo, ctypes.byref(h)), "adfwi_acoustic_plan_create")
        else:
            sm = _i32(shot_model)
            if len(sm) != self.ns:
                raise ValueError("shot_model has %d entries for %d shots" % (len(sm), self.ns))
            self.nm, self.batched = int(sm.max()) + 1, True
            self._shot_model = sm
            N.check(self.lib.adfwi_acoustic_plan_create_batched(*geo, self.nm, sm.ctypes.data_as(ctypes.c_void_p),
                                                                 ctypes.byref(h)), "adfwi_acoustic_plan_create_batched")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.adfwi_acoustic_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def workspace_bytes(self, with_gradient):
        b = ctypes.c_int64()
        N.check(self.lib.adfwi_acoustic_workspace_bytes(self.handle, int(bool(with_gradient)), ctypes.byref(b)),
                "adfwi_acoustic_workspace_bytes")
        return b.value

    @property
    def snapshot_every(self):
        k = ctypes.c_int32()
        N.check(self.lib.adfwi_acoustic_snapshot_every(self.handle, ctypes.byref(k)), "adfwi_acoustic_snapshot_every")
        return k.value

    def _check(self, t, shape, name):
        if not t.is_cuda:
            raise RuntimeError("%s must be a CUDA tensor (adfwi_gb300 runs on the GPU only)" % name)
        if t.dtype != self.dtype:
            raise TypeError("%s has dtype %s, the plan uses %s" % (name, t.dtype, self.dtype))
        if tuple(t.shape) != tuple(shape):
            raise ValueError("%s has shape %s, expected %s" % (name, tuple(t.shape), tuple(shape)))
        if not t.is_contiguous():
            raise ValueError("%s must be contiguous" % name)

    def grid_shape(self):
        return (self.nz + 2 * self.nabc, self.nx + 2 * self.nabc)

    def check_boundary_saving(self, damp):
        """Boundary saving inverts the update where the damping vanishes: check that ``damp``
        (nzp, nxp) or (nmodels, nzp, nxp) is zero on the plan's rebuilt interior and the one
        cell beyond it that the u / w damping averages in (raises ValueError otherwise)."""
        nzp, nxp = self.grid_shape()
        fs = self.nabc if bool(self.desc.free_surface) else 1
        i_lo, i_hi = max(self.nabc, fs + 1), min(self.nabc + self.nz - 2, nzp - 4)
        j_lo, j_hi = max(self.nabc, 2), min(self.nabc + self.nx - 2, nxp - 4)
        if i_hi < i_lo or j_hi < j_lo:
            return
        inner = damp[..., i_lo:i_hi + 2, j_lo:j_hi + 2]
        if bool((inner != 0).any()):
            raise ValueError("boundary saving needs a damping frame that vanishes inside the model "
                             "(rows %d-%d, columns %d-%d of the padded grid)" % (i_lo, i_hi + 1, j_lo, j_hi + 1))

    def _model_shape(self, shape):
        """Shape of a per-model array: with a leading model axis for a batched plan."""
        return (self.nm,) + tuple(shape) if self.batched else tuple(shape)

    def run_forward(self, alpha1, alpha2, damp, wavelet, with_gradient, workspace=None, records=None,
                    fw=None, stream=None):
        """Run the forward solve; returns (rec_p, rec_u, rec_w, fw_p, fw_u, fw_w, workspace)."""
        g = self._model_shape(self.grid_shape())
        for t, n in ((alpha1, "alpha1"), (alpha2, "alpha2"), (damp, "damp")):
            self._check(t, g, n)
        self._check(wavelet, (self.ns, self.nt), "wavelet")
        dev = alpha1.device
        need = self.workspace_bytes(with_gradient)
        if workspace is None:
            workspace = torch.empty(need, dtype=torch.uint8, device=dev)
        if records is None:
            shp = (self.ns, self.nt, self.nr)
            records = tuple(torch.empty(shp, dtype=self.dtype, device=dev) for _ in range(3)) if self.nr else (None,) * 3
        if fw is None:
            fw = tuple(torch.empty(self._model_shape((self.nz, self.nx)), dtype=self.dtype, device=dev)
                       for _ in range(3))
        st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(dev)
        rc = self.lib.adfwi_acoustic_forward(
            self.handle, N.ptr(alpha1), N.ptr(alpha2), N.ptr(damp), N.ptr(wavelet),
            N.ptr(records[0]), N.ptr(records[1]), N.ptr(records[2]), N.ptr(fw[0]), N.ptr(fw[1]), N.ptr(fw[2]),
            int(bool(with_gradient)), N.ptr(workspace), workspace.numel(), st)
        N.check(rc, "adfwi_acoustic_forward")
        return records + fw + (workspace,)

    def status(self, workspace, with_gradient, stream=None):
        """Device status of the last solve in ``workspace`` (0 = clean); waits for the stream."""
        v = ctypes.c_int32()
        st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(workspace.device)
        N.check(self.lib.adfwi_acoustic_status(self.handle, N.ptr(workspace), workspace.numel(),
                                               int(bool(with_gradient)), ctypes.byref(v), st), "adfwi_acoustic_status")
        return v.value

    def l2_loss(self, syn, obs, workspace, silent_rel=0.0, normalise_obs=False, stream=None):
        """Normalised L2 misfit of the forward's p records ``syn`` against ``obs`` (ns, nt, nr): each
        model's loss as FP64 device values (nmodels,); keeps the per-trace factors in the gradient
        ``workspace`` for l2_sources or run_backward_l2."""
        shp = (self.ns, self.nt, self.nr)
        self._check(syn, shp, "syn")
        obs = obs.to(dtype=self.dtype).contiguous()
        self._check(obs, shp, "obs")
        loss = torch.empty((self.nm,), dtype=torch.float64, device=syn.device)
        st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(syn.device)
        N.check(self.lib.adfwi_acoustic_l2_loss(self.handle, N.ptr(syn), N.ptr(obs), float(silent_rel),
                                                int(bool(normalise_obs)), N.ptr(loss), N.ptr(workspace),
                                                workspace.numel(), st), "adfwi_acoustic_l2_loss")
        return loss

    def l2_sources(self, syn, obs, workspace, grad_scale, normalise_obs=False, adj=None, stream=None):
        """The adjoint source of l2_loss's misfit times ``grad_scale`` (a one-element FP64 device
        tensor) as an (ns, nt, nr) array (``adj`` may name the output buffer), for run_backward's
        p-record gradient."""
        obs = obs.to(dtype=self.dtype).contiguous()
        gs = grad_scale.to(dtype=torch.float64).reshape(1).contiguous()
        if adj is None:
            adj = torch.empty_like(syn)
        self._check(adj, (self.ns, self.nt, self.nr), "adj")
        st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(syn.device)
        N.check(self.lib.adfwi_acoustic_l2_sources(self.handle, N.ptr(syn), N.ptr(obs), int(bool(normalise_obs)),
                                                   N.ptr(gs), N.ptr(adj), N.ptr(workspace), workspace.numel(), st),
                "adfwi_acoustic_l2_sources")
        return adj

    def run_backward_l2(self, alpha1, wavelet, syn, obs, workspace, grad_scale, normalise_obs=False, stream=None):
        """Adjoint solve whose p-record source is the misfit of l2_loss (formed as it is injected)
        times ``grad_scale`` (a one-element FP64 device tensor); returns (dL/d alpha1, dL/d alpha2)."""
        obs = obs.to(dtype=self.dtype).contiguous()
        gs = grad_scale.to(dtype=torch.float64).reshape(1).contiguous()
        ga1 = torch.empty_like(alpha1)
        ga2 = torch.empty_like(alpha1)
        st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(alpha1.device)
        N.check(self.lib.adfwi_acoustic_backward_l2(self.handle, N.ptr(wavelet), N.ptr(syn), N.ptr(obs),
                                                    int(bool(normalise_obs)), N.ptr(gs), N.ptr(ga1), N.ptr(ga2),
                                                    N.ptr(workspace), workspace.numel(), st),
                "adfwi_acoustic_backward_l2")
        return ga1, ga2

    def run_backward(self, alpha1, alpha2, damp, wavelet, grads, workspace, stream=None):
        """Adjoint solve after run_forward(with_gradient=True); returns (dL/d alpha1, dL/d alpha2)."""
        shp = (self.ns, self.nt, self.nr)
        gs = []
        for gr, n in zip(grads, ("grad_rec_p", "grad_rec_u", "grad_rec_w")):
            if gr is not None:
                gr = gr.to(dtype=self.dtype).contiguous()
                self._check(gr, shp, n)
            gs.append(gr)
        ga1 = torch.empty_like(alpha1)
        ga2 = torch.empty_like(alpha2)
        st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(alpha1.device)
        rc = self.lib.adfwi_acoustic_backward(
            self.handle, N.ptr(alpha1), N.ptr(alpha2), N.ptr(damp), N.ptr(wavelet),
            N.ptr(gs[0]), N.ptr(gs[1]), N.ptr(gs[2]), N.ptr(ga1), N.ptr(ga2), N.ptr(workspace),
            workspace.numel(), st)
        N.check(rc, "adfwi_acoustic_backward")
        return ga1, ga2


def _raise_on_status(code):
    if code != 0:
        raise RuntimeError("adfwi_gb300: a pipeline wait timed out on the GPU during this solve (status %d); "
                           "its results are invalid" % code)


class AcousticSolve(torch.autograd.Function):
    """records, forward wavefields = solve(alpha1, alpha2); backward = hand-written adjoint."""

    @staticmethod
    def forward(ctx, alpha1, alpha2, damp, wavelet, plan):
        alpha1 = alpha1.contiguous()
        alpha2 = alpha2.contiguous()
        damp = damp.contiguous()
        wavelet = wavelet.contiguous()
        need_grad = bool(ctx.needs_input_grad[0] or ctx.needs_input_grad[1])
        if need_grad and plan.snapshot_every == BOUNDARY_SAVING:
            plan.check_boundary_saving(damp)
        # records the loss does not use reach backward as None (no zero-filled adjoint sources
        # to allocate and inject)
        ctx.set_materialize_grads(False)
        rp, ru, rw, fp, fu, fw, ws = plan.run_forward(alpha1, alpha2, damp, wavelet, need_grad)
        if not need_grad:
            # no backward will read the device status of this solve: check it now (a gradient
            # solve is checked after its adjoint, which covers both passes)
            _raise_on_status(plan.status(ws, False))
        ctx.plan = plan
        ctx.ws = ws if need_grad else None
        ctx.save_for_backward(alpha1, alpha2, damp, wavelet)
        ctx.mark_non_differentiable(fp, fu, fw)
        return rp, ru, rw, fp, fu, fw

    @staticmethod
    def backward(ctx, grp, gru, grw, _gfp, _gfu, _gfw):
        alpha1, alpha2, damp, wavelet = ctx.saved_tensors
        if ctx.ws is None:
            raise RuntimeError("AcousticSolve.backward: the forward kept no snapshots (inputs did not require "
                               "grad) or they were already used by an earlier backward; run forward again")
        ga1, ga2 = ctx.plan.run_backward(alpha1, alpha2, damp, wavelet, (grp, gru, grw), ctx.ws)
        _raise_on_status(ctx.plan.status(ctx.ws, True))
        ctx.ws = None  # release the snapshot workspace as soon as the adjoint has consumed it
        return ga1, ga2, None, None, None


ADJOINT_SOURCES = ("array", "inject")


class AcousticL2Solve(torch.autograd.Function):
    """loss, records, forward wavefields = normalised L2 misfit of the solve's p records against
    ``obs``; backward = the hand-written adjoint driven by the misfit's adjoint source. The misfit
    is ADFWI/fwi/misfit/L2.py:26-29 on traces divided by their peak
    (ADFWI/fwi/acoustic_fwi.py:149-150; ``normalise_obs`` divides obs too, else obs is taken as
    given, already normalised); the records come back without gradient.

    ``adjoint_source``: "array" writes the source as an (ns, nt, nr) array in one
    bandwidth-bound pass that the adjoint reads (the faster form on GB300); "inject" forms each
    sample inside the adjoint step as it is injected, with no array (the lanes that inject the
    receivers then pace their tiles: about 10-15% more time per adjoint step on the 300 x 700,
    30-shot workload). Both give the same bits."""

    @staticmethod
    def forward(ctx, alpha1, alpha2, damp, wavelet, obs, plan, silent_rel, normalise_obs, adjoint_source="array"):
        if adjoint_source not in ADJOINT_SOURCES:
            raise ValueError("adjoint_source must be one of %s, got %r" % (ADJOINT_SOURCES, adjoint_source))
        if plan.nm != 1:
            raise ValueError("AcousticL2Solve takes a single-model plan")
        alpha1, alpha2, damp, wavelet = (t.contiguous() for t in (alpha1, alpha2, damp, wavelet))
        obs = obs.to(dtype=plan.dtype).contiguous()
        if plan.snapshot_every == BOUNDARY_SAVING:
            plan.check_boundary_saving(damp)
        rp, ru, rw, fp, fu, fw, ws = plan.run_forward(alpha1, alpha2, damp, wavelet, True)
        loss = plan.l2_loss(rp, obs, ws, silent_rel, normalise_obs)[0]
        ctx.plan, ctx.ws, ctx.norm, ctx.source = plan, ws, normalise_obs, adjoint_source
        ctx.save_for_backward(alpha1, alpha2, damp, wavelet, rp, obs)
        ctx.mark_non_differentiable(rp, ru, rw, fp, fu, fw)
        return loss, rp, ru, rw, fp, fu, fw

    @staticmethod
    def backward(ctx, gloss, *_):
        alpha1, alpha2, damp, wavelet, rp, obs = ctx.saved_tensors
        if ctx.ws is None:
            raise RuntimeError("AcousticL2Solve.backward: the snapshots were already used by an earlier backward")
        if gloss is None:
            gloss = torch.ones((), dtype=torch.float64, device=alpha1.device)
        if ctx.source == "array":
            adj = ctx.plan.l2_sources(rp, obs, ctx.ws, gloss, ctx.norm)
            ga1, ga2 = ctx.plan.run_backward(alpha1, alpha2, damp, wavelet, (adj, None, None), ctx.ws)
            del adj
        else:
            ga1, ga2 = ctx.plan.run_backward_l2(alpha1, wavelet, rp, obs, ctx.ws, gloss, ctx.norm)
        _raise_on_status(ctx.plan.status(ctx.ws, True))
        ctx.ws = None
        return ga1, ga2, None, None, None, None, None, None, None
