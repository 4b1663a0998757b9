"""Drop-in propagators: ``AcousticPropagator`` and ``ElasticPropagator``.

Same constructors, attributes (``src_n``, ``damp``, ``bcx``, ``bcz``, ``wavelet``, ...),
``forward`` signatures and returned record dicts as the reference's
``ADFWI/propagator/acoustic_propagator.py:21-157`` and ``elastic_propagator.py:20-142``.
The time loop runs in the adfwi_gb300 CUDA library; the model parameterisation and the
edge padding stay in PyTorch autograd, so ``loss.backward()`` reaches vp / vs / rho / eps /
delta exactly as in the reference, with the hand-written adjoint in place of autograd
through the time loop.

Options beyond the reference's (all keyword-only, with reference-compatible defaults):
``snapshot_precision`` ("native", "bf16", "fp16", "fp24"), ``snapshot_every`` (steps between
checkpoint snapshots, 0 = chosen from ``memory_budget``; for the acoustic propagator -1 =
boundary saving: the forward keeps the absorbing frame of every step and the adjoint rebuilds
the interior states backwards), ``memory_budget`` (bytes for the
gradient workspace; default half of the free device memory when the plan is built),
``shots_per_block`` (0 = automatic); for the acoustic propagator ``ring_depth`` (TMA ring of
the step kernels: 0 = automatic, 1 = shallow, 2 = deep; results do not depend on it).

``device="cpu"`` (the reference's default) keeps the reference's placement: the model's
parameters and the returned records stay on the CPU, and the solve itself runs on the current
CUDA device (the parameters' padded coefficients are copied there and the records back, both
differentiably, so gradients reach the CPU parameters). There is no CPU solver: without a CUDA
device the constructor raises.
"""
from typing import Dict, Optional

import numpy as np
import torch
from torch import Tensor

from .acoustic import AcousticPlan, AcousticSolve
from .boundary import bc_gerjan, bc_pml, bc_pml_xz, bc_sincos
from .utils import numpy2tensor


def _is_model(m):
    return all(hasattr(m, a) for a in ("nx", "nz", "dx", "dz", "nabc", "free_surface", "abc_type", "forward"))


def _is_survey(s):
    return hasattr(s, "source") and hasattr(s, "receiver")


def fold_replicate(g, top, bottom, left, right):
    """Adjoint of edge-replicate padding by (top, bottom, left, right) cells: the padded strips
    fold into the edge rows / columns and the corner blocks into the corner cells, with
    fixed-order reductions (the same sums on every run)."""
    nz, nx = g.shape[0] - top - bottom, g.shape[1] - left - right
    r0, r1, c0, c1 = top, top + nz, left, left + nx
    out = g[r0:r1, c0:c1].clone()
    if top:
        out[0, :] += g[:r0, c0:c1].sum(0)
    if bottom:
        out[-1, :] += g[r1:, c0:c1].sum(0)
    if left:
        out[:, 0] += g[r0:r1, :c0].sum(1)
    if right:
        out[:, -1] += g[r0:r1, c1:].sum(1)
    if top and left:
        out[0, 0] += g[:r0, :c0].sum()
    if top and right:
        out[0, -1] += g[:r0, c1:].sum()
    if bottom and left:
        out[-1, 0] += g[r1:, :c0].sum()
    if bottom and right:
        out[-1, -1] += g[r1:, c1:].sum()
    return out


class _PadReplicate(torch.autograd.Function):
    """Edge-replicate padding with the fold above as its backward (PyTorch's replicate-pad
    backward accumulates with atomics on CUDA, so its FP32 sums vary from run to run)."""

    @staticmethod
    def forward(ctx, v, top, bottom, left, right):
        ctx.pads = (top, bottom, left, right)
        return torch.nn.functional.pad(v[None, None], (left, right, top, bottom), mode="replicate")[0, 0]

    @staticmethod
    def backward(ctx, g):
        return fold_replicate(g, *ctx.pads), None, None, None, None


def _pad_replicate(v, top, bottom, left, right):
    """Edge-replicate padding (acoustic_kernels.py:16-37, elastic_kernels.py:175-216),
    differentiable with a deterministic backward."""
    return _PadReplicate.apply(v, top, bottom, left, right)


class _PropagatorBase(torch.nn.Module):
    def __init__(self, model, survey, device, cpu_num, gpu_num, dtype, snapshot_precision, snapshot_every,
                 memory_budget, shots_per_block):
        super().__init__()
        if not _is_model(model):
            raise ValueError("model is not an instance of AbstractModel")
        if not _is_survey(survey):
            raise ValueError("survey is not an instance of Survey")
        dev = torch.device(device)
        # device="cpu": CPU placement of the model and the records, the solve on the GPU
        self._host_io = dev.type == "cpu"
        if self._host_io:
            if not torch.cuda.is_available():
                raise RuntimeError("adfwi_gb300 propagators solve on a CUDA device and none is available "
                                   "(device=%r; there is no CPU implementation)" % (device,))
            dev = torch.device("cuda", torch.cuda.current_device())
        elif dev.type != "cuda":
            raise RuntimeError("adfwi_gb300 propagators run on a CUDA device (got device=%r); "
                               "there is no CPU implementation" % (device,))
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.model = model
        self.survey = survey
        self.device = device
        self._dev = dev
        self.dtype = dtype
        self.cpu_num = cpu_num
        self.gpu_num = gpu_num
        self.ox, self.oz = model.ox, model.oz
        self.dx, self.dz = model.dx, model.dz
        self.nx, self.nz = model.nx, model.nz
        self.nt = survey.source.nt
        self.dt = survey.source.dt
        self.f0 = survey.source.f0
        self.abc_type = model.abc_type
        self.nabc = model.nabc
        self.free_surface = model.free_surface
        self.snapshot_precision = snapshot_precision
        self.snapshot_every = snapshot_every
        self.memory_budget = memory_budget
        self.shots_per_block = shots_per_block
        self.bcx, self.bcz, self.damp = None, None, None
        self.boundary_condition()
        self.source = survey.source
        self.src_loc = self.source.get_loc()
        self.src_x = numpy2tensor(self.src_loc[:, 0], torch.long).to(dev)
        self.src_z = numpy2tensor(self.src_loc[:, 1], torch.long).to(dev)
        self.src_n = self.source.num
        self.wavelet = numpy2tensor(self.source.get_wavelet(), self.dtype).to(dev)
        self.moment_tensor = numpy2tensor(self.source.get_moment_tensor(), self.dtype).to(dev)
        self.receiver = survey.receiver
        self.rcv_loc = self.receiver.get_loc()
        self.rcv_x = numpy2tensor(self.rcv_loc[:, 0], torch.long).to(dev)
        self.rcv_z = numpy2tensor(self.rcv_loc[:, 1], torch.long).to(dev)
        self.rcv_n = self.receiver.num
        self._plans = {}

    def _select(self, shot_index):
        idx = np.arange(self.src_n)
        if shot_index is not None:
            if torch.is_tensor(shot_index):
                shot_index = shot_index.cpu().numpy()
            idx = idx[shot_index]
        idx = np.atleast_1d(idx)
        return idx

    def _budget(self):
        if self.memory_budget is not None:
            return int(self.memory_budget)
        free, _ = torch.cuda.mem_get_info(self._dev)
        return int(0.5 * free)

    def _to_solver(self, *ts):
        """Tensors onto the solve's device (differentiable copies when they are elsewhere)."""
        return [t if t is None or t.device == self._dev else t.to(self._dev) for t in ts]

    def _to_caller(self, rec):
        """The record dict on the caller's device (the CPU for device="cpu")."""
        return {k: v.cpu() for k, v in rec.items()} if self._host_io else rec

    def _wavelet_rows(self, idx):
        if len(idx) == self.src_n and np.array_equal(idx, np.arange(self.src_n)):
            return self.wavelet
        return self.wavelet[torch.as_tensor(idx, device=self._dev)]


class AcousticPropagator(_PropagatorBase):
    """Isotropic acoustic (p, u, w) propagator (acoustic_propagator.py:21-157)."""

    def __init__(self, model, survey, device: Optional[str] = "cpu", cpu_num: Optional[int] = 1,
                 gpu_num: Optional[int] = 1, dtype: torch.dtype = torch.float32, *,
                 snapshot_precision="native", snapshot_every=0, memory_budget=None, shots_per_block=0,
                 ring_depth=0):
        super().__init__(model, survey, device, cpu_num, gpu_num, dtype, snapshot_precision, snapshot_every,
                         memory_budget, shots_per_block)
        self.ring_depth = int(ring_depth)

    def boundary_condition(self, vmax=None):
        """Damping frame of acoustic_propagator.py:102-118 (always built without a free surface)."""
        if self.abc_type.lower() == "pml":
            if vmax is None:
                vmax = self.model.vp.cpu().detach().numpy().max()
            damp = bc_pml(self.nx, self.nz, self.dx, self.dz, pml=self.nabc, vmax=vmax, free_surface=False)
        elif self.abc_type.lower() == "gerjan":
            damp = bc_gerjan(self.nx, self.nz, self.dx, self.dz, pml=self.nabc,
                             alpha=self.model.abc_jerjan_alpha, free_surface=False)
        else:
            damp = bc_sincos(self.nx, self.nz, self.dx, self.dz, pml=self.nabc, free_surface=False)
        self.damp = numpy2tensor(damp, self.dtype).to(self._dev)

    def plan(self, shot_index=None, checkpoint_segments=1):
        idx = self._select(shot_index)
        key = (idx.tobytes(), int(checkpoint_segments))
        p = self._plans.get(key)
        if p is None:
            p = AcousticPlan(nz=self.nz, nx=self.nx, nabc=self.nabc, free_surface=self.free_surface,
                             src_z=self.src_loc[idx, 1], src_x=self.src_loc[idx, 0],
                             rcv_z=self.rcv_loc[:, 1], rcv_x=self.rcv_loc[:, 0], nt=self.nt, dt=self.dt,
                             dtype=self.dtype, checkpoint_segments=checkpoint_segments,
                             snapshot_every=self.snapshot_every, snapshot_precision=self.snapshot_precision,
                             shots_per_block=self.shots_per_block, memory_budget=self._budget(),
                             ring_depth=self.ring_depth)
            self._plans[key] = p
        return idx, p

    def coefficients(self, model=None):
        """alpha1 = rho c^2 dt/dz and alpha2 = dt/(rho dz) on the padded grid (acoustic_kernels.py:225-260)."""
        model = self.model if model is None else model
        n = self.nabc
        c = _pad_replicate(model.vp, n, n, n, n)
        den = _pad_replicate(model.rho, n, n, n, n)
        # The divisor is a 0-d tensor on the device: PyTorch's CUDA division by a host scalar
        # multiplies by its reciprocal, which rounds differently from the reference's division
        # (1 ulp on about a quarter of the cells); an elementwise division rounds like the CPU.
        dz = torch.tensor(self.dz, dtype=den.dtype, device=den.device)
        alpha1 = den * c * c * self.dt / dz
        alpha2 = self.dt / (den * self.dz)
        return alpha1, alpha2

    def forward(self, model=None, shot_index: Optional[int] = None, checkpoint_segments: int = 1) -> Dict[str, Tensor]:
        model = self.model if model is None else model
        model.forward()
        idx, plan = self.plan(shot_index, checkpoint_segments)
        alpha1, alpha2 = self.coefficients(model)
        if alpha1.dtype != self.dtype:
            alpha1, alpha2 = alpha1.to(self.dtype), alpha2.to(self.dtype)
        alpha1, alpha2 = self._to_solver(alpha1, alpha2)
        wav = self._wavelet_rows(idx)
        rp, ru, rw, fp, fu, fw = AcousticSolve.apply(alpha1, alpha2, self.damp, wav, plan)
        return self._to_caller({"p": rp, "u": ru, "w": rw, "forward_wavefield_p": fp, "forward_wavefield_u": fu,
                                "forward_wavefield_w": fw})


    def forward_l2(self, obs, model=None, shot_index=None, checkpoint_segments: int = 1, silent_rel=0.0,
                   normalise_obs=False, adjoint_source="array"):
        """The normalised L2 misfit of the selected shots' pressure records against ``obs``
        (ns, nt, nr) with the solve: returns (loss, record dict). ``loss`` (FP64) is
        differentiable with respect to the model parameters; its backward runs the hand-written
        adjoint driven by the misfit's adjoint source (the reference computes the records, the
        misfit of ADFWI/fwi/misfit/L2.py:26-29 on peak-normalised traces
        (ADFWI/fwi/acoustic_fwi.py:149-150) and its autograd gradient as separate PyTorch passes).
        ``normalise_obs`` divides obs by its trace peaks too; ``silent_rel`` > 0 treats traces
        whose peak is at most that share of their gather's peak as zero (0 = the reference).
        ``adjoint_source``: "array" (one (ns, nt, nr) source array, the faster form) or "inject"
        (formed inside the adjoint step, no array); the same bits either way."""
        from .acoustic import AcousticL2Solve
        model = self.model if model is None else model
        model.forward()
        idx, plan = self.plan(shot_index, checkpoint_segments)
        alpha1, alpha2 = self.coefficients(model)
        if alpha1.dtype != self.dtype:
            alpha1, alpha2 = alpha1.to(self.dtype), alpha2.to(self.dtype)
        alpha1, alpha2 = self._to_solver(alpha1, alpha2)
        obs = torch.as_tensor(obs, device=self._dev)
        loss, rp, ru, rw, fp, fu, fw = AcousticL2Solve.apply(alpha1, alpha2, self.damp, self._wavelet_rows(idx), obs,
                                                             plan, float(silent_rel), bool(normalise_obs),
                                                             adjoint_source)
        rec = self._to_caller({"p": rp, "u": ru, "w": rw, "forward_wavefield_p": fp, "forward_wavefield_u": fu,
                               "forward_wavefield_w": fw})
        return (loss.cpu() if self._host_io else loss), rec


class ElasticPropagator(_PropagatorBase):
    """Isotropic / VTI / HTI elastic velocity-stress propagator (elastic_propagator.py:20-142)."""

    def __init__(self, model, survey, device: Optional[str] = "cpu", cpu_num: Optional[int] = 1,
                 gpu_num: Optional[int] = 1, dtype=torch.float32, *, snapshot_precision="native", snapshot_every=0,
                 memory_budget=None):
        super().__init__(model, survey, device, cpu_num, gpu_num, dtype, snapshot_precision, snapshot_every,
                         memory_budget, 0)

    def boundary_condition(self):
        """bcx / bcz (abc_type "PML", case-sensitive as elastic_propagator.py:100) or a damping frame."""
        if self.abc_type == "PML":
            vmax = self.model.vp.cpu().detach().numpy().max()
            bcx, bcz = bc_pml_xz(self.nx, self.nz, self.dx, self.dz, pml=self.nabc, vmax=vmax,
                                 free_surface=self.free_surface)
            self.bcx = numpy2tensor(bcx, self.dtype).to(self._dev)
            self.bcz = numpy2tensor(bcz, self.dtype).to(self._dev)
        elif self.abc_type == "gerjan":
            damp = bc_gerjan(self.nx, self.nz, self.dx, self.dz, pml=self.nabc, alpha=self.model.abc_jerjan_alpha,
                             free_surface=self.free_surface)
            self.damp = numpy2tensor(damp, self.dtype).to(self._dev)
        else:
            damp = bc_sincos(self.nx, self.nz, self.dx, self.dz, pml=self.nabc, free_surface=self.free_surface)
            self.damp = numpy2tensor(damp, self.dtype).to(self._dev)

    def plan(self, shot_index=None, fd_order=4, checkpoint_segments=1):
        from .elastic import ElasticPlan
        idx = self._select(shot_index)
        key = (idx.tobytes(), int(fd_order), int(checkpoint_segments))
        p = self._plans.get(key)
        if p is None:
            p = ElasticPlan(nz=self.nz, nx=self.nx, nabc=self.nabc, free_surface=self.free_surface,
                            src_z=self.src_loc[idx, 1], src_x=self.src_loc[idx, 0], rcv_z=self.rcv_loc[:, 1],
                            rcv_x=self.rcv_loc[:, 0],
                            moment_tensor=self.moment_tensor.detach().cpu().double().numpy()[idx],
                            nt=self.nt, dt=self.dt, dx=self.dx, dz=self.dz, dtype=self.dtype, fd_order=fd_order,
                            pml=self.abc_type.lower() == "pml", checkpoint_segments=checkpoint_segments,
                            snapshot_every=self.snapshot_every, snapshot_precision=self.snapshot_precision,
                            memory_budget=self._budget())
            self._plans[key] = p
        return idx, p

    def padded_coefficients(self, model=None, fd_order=4):
        """Padded C11, C13, C15, C33, C35, C55, bx, bz and boundary arrays (elastic_kernels.py:928-953)."""
        model = self.model if model is None else model
        fs_off = fd_order // 2
        n = self.nabc
        top = fs_off if self.free_surface else fs_off + n
        pad = lambda a: _pad_replicate(a, top, n, n, n)  # noqa: E731
        CC = model.CC
        coefs = [pad(CC[k]) for k in (0, 2, 4, 11, 13, 18)] + [pad(model.bx), pad(model.bz)]
        coefs = [c.to(self.dtype) if c.dtype != self.dtype else c for c in coefs]
        bpad = lambda a: _pad_replicate(a, fs_off, 0, 0, 0)  # noqa: E731
        if self.abc_type.lower() == "pml":
            if self.bcx is None:
                raise ValueError("abc_type %r selects the PML kernel but no bcx/bcz were built (the reference "
                                 "builds them only for abc_type == 'PML')" % self.abc_type)
            abc = [bpad(self.bcx), bpad(self.bcz)]
        else:
            abc = [bpad(self.damp), None]
        return coefs, abc

    def forward(self, model=None, shot_index=None, fd_order=4, checkpoint_segments=1) -> Dict[str, Tensor]:
        from .elastic import COMPONENTS, ElasticSolve
        model = self.model if model is None else model
        model.forward()
        idx, plan = self.plan(shot_index, fd_order, checkpoint_segments)
        coefs, abc = self.padded_coefficients(model, fd_order)
        coefs = self._to_solver(*coefs)
        wav = self._wavelet_rows(idx)
        outs = ElasticSolve.apply(*coefs, abc[0], abc[1], wav, plan)
        rec = {k: outs[q] for q, k in enumerate(COMPONENTS)}
        for q, k in enumerate(COMPONENTS):
            rec["forward_wavefield_" + k] = outs[5 + q]
        return self._to_caller(rec)
