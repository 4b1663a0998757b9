"""Normalised L2 trace misfit on the GPU (``adfwi_l2_misfit`` of the C ABI).

``l2_misfit(syn, obs, dt)`` is ``Misfit_waveform_L2`` (ADFWI/fwi/misfit/L2.py:26-29) applied to
traces divided by their max |value| (ADFWI/fwi/acoustic_fwi.py:149-150), differentiable with
respect to ``syn``: one fused CUDA pass set computes the loss (FP64 sums in a fixed order) and
the adjoint source, which the backward hands on. ``l2_misfit_and_adjoint`` returns both without
autograd.
"""
import ctypes

import torch

from . import _native as N
from .acoustic import dtype_code


def l2_misfit_and_adjoint(syn, obs, dt, silent_rel=0.0, normalise_obs=True, stream=None, adj=None):
    """(loss as a 0-d FP64 device tensor, dL/dsyn) for records of shape (ns, nt, nr); ``adj``
    may name the output buffer (same shape and dtype as ``syn``)."""
    if not syn.is_cuda or not obs.is_cuda:
        raise RuntimeError("l2_misfit runs on CUDA tensors only (adfwi_gb300 has no CPU implementation)")
    if syn.shape != obs.shape or syn.dim() != 3:
        raise ValueError("syn and obs must both be (ns, nt, nr), got %s and %s" % (tuple(syn.shape), tuple(obs.shape)))
    syn = syn.contiguous()
    obs = obs.to(syn.dtype).contiguous()
    ns, nt, nr = syn.shape
    lib = N.lib()
    code = dtype_code(syn.dtype)
    need = ctypes.c_int64()
    N.check(lib.adfwi_l2_misfit_workspace_bytes(code, ns, nr, ctypes.byref(need)), "adfwi_l2_misfit_workspace_bytes")
    ws = torch.empty(need.value, dtype=torch.uint8, device=syn.device)
    if adj is None:
        adj = torch.empty_like(syn)
    elif adj.shape != syn.shape or adj.dtype != syn.dtype or not adj.is_contiguous() or adj.device != syn.device:
        raise ValueError("adj must be a contiguous tensor like syn")
    loss = torch.empty((), dtype=torch.float64, device=syn.device)
    st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(syn.device)
    N.check(lib.adfwi_l2_misfit(code, ns, nt, nr, float(dt), float(silent_rel), int(bool(normalise_obs)),
                                N.ptr(syn), N.ptr(obs), N.ptr(adj), N.ptr(loss), N.ptr(ws), ws.numel(), st),
            "adfwi_l2_misfit")
    return loss, adj


class _NormalisedL2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, syn, obs, dt, silent_rel, normalise_obs):
        loss, adj = l2_misfit_and_adjoint(syn, obs, dt, silent_rel, normalise_obs)
        ctx.save_for_backward(adj)
        return loss

    @staticmethod
    def backward(ctx, g):
        (adj,) = ctx.saved_tensors
        return adj * g.to(adj.dtype), None, None, None, None


def l2_misfit(syn, obs, dt, silent_rel=0.0, normalise_obs=True):
    """Normalised L2 misfit (0-d FP64 tensor), differentiable with respect to ``syn``."""
    return _NormalisedL2.apply(syn, obs, dt, silent_rel, normalise_obs)
