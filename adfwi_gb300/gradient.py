"""Gradient processor on the GPU: drop-in for ADFWI's ``GradProcessor``.

Mirrors ``ADFWI/propagator/gradient_process.py`` (``GradProcessor``, 74-134; ``grad_taper``,
52-71; ``smooth2d``, 32-49) with the same constructor, ``forward(nx, nz, vmax, grad, forw)``
signature, results and dtype flow, but runs on the device: the Gaussian smoothing of the
illumination (span 40) and of the gradient is the FP64 CUDA kernel ``adfwi_smooth2d``, and the
taper, mask, preconditioner and scaling are elementwise device operations, so an FWI loop
keeps its gradient on the GPU (the reference copies it to the host and convolves with scipy).

``forward`` accepts numpy arrays (returns numpy, as the reference) or CUDA tensors (returns a
CUDA tensor). Results follow the reference's dtypes: float32 until the preconditioner or the
land smoothing makes them float64.
"""
import ctypes

import numpy as np
import torch

from . import _native as N


def smooth2d(z, span=10, stream=None):
    """FP64 Gaussian smoothing of a (nz, nx) CUDA tensor (gradient_process.py:32-49)."""
    if not torch.is_tensor(z) or not z.is_cuda:
        raise RuntimeError("smooth2d runs on CUDA tensors only (adfwi_gb300 has no CPU implementation)")
    if z.dim() != 2:
        raise ValueError("smooth2d expects a 2-D plane, got shape %s" % (tuple(z.shape),))
    span = int(span)
    if span < 1:
        raise ValueError("span must be a positive integer")
    z = z.to(torch.float64).contiguous()
    nz, nx = z.shape
    lib = N.lib()
    need = ctypes.c_int64()
    N.check(lib.adfwi_smooth2d_workspace_bytes(nz, nx, span, ctypes.byref(need)), "adfwi_smooth2d_workspace_bytes")
    ws = torch.empty(need.value, dtype=torch.uint8, device=z.device)
    out = torch.empty_like(z)
    st = ctypes.c_void_p(stream) if stream is not None else N.stream_handle(z.device)
    N.check(lib.adfwi_smooth2d(nz, nx, span, N.ptr(z), N.ptr(out), N.ptr(ws), ws.numel(), st), "adfwi_smooth2d")
    return out


def _hamming(m):
    n = np.arange(m)
    return 0.54 - 0.46 * np.cos(2.0 * np.pi * n / (m - 1))


def grad_taper(nz, nx, tapersize=20, thred=0.05, marine_or_land="Marine", device="cuda"):
    """Gradient taper of gradient_process.py:52-71 as an FP64 CUDA tensor."""
    dev = torch.device(device)
    if marine_or_land in ("Marine", "Offshore"):
        taper = torch.ones((nz, nx), dtype=torch.float64, device=dev)
        taper[:tapersize, :] = 0.0
        return taper
    h = torch.as_tensor(_hamming(2 * tapersize)[tapersize:], dtype=torch.float64, device=dev)
    taper = torch.zeros((nz, nx), dtype=torch.float64, device=dev)
    taper[:, :tapersize] = h
    taper = smooth2d(taper, span=tapersize // 2)
    taper = taper / taper.max()
    taper = taper * (1 - thred)
    taper = -taper + 1
    return taper * taper


class GradProcessor(object):
    """Same constructor and ``forward`` as the reference's GradProcessor (gradient_process.py:74-134)."""

    def __init__(self, grad_mute=0, grad_smooth=0, grad_mask=None, norm_grad=True, forw_illumination=True,
                 marine_or_land="land"):
        self.grad_mute = grad_mute
        self.grad_smooth = grad_smooth
        self.grad_mask = grad_mask
        self.marine_or_land = marine_or_land
        self.norm_grad = norm_grad
        self.forw_illumination = forw_illumination
        self._taper = {}

    def _taper_for(self, nz, nx, thred, dev):
        key = (nz, nx, self.grad_mute, thred, self.marine_or_land, str(dev))
        t = self._taper.get(key)
        if t is None:
            t = grad_taper(nz, nx, tapersize=self.grad_mute, thred=thred, marine_or_land=self.marine_or_land,
                           device=dev)
            self._taper[key] = t
        return t

    def forward(self, nx, nz, vmax, grad, forw=None):
        numpy_io = not torch.is_tensor(grad)
        if numpy_io:
            dev = torch.device("cuda", torch.cuda.current_device())
        else:
            if not grad.is_cuda:
                raise RuntimeError("GradProcessor runs on CUDA tensors (adfwi_gb300 has no CPU implementation)")
            dev = grad.device
        mol = self.marine_or_land.lower()
        if mol in ("marine", "offshore"):
            thred = 0.0
        elif mol in ("land", "onshore"):
            thred = 0.001
        else:
            raise ValueError("not supported modeling marine_or_land: %s" % self.marine_or_land)
        g = torch.as_tensor(grad, device=dev).to(torch.float32)
        if self.grad_mute > 0:  # in place on the float32 gradient
            g = (g.double() * self._taper_for(nz, nx, thred, dev)).float()
        if self.grad_mask is not None:
            mask = torch.as_tensor(np.asarray(self.grad_mask) if not torch.is_tensor(self.grad_mask) else self.grad_mask,
                                   device=dev)
            if tuple(mask.shape) != tuple(g.shape):
                raise ValueError("Wrong size of grad mask: the size of the mask should be identical to the size of "
                                 "vp model")
            g = (g.double() * mask.double()).float()
        span = 40 if min(nz, nx) > 40 else int(min(nz, nx) / 2)
        if self.forw_illumination and forw is not None:
            precond = smooth2d(torch.as_tensor(forw, device=dev), span)
            precond = precond / torch.max(precond + 1e-5)
            precond = torch.where(precond < 1e-4, torch.full_like(precond, 1e-4), precond)
            g = g.double() / precond ** 2
        if self.grad_smooth > 0:
            if self.marine_or_land in ("marine", "offshore"):
                g = g.clone()
                g[self.grad_mute:, :] = smooth2d(g[self.grad_mute:, :], span=self.grad_smooth).to(g.dtype)
            else:
                g = smooth2d(g, span=self.grad_smooth)
        if self.norm_grad:
            vm = torch.as_tensor(float(vmax), dtype=g.dtype, device=dev)
            g = (vm * g) / torch.abs(g).max()
        return g.cpu().numpy() if numpy_io else g
