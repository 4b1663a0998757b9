"""Elastic solve: native plan wrapper and the autograd Function around the CUDA library.

``ElasticSolve.apply(C11, C13, C15, C33, C35, C55, bx, bz, abc0, abc1, wavelet, plan)``
replaces the reference's elastic ``forward_kernel`` time loop
(ADFWI/propagator/elastic_kernels.py:917-1037) and its autograd backward through
``torch.utils.checkpoint`` (975-1008). Inputs are the padded coefficient arrays exactly as the
reference pads them (``bx`` (nzp, nxp-1), ``bz`` (nzp-1, nxp), ``C55`` (nzp-2, nxp-2)), and
either the padded PML profiles ``bcx``, ``bcz`` or the padded multiplicative ``damp`` (then
``abc1`` is None). The backward returns dL/d of the eight model coefficients.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .acoustic import _i32, dtype_code, snapshot_code

COMPONENTS = ("txx", "tzz", "txz", "vx", "vz")


def diff_coef(nn):
    """Staggered-grid coefficients from the float32 linear solve of elastic_kernels.py:20-58."""
    a = torch.empty((nn, nn), dtype=torch.float32)
    for i in range(nn):
        for j in range(nn):
            a[i, j] = (2 * (j + 1) - 1) ** (2 * (i + 1) - 1)
    b = torch.cat((torch.tensor([1.0], dtype=torch.float32), torch.zeros(nn - 1, dtype=torch.float32)))
    return (torch.linalg.inv(a) @ b).tolist()


class ElasticPlan(object):
    """Geometry and launch configuration of one elastic solve shape (host object)."""

    def __init__(self, *, nz, nx, nabc, free_surface, src_z, src_x, rcv_z, rcv_x, moment_tensor, nt, dt, dx, dz,
                 dtype, fd_order=4, pml=True, checkpoint_segments=1, snapshot_every=0, snapshot_precision="native",
                 memory_budget=0):
        if fd_order not in (4, 6):
            raise ValueError("adfwi_gb300 supports fd_order 4 and 6 (the reference selects its 6th-order "
                             "operators for every fd_order other than 4)")
        self.lib = N.lib()
        self.src_z, self.src_x = _i32(src_z), _i32(src_x)
        self.rcv_z, self.rcv_x = _i32(rcv_z), _i32(rcv_x)
        self.mt = np.ascontiguousarray(np.asarray(moment_tensor, dtype=np.float64).reshape(-1, 3, 3))
        self.ns, self.nr, self.nt = len(self.src_z), len(self.rcv_z), int(nt)
        self.nz, self.nx, self.nabc = int(nz), int(nx), int(nabc)
        self.fd_order, self.pml, self.dtype = int(fd_order), bool(pml), dtype
        self.free_surface = bool(free_surface)
        d = N.ElasticDesc()
        d.nz, d.nx, d.nabc, d.free_surface = self.nz, self.nx, self.nabc, int(self.free_surface)
        d.ns, d.nt, d.nr, d.dtype = self.ns, self.nt, self.nr, dtype_code(dtype)
        d.fd_order, d.pml = self.fd_order, int(self.pml)
        d.checkpoint_segments = int(checkpoint_segments)
        d.snapshot_every = int(snapshot_every or 0)
        d.snapshot_precision = snapshot_code(snapshot_precision)
        d.dt, d.dx, d.dz = float(dt), float(dx), float(dz)
        f = diff_coef(self.fd_order // 2) + [0.0, 0.0]
        for k in range(3):
            d.fdc[k] = float(f[k])
        d.memory_budget = int(memory_budget or 0)
        self.desc = d
        h = ctypes.c_void_p()
        arr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = self.lib.adfwi_elastic_plan_create(ctypes.byref(d), arr(self.src_z), arr(self.src_x), arr(self.rcv_z),
                                                arr(self.rcv_x), arr(self.mt), ctypes.byref(h))
        N.check(rc, "adfwi_elastic_plan_create")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.adfwi_elastic_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    def workspace_bytes(self, with_gradient):
        b = ctypes.c_int64()
        N.check(self.lib.adfwi_elastic_workspace_bytes(self.handle, int(bool(with_gradient)), ctypes.byref(b)),
                "adfwi_elastic_workspace_bytes")
        return b.value

    @property
    def snapshot_every(self):
        k = ctypes.c_int32()
        N.check(self.lib.adfwi_elastic_snapshot_every(self.handle, ctypes.byref(k)), "adfwi_elastic_snapshot_every")
        return k.value

    def _coef_arrays(self, coefs):
        ts = [c.contiguous() for c in coefs if c is not None]
        for t in ts:
            if not t.is_cuda:
                raise RuntimeError("elastic coefficients must be CUDA tensors (adfwi_gb300 runs on the GPU only)")
            if t.dtype != self.dtype:
                raise TypeError("coefficient dtype %s differs from the plan's %s" % (t.dtype, self.dtype))
        ptrs = (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])
        shapes = (ctypes.c_int32 * (2 * len(ts)))(*[d for t in ts for d in t.shape])
        return ts, ptrs, shapes

    def run_forward(self, coefs, wavelet, with_gradient, workspace=None):
        ts, ptrs, shapes = self._coef_arrays(coefs)
        dev = ts[0].device
        ws = workspace
        if ws is None:
            ws = torch.empty(self.workspace_bytes(with_gradient), dtype=torch.uint8, device=dev)
        rec = torch.empty((5, self.ns, self.nt, self.nr), dtype=self.dtype, device=dev)
        fw = torch.empty((5, self.nz, self.nx), dtype=self.dtype, device=dev)
        wavelet = wavelet.contiguous()
        if tuple(wavelet.shape) != (self.ns, self.nt):
            raise ValueError("wavelet has shape %s, expected %s" % (tuple(wavelet.shape), (self.ns, self.nt)))
        rc = self.lib.adfwi_elastic_forward(self.handle, ptrs, shapes, N.ptr(wavelet), N.ptr(rec), N.ptr(fw),
                                            int(bool(with_gradient)), N.ptr(ws), ws.numel(), N.stream_handle(dev))
        N.check(rc, "adfwi_elastic_forward")
        return rec, fw, ws, ts

    def run_backward(self, coefs, wavelet, grad_rec, ws):
        ts, ptrs, shapes = self._coef_arrays(coefs)
        grads = [torch.empty_like(t) for t in ts[:8]]
        gptrs = (ctypes.c_void_p * 8)(*[g.data_ptr() for g in grads])
        gr = None if grad_rec is None else grad_rec.to(self.dtype).contiguous()
        rc = self.lib.adfwi_elastic_backward(self.handle, N.ptr(wavelet.contiguous()), N.ptr(gr), gptrs, shapes,
                                             N.ptr(ws), ws.numel(), N.stream_handle(ts[0].device))
        N.check(rc, "adfwi_elastic_backward")
        return grads


class ElasticSolve(torch.autograd.Function):
    """records (txx, tzz, txz, vx, vz), energy maps = solve(C11 .. bz); backward = hand-written adjoint."""

    @staticmethod
    def forward(ctx, c11, c13, c15, c33, c35, c55, bx, bz, abc0, abc1, wavelet, plan):
        coefs = [c11, c13, c15, c33, c35, c55, bx, bz, abc0, abc1]
        need = any(ctx.needs_input_grad[:8])
        ctx.set_materialize_grads(False)  # unused record components reach backward as None
        rec, fw, ws, ts = plan.run_forward(coefs, wavelet, need)
        ctx.plan = plan
        ctx.ws = ws if need else None
        ctx.save_for_backward(*ts, wavelet)
        outs = tuple(rec[k] for k in range(5)) + tuple(fw[k] for k in range(5))
        ctx.mark_non_differentiable(*outs[5:])
        return outs

    @staticmethod
    def backward(ctx, *grads):
        saved = ctx.saved_tensors
        coefs, wavelet = list(saved[:-1]), saved[-1]
        if ctx.ws is None:
            raise RuntimeError("ElasticSolve.backward: the forward kept no snapshots (inputs did not require grad) "
                               "or they were already used by an earlier backward; run forward again")
        g = grads[:5]
        if all(x is None for x in g):
            grec = None
        else:
            ref = next(x for x in g if x is not None)
            grec = torch.stack([x if x is not None else torch.zeros_like(ref) for x in g])
        out = ctx.plan.run_backward(coefs, wavelet, grec, ctx.ws)
        ctx.ws = None
        return tuple(out) + (None, None, None, None)
