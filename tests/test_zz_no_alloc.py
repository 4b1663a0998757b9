"""The allocation-free forward entry point, called through the C ABI.

``adfwi_acoustic_forward_noalloc`` serves callers that may not call cudaMalloc (their device
memory belongs to another allocator or pool, or their footprint is fixed after start-up):
it keeps its scratch in a 64 MiB static device array inside the library instead of a
caller workspace. This file runs last in the suite (pytest collects files in name order) so
that a failure here leaves every other test already run. Each check makes two calls in a
row on different problems: the array keeps the previous call's contents, so the second call
shows that nothing stale leaks into a result.
"""
import ctypes

import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300 import _native as N
from _cases import acoustic_problem, rel

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    fn = N.lib().adfwi_acoustic_forward_noalloc
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p] * 12
    return fn


def _inputs(seed, **kw):
    model, survey, prop = acoustic_problem(A, seed=seed, **kw)
    model.forward()
    a1, a2 = (t.detach().contiguous() for t in prop.coefficients(model))
    _, plan = prop.plan()
    return plan, a1, a2, prop.damp, prop.wavelet.contiguous()


def _noalloc_status(plan, dev):
    fn = N.lib().adfwi_acoustic_noalloc_status
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]
    v = ctypes.c_int32(-1)
    N.check(fn(plan.handle, ctypes.byref(v), N.stream_handle(dev)), "adfwi_acoustic_noalloc_status")
    return v.value


def _call_noalloc(plan, a1, a2, damp, wav):
    dev = a1.device
    rec = [torch.empty((plan.ns, plan.nt, plan.nr), dtype=plan.dtype, device=dev) for _ in range(3)]
    fw = [torch.empty((plan.nz, plan.nx), dtype=plan.dtype, device=dev) for _ in range(3)]
    rc = _noalloc_fn()(plan.handle, N.ptr(a1), N.ptr(a2), N.ptr(damp), N.ptr(wav), *[N.ptr(t) for t in rec + fw],
                       N.stream_handle(dev))
    N.check(rc, "adfwi_acoustic_forward_noalloc")
    return rec + fw


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_noalloc_forward_matches_workspace_forward_twice(dtype):
    tol = 1e-5 if dtype == torch.float32 else 1e-12
    for seed, kw in ((41, dict(free_surface=False, ns=3)), (42, dict(free_surface=True, ns=5, nt=180))):
        plan, a1, a2, damp, wav = _inputs(seed, dtype=dtype, **kw)
        assert plan.workspace_bytes(False) <= 64 << 20
        got = _call_noalloc(plan, a1, a2, damp, wav)
        # the call's bounded pipeline waits all completed (its error flag lives in the static array)
        assert _noalloc_status(plan, a1.device) == 0
        want = plan.run_forward(a1, a2, damp, wav, False)[:6]
        torch.cuda.synchronize()
        for g, w in zip(got, want):
            assert rel(g, w) <= tol, rel(g, w)


def test_noalloc_rejects_solves_larger_than_its_static_scratch():
    plan, a1, a2, damp, wav = _inputs(43, nz=300, nx=400, nabc=40, ns=40, nt=20, nr=50)
    assert plan.workspace_bytes(False) > 64 << 20
    with pytest.raises(RuntimeError, match="static scratch"):
        _call_noalloc(plan, a1, a2, damp, wav)
