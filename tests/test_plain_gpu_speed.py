"""Speed of the library against the plain GPU path on the same gradient sample (GPU test).

The plain path is the reference's algorithm as PyTorch tensor operations (the oracle's loop,
which reproduces the reference's records bit for bit on the CPU), run on CUDA tensors with
autograd for the gradient, every time chunk under torch.utils.checkpoint as the reference's
propagator always runs it (acoustic_kernels.py:268-278): what the reference does on a GPU. The sample is the
200 x 600 gradient workload (30 shots, 300 x 700 padded cells) cut to 100 time steps. The
library must be at least 20x faster and give the same gradient within 1e-5; the measured
ratio is printed.
"""
import json
import time

import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300.synthetic import acoustic_gradient_case

pytestmark = pytest.mark.gpu


def _time(f, reps):
    f()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        f()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / reps


def test_gradient_beats_the_plain_gpu_path():
    from oracle.acoustic import acoustic_forward
    nt = 100
    model, survey, _, _ = acoustic_gradient_case(seed=0, device="cuda:0", nt=nt)
    prop = A.AcousticPropagator(model, survey, device="cuda:0", memory_budget=60 << 30)
    cells = prop.src_n * (prop.nz + 2 * prop.nabc) * (prop.nx + 2 * prop.nabc) * nt
    gen = torch.Generator().manual_seed(0)
    wts = torch.randn((prop.src_n, nt, prop.rcv_n), generator=gen).cuda()

    def ours():
        model.vp.grad = None
        (prop.forward()["p"] * wts).sum().backward()
        return model.vp.grad

    def plain():
        model.forward()
        vp = model.vp.detach().clone().requires_grad_(True)
        out = acoustic_forward(vp, model.rho.detach(), prop.damp, prop.src_loc[:, 0], prop.src_loc[:, 1],
                               prop.wavelet, prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=prop.nabc,
                               free_surface=False, dx=prop.dx, dz=prop.dz, dt=prop.dt, allow_gpu=True,
                               checkpoint_chunks=True)
        (out["p"] * wts).sum().backward()
        return vp.grad

    t_plain = _time(plain, 2)
    t_ours = _time(ours, 5)
    g_plain, g_ours = plain().detach(), ours().detach()
    rel = float((g_ours - g_plain).norm() / g_plain.norm())
    print(json.dumps({"sample": "30 shots x 300x700 padded x %d steps, forward + gradient" % nt,
                      "plain_gpu_gcell_per_s": round(cells / t_plain / 1e9, 3),
                      "library_gcell_per_s": round(cells / t_ours / 1e9, 3), "speedup": round(t_plain / t_ours, 2),
                      "gradient_rel_diff": rel}))
    assert rel <= 1e-5
    assert t_plain / t_ours >= 20.0
