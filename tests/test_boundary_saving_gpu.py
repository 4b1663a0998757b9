"""Boundary-saving gradient (GPU): the forward keeps p, u, w of the absorbing frame after every
step and the adjoint rebuilds the interior states backwards by inverting the update
(replaces the reference's planned ADFWI/propagator/acoustic_kernels_bs.py:40-54, 202-313).
Records are those of any other gradient mode; the gradient matches the full-history gradient to
the rounding of the inverted updates (1e-5 in FP32, 1e-12 in FP64) and the oracle's autograd
gradient within 1e-4; the workspace is smaller than the full history's; a damping frame that
does not vanish inside the model is refused."""
import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300.acoustic import BOUNDARY_SAVING
from _cases import acoustic_problem, oracle_acoustic, rel

pytestmark = pytest.mark.gpu


def _gradient(prop, model, w):
    model.vp.grad = None
    model.rho.grad = None
    rec = prop.forward()
    (rec["p"] * w).sum().backward()
    return rec["p"].detach().clone(), model.vp.grad.detach().clone(), model.rho.grad.detach().clone()


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-12)])
@pytest.mark.parametrize("free_surface", [False, True])
def test_boundary_saving_matches_the_full_history(dtype, tol, free_surface):
    out = {}
    for K in (0, BOUNDARY_SAVING):
        model, survey, prop = acoustic_problem(A, seed=23, ns=3, nt=300, dtype=dtype, free_surface=free_surface,
                                               snapshot_every=K, memory_budget=4 << 30)
        w = torch.randn((prop.src_n, prop.nt, prop.rcv_n), generator=torch.Generator().manual_seed(3),
                        dtype=dtype).cuda()
        out[K] = _gradient(prop, model, w)
        plan = prop.plan()[1]
        assert plan.snapshot_every == (300 if K == 0 else BOUNDARY_SAVING)
        out[K] += (plan.workspace_bytes(True),)
    r0, gv0, gr0, b0 = out[0]
    r1, gv1, gr1, b1 = out[BOUNDARY_SAVING]
    assert torch.equal(r0, r1)
    assert rel(gv1, gv0) <= tol, rel(gv1, gv0)
    assert rel(gr1, gr0) <= tol, rel(gr1, gr0)
    assert b1 < b0  # the frame of every step takes less than the two planes of full history


def test_boundary_saving_gradient_matches_oracle():
    model, survey, prop = acoustic_problem(A, seed=24, ns=2, nt=250, snapshot_every=BOUNDARY_SAVING)
    rec = prop.forward()
    w = torch.randn(rec["p"].shape, generator=torch.Generator().manual_seed(4))
    (rec["p"] * w.cuda()).sum().backward()
    ref, vp, rho = oracle_acoustic(prop, model)
    (ref["p"] * w).sum().backward()
    assert rel(rec["p"], ref["p"]) <= 1e-5
    assert rel(model.vp.grad, vp.grad) <= 1e-4, rel(model.vp.grad, vp.grad)
    assert rel(model.rho.grad, rho.grad) <= 1e-4, rel(model.rho.grad, rho.grad)


def test_boundary_saving_refuses_damping_inside_the_model():
    model, survey, prop = acoustic_problem(A, seed=25, ns=1, nt=60, snapshot_every=BOUNDARY_SAVING)
    nzp, nxp = prop.damp.shape
    prop.damp[nzp // 2, nxp // 2] = 1.0
    with pytest.raises(ValueError, match="vanishes inside the model"):
        prop.forward()["p"].sum().backward()
