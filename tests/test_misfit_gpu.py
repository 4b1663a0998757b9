"""Fused normalised-L2 misfit kernel (adfwi_l2_misfit) against the PyTorch formulation and
autograd (GPU tests): loss within 1e-12 (FP64 sums on both sides), adjoint source within
1e-6 relative (FP32 records) / 1e-12 (FP64), silent traces, determinism."""
import pytest
import torch

from adfwi_gb300 import serving as S
from adfwi_gb300.misfit import l2_misfit, l2_misfit_and_adjoint

pytestmark = pytest.mark.gpu


def _records(dtype, seed=0, ns=3, nt=240, nr=37):
    g = torch.Generator().manual_seed(seed)
    syn = torch.randn(ns, nt, nr, generator=g, dtype=torch.float64)
    obs = torch.randn(ns, nt, nr, generator=g, dtype=torch.float64)
    syn[1, :, 5] *= -4.0          # negative peaks
    syn[2, :, 7] = 0.0            # a silent synthetic trace
    obs[0, :, 9] = 0.0            # a silent observed trace
    syn[0, :, 11] *= 1e-30        # only a precursor reached this receiver
    return syn.to(dtype).cuda(), obs.to(dtype).cuda()


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-6), (torch.float64, 1e-12)])
@pytest.mark.parametrize("silent_rel", [0.0, 1e-6])
def test_fused_misfit_matches_pytorch(dtype, tol, silent_rel):
    syn, obs = _records(dtype)
    loss, adj = l2_misfit_and_adjoint(syn, obs, 1.5e-3, silent_rel=silent_rel)
    ref_loss, ref_adj = S.l2_misfit_grad(syn, S.normalise_traces(obs, silent_rel), 1.5e-3, silent_rel)
    assert torch.isfinite(adj).all() and torch.isfinite(loss)
    assert abs(float(loss) - float(ref_loss)) <= 1e-12 * abs(float(ref_loss))
    assert float((adj - ref_adj).double().norm() / ref_adj.double().norm()) <= tol
    assert float(adj[2, :, 7].abs().max()) == 0.0
    if silent_rel > 0:
        assert float(adj[0, :, 11].abs().max()) == 0.0


def test_fused_misfit_is_the_autograd_gradient():
    syn, obs = _records(torch.float64, seed=3)
    syn[0, :, 11] = 1.0  # no precursor trace: the plain reference rule applies everywhere
    obs[0, :, 9] = 1.0
    syn[2, :, 7] = 1.0
    s = syn.clone().requires_grad_(True)
    sn = s / torch.max(torch.abs(s), dim=1, keepdim=True).values
    on = obs / torch.max(torch.abs(obs), dim=1, keepdim=True).values
    ref = torch.sum(torch.sqrt(torch.sum((on - sn) ** 2 * 1e-3, dim=1)))
    ref.backward()
    s2 = syn.clone().requires_grad_(True)
    loss = l2_misfit(s2, obs, 1e-3)
    (2.0 * loss).backward()
    r = float(ref.detach())
    assert abs(float(loss.detach()) - r) <= 1e-12 * r
    assert float((s2.grad - 2.0 * s.grad).norm() / (2.0 * s.grad).norm()) <= 1e-12


def test_misfit_peaks_keep_the_first_arg_max_across_time_phases():
    """Equal peaks at several samples (their time phases in either order, a negative one first):
    the max's share of the adjoint source goes to the earliest, as a scan in time order gives.
    Expected values: the formula restated with numpy in FP64 (argmax: first occurrence)."""
    import numpy as np
    g = torch.Generator().manual_seed(11)
    ns, nt, nr, dt = 2, 300, 40, 1e-3
    syn = torch.randn(ns, nt, nr, generator=g, dtype=torch.float64) * 0.1
    obs = torch.randn(ns, nt, nr, generator=g, dtype=torch.float64)
    syn[0, 20, 3] = 2.0; syn[0, 7, 3] = 2.0        # first at t=7 (phase 7), tie at t=20 (phase 4)
    syn[0, 35, 4] = -3.0; syn[0, 19, 4] = 3.0      # first at t=19, positive; tie at t=35, negative
    syn[1, 50, 5] = -1.5; syn[1, 66, 5] = -1.5; syn[1, 290, 5] = 1.5  # same phase: first t=50
    syn[1, 0, 6] = 4.0; syn[1, 299, 6] = -4.0      # ends of the trace
    loss, adj = l2_misfit_and_adjoint(syn.cuda(), obs.cuda(), dt, normalise_obs=True)
    y, o = syn.numpy(), obs.numpy()
    exp = np.zeros_like(y)
    tot = 0.0
    for s in range(ns):
        for r in range(nr):
            v = y[s, :, r]
            k = int(np.argmax(np.abs(v)))
            m = abs(v[k])
            on = o[s, :, r] / np.abs(o[s, :, r]).max()
            rsd = on - v / m
            n = np.sqrt(np.sum(rsd * rsd) * dt)
            tot += n
            e = -rsd * dt / (n * m)
            e[k] += dt * np.sum(rsd * v) / (n * m * m) * np.sign(v[k])
            exp[s, :, r] = e
    assert abs(float(loss) - tot) <= 1e-12 * tot
    a = adj.cpu().numpy()
    assert np.abs(a - exp).max() <= 1e-12 * np.abs(exp).max()
    for s, r, t in ((0, 3, 7), (0, 4, 19), (1, 5, 50), (1, 6, 0)):
        assert abs(a[s, t, r] - exp[s, t, r]) <= 1e-12 * abs(exp[s, t, r])


def test_fused_misfit_is_deterministic():
    syn, obs = _records(torch.float32, seed=5, ns=4, nt=500, nr=300)
    a = l2_misfit_and_adjoint(syn, obs, 1e-3)
    b = l2_misfit_and_adjoint(syn, obs, 1e-3)
    assert float(a[0]) == float(b[0]) and torch.equal(a[1], b[1])


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("silent_rel,normalise_obs", [(0.0, False), (1e-3, True)])
@pytest.mark.parametrize("snapshot_every", [0, 31])
def test_misfit_fused_into_the_adjoint_equals_the_two_pass_gradient(dtype, silent_rel, normalise_obs,
                                                                    snapshot_every):
    """The adjoint with the misfit's source formed as it is injected (adfwi_acoustic_l2_loss +
    adfwi_acoustic_backward_l2) gives the same loss and the same coefficient gradients, bit for
    bit, as the two-pass form: adfwi_l2_misfit writing the (ns, nt, nr) source, then
    adfwi_acoustic_backward reading it."""
    import adfwi_gb300 as A
    from _cases import acoustic_problem
    model, survey, prop = acoustic_problem(A, dtype=dtype, ns=3, nt=200, seed=8, free_surface=True,
                                           snapshot_every=snapshot_every)
    model.forward()
    a1, a2 = (t.detach().contiguous() for t in prop.coefficients(model))
    _, plan = prop.plan()
    damp, wav = prop.damp.contiguous(), prop.wavelet.contiguous()
    g = torch.Generator().manual_seed(2)
    obs = (torch.randn((plan.ns, plan.nt, plan.nr), generator=g, dtype=dtype) * 1e-3).cuda()
    # two-pass
    rp, _, _, _, _, _, ws = plan.run_forward(a1, a2, damp, wav, True)
    loss0, adj = l2_misfit_and_adjoint(rp, obs, plan_dt(prop), silent_rel=silent_rel, normalise_obs=normalise_obs)
    g1, g2 = plan.run_backward(a1, a2, damp, wav, (adj, None, None), ws)
    # fused
    rpf, _, _, _, _, _, wsf = plan.run_forward(a1, a2, damp, wav, True)
    loss1 = plan.l2_loss(rpf, obs, wsf, silent_rel, normalise_obs)
    one = torch.ones(1, dtype=torch.float64, device="cuda")
    f1, f2 = plan.run_backward_l2(a1, wav, rpf, obs, wsf, one, normalise_obs)
    assert plan.status(wsf, True) == 0
    assert torch.equal(rp, rpf)
    assert float(loss0) == float(loss1[0])
    assert torch.equal(g1, f1) and torch.equal(g2, f2)
    # the plan's array form of the source: the same bits as adfwi_l2_misfit's
    src = plan.l2_sources(rpf, obs, wsf, one, normalise_obs)
    assert torch.equal(src, adj)
    src2 = plan.l2_sources(rpf, obs, wsf, 2.0 * one, normalise_obs)
    assert torch.equal(src2, adj * 2.0)
    # the scale of the source scales the gradient
    rpf, _, _, _, _, _, wsf = plan.run_forward(a1, a2, damp, wav, True)
    plan.l2_loss(rpf, obs, wsf, silent_rel, normalise_obs)
    h1, _ = plan.run_backward_l2(a1, wav, rpf, obs, wsf, 2.0 * one, normalise_obs)
    assert float((h1 - 2.0 * f1).norm() / (2.0 * f1).norm()) <= (1e-6 if dtype == torch.float32 else 1e-14)


def plan_dt(prop):
    return prop.dt
