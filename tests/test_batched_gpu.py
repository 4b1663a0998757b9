"""Batched acoustic plans against single-model solves (GPU).

A batched plan solves several velocity models of one grid shape in the same launches: each
shot group reads its own model's coefficient block. Per shot the arithmetic is that of a
single-model plan, and each model's shots are grouped as a plan of that model alone groups
them, so the records, the forward-wavefield maps and the coefficient gradients are
bit-identical to solving each model alone.
"""
import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300.acoustic import AcousticPlan
from _cases import acoustic_problem, rel

pytestmark = pytest.mark.gpu


def _model_inputs(seed, ns, dtype, free_surface):
    model, survey, prop = acoustic_problem(A, seed=seed, ns=ns, nt=150, dtype=dtype, free_surface=free_surface)
    model.forward()
    a1, a2 = (t.detach().contiguous() for t in prop.coefficients(model))
    return prop, a1, a2, prop.damp.contiguous(), prop.wavelet.contiguous()


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("free_surface", [False, True])
@pytest.mark.parametrize("snapshot_every", [0, 23])
def test_batched_solve_equals_single_model_solves(dtype, free_surface, snapshot_every):
    cases = [_model_inputs(seed, ns, dtype, free_surface) for seed, ns in ((3, 2), (4, 1), (5, 3))]
    p0 = cases[0][0]
    src_z = np.concatenate([c[0].src_loc[:, 1] for c in cases])
    src_x = np.concatenate([c[0].src_loc[:, 0] for c in cases])
    shot_model = np.concatenate([np.full(c[0].src_n, m) for m, c in enumerate(cases)])
    kw = dict(nz=p0.nz, nx=p0.nx, nabc=p0.nabc, free_surface=free_surface, rcv_z=p0.rcv_loc[:, 1],
              rcv_x=p0.rcv_loc[:, 0], nt=p0.nt, dt=p0.dt, dtype=dtype, snapshot_every=snapshot_every)
    batched = AcousticPlan(src_z=src_z, src_x=src_x, shot_model=shot_model, **kw)
    assert batched.nm == 3
    stack = lambda k: torch.stack([c[k] for c in cases]).contiguous()  # noqa: E731
    a1, a2, damp = stack(1), stack(2), stack(3)
    wav = torch.cat([c[4] for c in cases]).contiguous()
    out = batched.run_forward(a1, a2, damp, wav, True)
    gen = torch.Generator().manual_seed(9)
    w = torch.randn(out[0].shape, generator=gen, dtype=dtype).cuda()
    ga1, ga2 = batched.run_backward(a1, a2, damp, wav, (w, None, None), out[6])
    assert batched.status(out[6], True) == 0
    s0 = 0
    for m, (prop, b1, b2, bd, bw) in enumerate(cases):
        single = AcousticPlan(src_z=prop.src_loc[:, 1], src_x=prop.src_loc[:, 0], **kw)
        o = single.run_forward(b1, b2, bd, bw, True)
        s1 = s0 + prop.src_n
        g1, g2 = single.run_backward(b1, b2, bd, bw, (w[s0:s1].contiguous(), None, None), o[6])
        for q in range(3):
            assert torch.equal(out[q][s0:s1], o[q]), (m, q)
        for q in range(3, 6):
            assert torch.equal(out[q][m], o[q]), (m, q, rel(out[q][m], o[q]))
        assert torch.equal(ga1[m], g1), (m, rel(ga1[m], g1))
        assert torch.equal(ga2[m], g2), (m, rel(ga2[m], g2))
        s0 = s1



@pytest.mark.parametrize("free_surface", [False, True])
@pytest.mark.parametrize("snapshot_every", [0, 23])
def test_ring_depth_changes_no_result(free_surface, snapshot_every):
    """The deep-ring variants of the step kernels (2 blocks per SM, one stage more) launch with
    other widths and stages but the same units and arithmetic: records, forward-wavefield maps
    and gradients are bit-identical to the shallow ring's, also on a batched plan."""
    cases = [_model_inputs(seed, ns, torch.float32, free_surface) for seed, ns in ((6, 3), (7, 2))]
    p0 = cases[0][0]
    src_z = np.concatenate([c[0].src_loc[:, 1] for c in cases])
    src_x = np.concatenate([c[0].src_loc[:, 0] for c in cases])
    shot_model = np.concatenate([np.full(c[0].src_n, m) for m, c in enumerate(cases)])
    kw = dict(nz=p0.nz, nx=p0.nx, nabc=p0.nabc, free_surface=free_surface, rcv_z=p0.rcv_loc[:, 1],
              rcv_x=p0.rcv_loc[:, 0], nt=p0.nt, dt=p0.dt, dtype=torch.float32, snapshot_every=snapshot_every,
              src_z=src_z, src_x=src_x, shot_model=shot_model)
    stack = lambda k: torch.stack([c[k] for c in cases]).contiguous()  # noqa: E731
    a1, a2, damp = stack(1), stack(2), stack(3)
    wav = torch.cat([c[4] for c in cases]).contiguous()
    w = None
    res = []
    for depth in (1, 2):
        plan = AcousticPlan(ring_depth=depth, **kw)
        out = plan.run_forward(a1, a2, damp, wav, True)
        if w is None:
            w = torch.randn(out[0].shape, generator=torch.Generator().manual_seed(4)).cuda()
        ga1, ga2 = plan.run_backward(a1, a2, damp, wav, (w, None, None), out[6])
        assert plan.status(out[6], True) == 0
        res.append([t.clone() for t in out[:6]] + [ga1, ga2])
    for q, (x, y) in enumerate(zip(*res)):
        assert torch.equal(x, y), (q, rel(x, y))


def test_drop_in_gradients_are_bitwise_repeatable():
    """Two gradient evaluations through the drop-in propagators give the same bits: the step
    kernels reduce in a fixed order and the edge-replicate padding folds back without atomics."""
    from _cases import elastic_problem
    model, survey, prop = acoustic_problem(A, seed=11, ns=3, nt=200, free_surface=True)
    w = torch.randn((prop.src_n, prop.nt, prop.rcv_n), generator=torch.Generator().manual_seed(2)).cuda()
    grads = []
    for _ in range(2):
        model.vp.grad = None
        model.rho.grad = None
        (prop.forward()["p"] * w).sum().backward()
        grads.append((model.vp.grad.clone(), model.rho.grad.clone()))
    assert torch.equal(grads[0][0], grads[1][0]) and torch.equal(grads[0][1], grads[1][1])
    model, survey, prop = elastic_problem(A, seed=3, ns=2, nt=120)
    wv = torch.randn((prop.src_n, prop.nt, prop.rcv_n), generator=torch.Generator().manual_seed(3)).cuda()
    egrads = []
    for _ in range(2):
        for par in ("vp", "vs", "rho", "eps", "delta"):
            getattr(model, par).grad = None
        rec = prop.forward(fd_order=4)
        ((rec["vx"] + rec["vz"]) * wv).sum().backward()
        egrads.append([getattr(model, par).grad.clone() for par in ("vp", "vs", "rho", "eps", "delta")])
    for a, b in zip(*egrads):
        assert torch.equal(a, b)


def test_cpu_device_keeps_cpu_placement_and_solves_on_the_gpu():
    """device="cpu" (the reference's default): CPU model parameters and CPU records, the solve on
    the GPU, gradients on the CPU parameters equal to those of the same solve on cuda:0."""
    from _cases import elastic_problem
    out = {}
    for dev in ("cuda:0", "cpu"):
        model, survey, prop = acoustic_problem(A, seed=21, ns=2, nt=160, device=dev)
        assert model.vp.device.type == torch.device(dev).type
        rec = prop.forward()
        assert rec["p"].device.type == torch.device(dev).type
        w = torch.randn(rec["p"].shape, generator=torch.Generator().manual_seed(5)).to(rec["p"].device)
        (rec["p"] * w).sum().backward()
        out[dev] = (rec["p"].detach().cpu(), model.vp.grad.detach().cpu())
    assert rel(out["cpu"][0], out["cuda:0"][0]) <= 1e-6 and rel(out["cpu"][1], out["cuda:0"][1]) <= 1e-5
    eout = {}
    for dev in ("cuda:0", "cpu"):
        model, survey, prop = elastic_problem(A, seed=4, ns=2, nt=100, device=dev)
        rec = prop.forward(fd_order=4)
        assert rec["vx"].device.type == torch.device(dev).type
        w = torch.randn(rec["vx"].shape, generator=torch.Generator().manual_seed(6)).to(rec["vx"].device)
        (rec["vx"] * w).sum().backward()
        eout[dev] = (rec["vx"].detach().cpu(), model.vp.grad.detach().cpu())
    assert rel(eout["cpu"][0], eout["cuda:0"][0]) <= 1e-5 and rel(eout["cpu"][1], eout["cuda:0"][1]) <= 1e-4


def test_checkpointed_gradient_is_bit_identical_to_the_full_history():
    """With native snapshots the recomputed segments replay the forward states exactly, so the
    gradient of K < nt equals the full-history gradient bit for bit (loss through forward_l2)."""
    res = {}
    for K in (0, 40, 75):
        model, survey, prop = acoustic_problem(A, seed=17, ns=6, nt=300, snapshot_every=K, memory_budget=4 << 30)
        obs = torch.randn((prop.src_n, prop.nt, prop.rcv_n), generator=torch.Generator().manual_seed(8)).cuda()
        model.vp.grad = None
        loss, rec = prop.forward_l2(obs, silent_rel=1e-3, normalise_obs=True)
        loss.backward()
        assert prop.plan()[1].snapshot_every == (300 if K == 0 else K)
        res[K] = (float(loss.detach()), rec["p"].detach().clone(), model.vp.grad.detach().clone())
    for K in (40, 75):
        assert res[K][0] == res[0][0]
        assert torch.equal(res[K][1], res[0][1]) and torch.equal(res[K][2], res[0][2])
