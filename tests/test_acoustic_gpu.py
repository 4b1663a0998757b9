"""Acoustic CUDA path vs the CPU oracle and the reference's golden vectors (GPU tests).

Tolerances: records within 1e-5 relative L2 in float32 (the kernel keeps the reference's
operation order without FMA contraction, so they are usually bit-identical), gradients
within 1e-4 relative L2 of the oracle's autograd gradient in float32 and 1e-9 in float64,
and within 1e-6 of centred finite differences of the float64 scheme.
"""
import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from _cases import acoustic_problem, golden_files, oracle_acoustic, rel

pytestmark = pytest.mark.gpu

KEYS = ("p", "u", "w", "forward_wavefield_p", "forward_wavefield_u", "forward_wavefield_w")


@pytest.mark.parametrize("free_surface", [False, True])
@pytest.mark.parametrize("segments", [1, 3])
def test_forward_matches_oracle_f32(free_surface, segments):
    model, survey, prop = acoustic_problem(A, free_surface=free_surface, seed=1 + segments)
    rec = prop.forward(checkpoint_segments=segments)
    ref, _, _ = oracle_acoustic(prop, model, segments=segments, requires_grad=False)
    for k in KEYS:
        assert rel(rec[k], ref[k]) <= 1e-5, (k, rel(rec[k], ref[k]))


@pytest.mark.parametrize("free_surface", [False, True])
def test_forward_is_bit_identical_given_identical_coefficients(free_surface):
    """With the same alpha arrays (computed once on the CPU) the kernel reproduces the CPU
    reference arithmetic exactly: it keeps the reference's operation order, no FMA."""
    from adfwi_gb300.acoustic import AcousticSolve
    from oracle.acoustic import acoustic_forward_coef, pad_edge
    model, survey, prop = acoustic_problem(A, free_surface=free_surface, seed=4)
    model.forward()
    c = pad_edge(model.vp.detach().cpu(), prop.nabc)
    den = pad_edge(model.rho.detach().cpu(), prop.nabc)
    a1 = den * c * c * prop.dt / prop.dz
    a2 = prop.dt / (den * prop.dz)
    _, plan = prop.plan()
    out = AcousticSolve.apply(a1.cuda(), a2.cuda(), prop.damp, prop.wavelet, plan)
    ref = acoustic_forward_coef(a1, a2, prop.damp.cpu(), prop.src_loc[:, 0], prop.src_loc[:, 1],
                                prop.wavelet.cpu(), prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=prop.nabc,
                                free_surface=bool(free_surface), dt=prop.dt)
    for o, k in zip(out[:3], ("p", "u", "w")):
        assert torch.equal(o.cpu(), ref[k]), (k, rel(o, ref[k]))


def test_forward_matches_oracle_f64_subset():
    model, survey, prop = acoustic_problem(A, dtype=torch.float64, ns=4, seed=7)
    rec = prop.forward(shot_index=[3, 1])
    ref, _, _ = oracle_acoustic(prop, model, shot_index=[3, 1], requires_grad=False)
    for k in KEYS:
        assert rel(rec[k], ref[k]) <= 1e-13, k


@pytest.mark.parametrize("path", golden_files("acoustic"), ids=lambda p: p.split("/")[-1])
def test_forward_and_gradient_match_reference_golden(path):
    g = np.load(path)
    dt_ = torch.float64 if str(g["dtype"]) == "f64" else torch.float32
    nz, nx, nabc = int(g["nz"]), int(g["nx"]), int(g["nabc"])
    model = A.AcousticModel(0, 0, nx, nz, float(g["dx"]), float(g["dx"]), vp=g["vp_in"], rho=g["rho_in"],
                            vp_grad=True, rho_grad=True, free_surface=bool(g["free_surface"]), nabc=nabc,
                            device="cuda:0", dtype=dt_)
    src = A.Source(nt=int(g["nt"]), dt=float(g["dt"]), f0=float(g["f0"]))
    _, wav = A.wavelet(int(g["nt"]), float(g["dt"]), float(g["f0"]))
    src.add_sources(src_x=g["src_x"], src_z=g["src_z"], src_wavelet=wav)
    rcv = A.Receiver(nt=int(g["nt"]), dt=float(g["dt"]))
    rcv.add_receivers(rcv_x=g["rcv_x"], rcv_z=g["rcv_z"], rcv_type="pr")
    prop = A.AcousticPropagator(model, A.Survey(src, rcv), device="cuda:0", dtype=dt_)
    assert np.array_equal(prop.damp.cpu().numpy(), g["damp"])
    rec = prop.forward(checkpoint_segments=int(g["segments"]))
    for k in KEYS:
        assert rel(rec[k], g["rec_" + k]) <= 1e-5, k
    loss = sum((rec[k] * torch.tensor(g["w_" + k], dtype=dt_, device="cuda:0")).sum() for k in "puw")
    loss.backward()
    tol = 1e-9 if dt_ == torch.float64 else 1e-4
    assert rel(model.vp.grad, g["grad_vp"]) <= tol
    assert rel(model.rho.grad, g["grad_rho"]) <= tol


def _grad_case(dtype, free_surface, snapshot_every, seed, precision="native"):
    model, survey, prop = acoustic_problem(A, dtype=dtype, free_surface=free_surface, seed=seed,
                                           snapshot_every=snapshot_every, snapshot_precision=precision)
    rec = prop.forward()
    gen = torch.Generator().manual_seed(seed)
    w = {k: torch.randn(rec[k].shape, generator=gen, dtype=dtype) for k in "puw"}
    loss = sum((rec[k] * w[k].cuda()).sum() for k in "puw")
    loss.backward()
    ref, vp, rho = oracle_acoustic(prop, model)
    sum((ref[k] * w[k]).sum() for k in "puw").backward()
    return model, prop, vp, rho


@pytest.mark.parametrize("free_surface", [False, True])
@pytest.mark.parametrize("snapshot_every", [0, 37, 250])
def test_gradient_matches_oracle_f32(free_surface, snapshot_every):
    model, prop, vp, rho = _grad_case(torch.float32, free_surface, snapshot_every, seed=11)
    assert rel(model.vp.grad, vp.grad) <= 1e-4
    assert rel(model.rho.grad, rho.grad) <= 1e-4


@pytest.mark.parametrize("free_surface", [False, True])
def test_gradient_matches_oracle_f64(free_surface):
    model, prop, vp, rho = _grad_case(torch.float64, free_surface, 23, seed=12)
    assert rel(model.vp.grad, vp.grad) <= 1e-9
    assert rel(model.rho.grad, rho.grad) <= 1e-9


@pytest.mark.parametrize("precision,tol", [("bf16", 3e-2), ("fp16", 3e-3), ("fp24", 1e-4)])
def test_low_precision_snapshots_stay_close(precision, tol):
    m0, _, vp, _ = _grad_case(torch.float32, False, 25, seed=13)
    m1, _, _, _ = _grad_case(torch.float32, False, 25, seed=13, precision=precision)
    err = rel(m1.vp.grad, m0.vp.grad)
    assert err <= tol, err


def test_gradient_matches_centred_finite_differences_f64():
    """dL/d(alpha1, alpha2) from the adjoint vs centred differences of the float64 scheme."""
    from adfwi_gb300.acoustic import AcousticSolve
    model, survey, prop = acoustic_problem(A, dtype=torch.float64, nz=24, nx=30, nabc=8, nt=160, ns=2, nr=10,
                                           seed=21, snapshot_every=20)
    model.forward()
    a1, a2 = (t.detach().clone().requires_grad_(True) for t in prop.coefficients(model))
    _, plan = prop.plan()
    gen = torch.Generator().manual_seed(5)
    w = [torch.randn((2, 160, 10), generator=gen, dtype=torch.float64).cuda() for _ in range(3)]

    def loss(x1, x2):
        out = AcousticSolve.apply(x1, x2, prop.damp, prop.wavelet, plan)
        return sum((o * wi).sum() for o, wi in zip(out[:3], w))

    loss(a1, a2).backward()
    d1 = a1.detach() * torch.randn(a1.shape, generator=gen, dtype=torch.float64).cuda()
    d2 = a2.detach() * torch.randn(a2.shape, generator=gen, dtype=torch.float64).cuda()
    an = float((a1.grad * d1).sum() + (a2.grad * d2).sum())
    eps = 1e-6
    with torch.no_grad():
        fd = (float(loss(a1 + eps * d1, a2 + eps * d2)) - float(loss(a1 - eps * d1, a2 - eps * d2))) / (2 * eps)
    assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-4), (torch.float64, 1e-9)])
@pytest.mark.parametrize("free_surface", [False, True])
def test_gradient_of_pressure_records_only(dtype, tol, free_surface):
    """A loss on the pressure records alone (dL/d u- and w-records absent): receiver tiles take
    the ordinary path and their dL/d p-records are added to the stored adjoint state after
    each item. The survey puts 64 receiver cells in one 64-column tile, two receivers on some
    cells and receivers on two depths, so every variant of that injection runs (cached cells,
    the per-item table walk, a free-surface tile next to an ordinary one)."""
    nz, nx, nabc, nt = 40, 120, 12, 200
    rng = np.random.default_rng(41)
    from _cases import layered_vp
    npdt = np.float64 if dtype == torch.float64 else np.float32
    vp = layered_vp(nz, nx, rng).astype(npdt)
    rho = (np.power(vp, 0.25) * 310).astype(npdt)
    model = A.AcousticModel(0, 0, nx, nz, 10.0, 10.0, vp=vp, rho=rho, vp_grad=True, rho_grad=True,
                            free_surface=free_surface, nabc=nabc, device="cuda:0", dtype=dtype)
    src = A.Source(nt=nt, dt=1e-3, f0=20.0)
    _, wav = A.wavelet(nt, 1e-3, 20.0)
    src.add_sources(src_x=np.array([5, 60, 110]), src_z=np.array([1, 1, 1]), src_wavelet=wav)
    rx = np.concatenate([np.arange(nx), np.arange(0, nx, 7), np.arange(3, nx, 5)])
    rz = np.concatenate([np.full(nx, 2), np.full(len(np.arange(0, nx, 7)), 2), np.full(len(np.arange(3, nx, 5)), 21)])
    rcv = A.Receiver(nt=nt, dt=1e-3)
    rcv.add_receivers(rcv_x=rx, rcv_z=rz, rcv_type="pr")
    prop = A.AcousticPropagator(model, A.Survey(src, rcv), device="cuda:0", dtype=dtype, snapshot_every=30)
    rec = prop.forward()
    w = torch.randn(rec["p"].shape, generator=torch.Generator().manual_seed(3), dtype=dtype)
    (rec["p"] * w.cuda()).sum().backward()
    ref, vpo, rhoo = oracle_acoustic(prop, model)
    (ref["p"] * w).sum().backward()
    assert rel(model.vp.grad, vpo.grad) <= tol, rel(model.vp.grad, vpo.grad)
    assert rel(model.rho.grad, rhoo.grad) <= tol, rel(model.rho.grad, rhoo.grad)


def test_repeated_backward_and_shot_batches_agree():
    model, survey, prop = acoustic_problem(A, ns=4, seed=31, snapshot_every=40)
    rec = prop.forward()
    rec["p"].sum().backward()
    g_all = model.vp.grad.clone()
    model.vp.grad = None
    for idx in ([0, 1], [2, 3]):
        prop.forward(shot_index=idx)["p"].sum().backward()
    assert rel(model.vp.grad, g_all) <= 1e-5


def test_bad_geometry_is_rejected_on_the_host():
    model, survey, prop = acoustic_problem(A, seed=3)
    survey.source.loc_x[0] = 10 ** 6
    with pytest.raises(Exception):
        A.AcousticPropagator(model, survey, device="cuda:0").forward()


def test_full_size_gradient_is_additive_over_shots():
    """The 200 x 600 gradient workload at full size (30 shots, 300 x 700 padded, nt = 3000,
    600 receivers, pressure records): gradients are sums over shots, so the 30-shot gradient
    equals the sum of three 10-shot gradients (different unit groupings and partial sums) to
    rounding."""
    from adfwi_gb300.synthetic import acoustic_gradient_case
    model, survey, _, _ = acoustic_gradient_case(seed=0, device="cuda:0", nt=3000)
    prop = A.AcousticPropagator(model, survey, device="cuda:0")
    w = torch.randn((30, 3000, prop.rcv_n), generator=torch.Generator().manual_seed(8)).cuda()

    def grad(idx):
        model.vp.grad = None
        rec = prop.forward(shot_index=idx)
        sel = list(range(30)) if idx is None else idx
        (rec["p"] * w[sel]).sum().backward()
        return model.vp.grad.detach().clone()

    g_all = grad(None)
    g_sum = sum(grad(list(range(b, b + 10))) for b in (0, 10, 20))
    assert torch.isfinite(g_all).all()
    assert rel(g_all, g_sum) <= 1e-5, rel(g_all, g_sum)
