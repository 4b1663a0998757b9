"""Elastic CUDA path vs the CPU oracle and the reference's golden vectors (GPU tests).

Records within 1e-5 relative L2 (float32), gradients w.r.t. vp, vs, rho, eps, delta within
1e-4 (float32) / 1e-9 (float64) of autograd through the oracle, and the coefficient
gradients within 1e-6 of centred finite differences of the float64 scheme.
"""
import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from _cases import ELASTIC_KEYS, elastic_problem, golden_files, oracle_elastic, rel

pytestmark = pytest.mark.gpu
PARS = ("vp", "vs", "rho", "eps", "delta")


@pytest.mark.parametrize("path", golden_files("elastic"), ids=lambda p: p.split("/")[-1])
def test_elastic_matches_reference_golden(path):
    g = np.load(path)
    iso = bool(g["iso"])
    nz, nx, dx = int(g["nz"]), int(g["nx"]), float(g["dx"])
    common = dict(free_surface=bool(g["free_surface"]), abc_type=str(g["abc_type"]), nabc=int(g["nabc"]),
                  device="cuda:0")
    if iso:
        model = A.IsotropicElasticModel(0, 0, nx, nz, dx, dx, vp=g["vp"], vs=g["vs"], rho=g["rho"], vp_grad=True,
                                        vs_grad=True, rho_grad=True, auto_update_rho=False, **common)
    else:
        model = A.AnisotropicElasticModel(0, 0, nx, nz, dx, dx, vp=g["vp"], vs=g["vs"], rho=g["rho"], eps=g["eps"],
                                          gamma=g["gamma"], delta=g["delta"], vp_grad=True, vs_grad=True,
                                          rho_grad=True, eps_grad=True, delta_grad=True, **common)
    nt, dt, f0 = int(g["nt"]), float(g["dt"]), float(g["f0"])
    src = A.Source(nt=nt, dt=dt, f0=f0)
    _, wav = A.wavelet(nt, dt, f0)
    src.add_sources(src_x=g["src_x"], src_z=g["src_z"], src_wavelet=wav, src_mt=g["moment_tensor"][0])
    rcv = A.Receiver(nt=nt, dt=dt)
    rcv.add_receivers(rcv_x=g["rcv_x"], rcv_z=g["rcv_z"], rcv_type="pr")
    prop = A.ElasticPropagator(model, A.Survey(src, rcv), device="cuda:0")
    rec = prop.forward(fd_order=int(g["fd_order"]), checkpoint_segments=int(g["segments"]))
    for k in rec:
        assert rel(rec[k], g["rec_" + k]) <= 1e-5, (k, rel(rec[k], g["rec_" + k]))
    loss = sum((rec[k] * torch.tensor(g["w_" + k], device="cuda:0")).sum() for k in ELASTIC_KEYS)
    loss.backward()
    for p in PARS:
        if "grad_" + p in g:
            assert rel(getattr(model, p).grad, g["grad_" + p]) <= 1e-4, (p, rel(getattr(model, p).grad, g["grad_" + p]))


@pytest.mark.parametrize("fd_order,abc_type,free_surface", [(4, "PML", True), (6, "PML", False),
                                                            (4, "gerjan", True), (6, "sincos", True),
                                                            (4, "PML", False)])
def test_elastic_gradient_matches_oracle_with_segments(fd_order, abc_type, free_surface):
    model, survey, prop = elastic_problem(A, fd_order=fd_order, abc_type=abc_type, free_surface=free_surface,
                                          seed=fd_order, snapshot_every=23)
    rec = prop.forward(fd_order=fd_order, checkpoint_segments=3)
    gen = torch.Generator().manual_seed(3)
    w = {k: torch.randn(rec[k].shape, generator=gen) for k in ELASTIC_KEYS}
    sum((rec[k] * w[k].cuda()).sum() for k in ELASTIC_KEYS).backward()
    ref, pars = oracle_elastic(prop, model, fd_order=fd_order, segments=3)
    for k in rec:
        assert rel(rec[k], ref[k]) <= 1e-5, (k, rel(rec[k], ref[k]))
    sum((ref[k] * w[k]).sum() for k in ELASTIC_KEYS).backward()
    for p in PARS:
        assert rel(getattr(model, p).grad, pars[p].grad) <= 1e-4, (p, rel(getattr(model, p).grad, pars[p].grad))


def test_elastic_isotropic_general_moment_tensor_f64():
    mt = [[1.0, 0.0, 0.4], [0.0, 1.0, 0.0], [0.4, 0.0, 0.6]]
    model, survey, prop = elastic_problem(A, iso=True, dtype=torch.float64, free_surface=False, mt=mt, seed=9,
                                          snapshot_every=31)
    rec = prop.forward()
    gen = torch.Generator().manual_seed(4)
    w = {k: torch.randn(rec[k].shape, generator=gen, dtype=torch.float64) for k in ELASTIC_KEYS}
    sum((rec[k] * w[k].cuda()).sum() for k in ELASTIC_KEYS).backward()
    ref, pars = oracle_elastic(prop, model)
    for k in rec:
        assert rel(rec[k], ref[k]) <= 1e-12, k
    sum((ref[k] * w[k]).sum() for k in ELASTIC_KEYS).backward()
    for p in ("vp", "vs", "rho"):
        assert rel(getattr(model, p).grad, pars[p].grad) <= 1e-9, p


@pytest.mark.parametrize("abc_type", ["PML", "gerjan"])
def test_elastic_coefficient_gradient_matches_finite_differences_f64(abc_type):
    from adfwi_gb300.elastic import ElasticSolve
    model, survey, prop = elastic_problem(A, dtype=torch.float64, nz=20, nx=26, nabc=6, nt=90, ns=1, nr=8,
                                          abc_type=abc_type, seed=5, snapshot_every=17)
    model.forward()
    coefs, abc = prop.padded_coefficients(model)
    leaves = [c.detach().clone().requires_grad_(True) for c in coefs]
    _, plan = prop.plan()
    gen = torch.Generator().manual_seed(8)
    w = [torch.randn((1, 90, 8), generator=gen, dtype=torch.float64).cuda() for _ in range(5)]

    def loss(cs):
        out = ElasticSolve.apply(*cs, abc[0], abc[1], prop.wavelet, plan)
        return sum((o * wi).sum() for o, wi in zip(out[:5], w))

    loss(leaves).backward()
    dirs = [c.detach() * torch.randn(c.shape, generator=gen, dtype=torch.float64).cuda() for c in leaves]
    an = float(sum((l.grad * d).sum() for l, d in zip(leaves, dirs)))
    eps = 1e-6
    with torch.no_grad():
        plus = float(loss([l + eps * d for l, d in zip(leaves, dirs)]))
        minus = float(loss([l - eps * d for l, d in zip(leaves, dirs)]))
    fd = (plus - minus) / (2 * eps)
    assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)


@pytest.mark.parametrize("precision,tol", [("bf16", 3e-2), ("fp16", 3e-3), ("fp24", 1e-4)])
@pytest.mark.parametrize("abc_type", ["PML", "gerjan"])
def test_elastic_low_precision_snapshots_stay_close(precision, tol, abc_type):
    """BF16 / FP16 checkpoints (per-snapshot max-abs scale) change the elastic gradients by at
    most a few parts in 1e2 / 1e3 of the native-snapshot gradients; the records not at all."""
    grads, recs = {}, {}
    for prec in ("native", precision):
        model, survey, prop = elastic_problem(A, abc_type=abc_type, seed=17, snapshot_every=20,
                                              snapshot_precision=prec)
        rec = prop.forward(fd_order=4)
        gen = torch.Generator().manual_seed(7)
        w = {k: torch.randn(rec[k].shape, generator=gen) for k in ELASTIC_KEYS}
        sum((rec[k] * w[k].cuda()).sum() for k in ELASTIC_KEYS).backward()
        grads[prec] = {p: getattr(model, p).grad.detach().clone() for p in PARS}
        recs[prec] = {k: rec[k].detach().clone() for k in ELASTIC_KEYS}
    for k in ELASTIC_KEYS:
        assert torch.equal(recs["native"][k], recs[precision][k])
    for p in PARS:
        err = rel(grads[precision][p], grads["native"][p])
        assert err <= tol, (p, err)


def test_elastic_shot_groups_agree_with_single_shots():
    """On the 242 x 480 padded VTI grid 13 shots run as groups of 5, 5 and 3 (the gradient
    kernels loop over the shots of a group, restaging each shot's planes in shared memory). Gradients are sums over shots, so the 13-shot gradient equals the sum of the
    13 single-shot gradients (each a group of one) to rounding."""
    from adfwi_gb300.synthetic import vti_gradient_case
    model, survey = vti_gradient_case(seed=2, nt=150, n_shots=13, device="cuda:0")
    prop = A.ElasticPropagator(model, survey, device="cuda:0")
    gen = torch.Generator().manual_seed(4)
    w = {k: torch.randn((13, 150, prop.rcv_n), generator=gen).cuda() for k in ("vx", "vz")}

    def grads(idx):
        for p in PARS:
            getattr(model, p).grad = None
        rec = prop.forward(shot_index=idx)
        sel = list(range(13)) if idx is None else [idx]
        sum((rec[k] * w[k][sel]).sum() for k in ("vx", "vz")).backward()
        return {p: getattr(model, p).grad.detach().clone() for p in PARS}

    g_all = grads(None)
    acc = {p: torch.zeros_like(g_all[p]) for p in PARS}
    for s in range(13):
        gs = grads(s)
        for p in PARS:
            acc[p] += gs[p]
    for p in PARS:
        assert rel(g_all[p], acc[p]) <= 1e-5, (p, rel(g_all[p], acc[p]))
