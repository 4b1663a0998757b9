"""Parity of the CUDA path with the oracle at the benchmarked configurations' real sizes (GPU).

Every grid here is the full padded grid of a benchmarked configuration; where the CPU oracle
would take hours, the shot count and the number of time steps are cut (stated per test),
never the grid, the absorbing frame or the receiver line:

* 100 x 100 forward configuration in full (PML 50 -> 200 x 200, 10 shots, 100 receivers,
  nt = 1000): all six record-dict entries against the oracle, and against the reference's own
  outputs recorded in ``tests/golden/acoustic_c1_full.npz``;
* 200 x 600 gradient configuration (300 x 700 padded, 600 receivers), 2 of its 30 shots x 1000
  steps: the gradient of the trace-normalised L2 misfit against the oracle's autograd gradient,
  with the whole history kept and with snapshots every 50 steps (1000 rather than fewer steps:
  earlier, the first arrivals of the near traces barely differ between the two models, and the
  misfit's 1 / sqrt(residual energy) makes its gradient change by tens of percent under
  1e-7 relative changes of the records, a property of the functional, not of either solver);
* 200 x 400 VTI configuration (PML 40 + free surface -> 242 x 480 padded, 400 receivers), 1 of
  its 20 shots x 200 steps: vx / vz records and the vp, vs, rho, eps, delta gradients;
* 500 x 1500 precision configuration in FP64 (600 x 1600 padded, 1500 receivers), 1 of its 64
  shots x 200 steps with snapshots every 50 steps: records and the vp gradient.

Tolerances (relative L2): float32 records 1e-5, float32 gradients 1e-4; float64 records 1e-12,
float64 gradients 1e-9.
"""
import os

import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from _cases import GOLDEN, rel

pytestmark = pytest.mark.gpu

KEYS = ("p", "u", "w", "forward_wavefield_p", "forward_wavefield_u", "forward_wavefield_w")


def _threads():
    torch.set_num_threads(max(1, os.cpu_count() or 1))


# ---------------------------------------------------------------------------- 100 x 100, in full
def test_c1_forward_in_full_matches_oracle_and_reference():
    from oracle.acoustic import acoustic_forward
    _threads()
    g = np.load(os.path.join(GOLDEN, "acoustic_c1_full.npz"))
    nz, nx, nabc, nt, dt, dx, f0 = (int(g["nz"]), int(g["nx"]), int(g["nabc"]), int(g["nt"]), float(g["dt"]),
                                    float(g["dx"]), float(g["f0"]))
    vp = g["vp_in"]
    model = A.AcousticModel(0, 0, nx, nz, dx, dx, vp=vp, rho=np.power(vp, 0.25) * 310, nabc=nabc, device="cuda:0")
    src = A.Source(nt=nt, dt=dt, f0=f0)
    _, wav = A.wavelet(nt, dt, f0)
    src.add_sources(src_x=g["src_x"], src_z=g["src_z"], src_wavelet=wav)
    rcv = A.Receiver(nt=nt, dt=dt)
    rcv.add_receivers(rcv_x=g["rcv_x"], rcv_z=g["rcv_z"], rcv_type="pr")
    prop = A.AcousticPropagator(model, A.Survey(src, rcv), device="cuda:0")
    assert np.array_equal(prop.damp.cpu().numpy(), g["damp"])
    with torch.no_grad():
        rec = prop.forward()
    got = {k: v.cpu() for k, v in rec.items()}
    with torch.no_grad():
        ref = acoustic_forward(model.vp.detach().cpu(), model.rho.detach().cpu(), prop.damp.cpu(), g["src_x"],
                               g["src_z"], prop.wavelet.cpu(), g["rcv_x"], g["rcv_z"], nabc=nabc, free_surface=False,
                               dx=dx, dz=dx, dt=dt)
    for k in KEYS:
        assert rel(got[k], ref[k]) <= 1e-5, (k, rel(got[k], ref[k]))
    # the kernels keep the reference's operation order and the coefficients are formed with its
    # divisions, so the records are the oracle's (and the reference's) bit for bit
    for k in "puw":
        assert torch.equal(got[k], ref[k]), (k, rel(got[k], ref[k]))
    # the reference's own outputs at this size
    for k in "puw":
        e = np.sum(got[k].numpy().astype(np.float64) ** 2, axis=1)
        assert rel(e, g["energy_" + k]) <= 1e-5, k
        assert rel(got["forward_wavefield_" + k], g["forward_wavefield_" + k]) <= 1e-5, k
    assert rel(got["p"][:, ::int(g["decimate"]), :], g["rec_p_dec"]) <= 1e-5


# ---------------------------------------------------------------------------- 200 x 600 gradient
def normalised_l2(syn, obs, dt, silent_rel=1e-3):
    """Misfit_waveform_L2 (ADFWI/fwi/misfit/L2.py:26-29) on traces divided by their peak
    (ADFWI/fwi/acoustic_fwi.py:149-150). 1000 steps into the 200 x 600 workload the wave has not
    reached the far part of the line, and the reference's division of an all-zero trace by its
    zero peak gives NaN, so traces whose peak is at most silent_rel of their gather's peak count
    as zero on both sides (the rule of the library's server, here with silent_rel = 1e-3)."""
    def norm(x):
        m = torch.amax(torch.abs(x), dim=1, keepdim=True)
        live = m > silent_rel * torch.amax(m, dim=2, keepdim=True)
        return torch.where(live, x / torch.where(live, m, torch.ones_like(m)), torch.zeros_like(x))
    r = norm(obs) - norm(syn)
    s = torch.sum(r * r * dt, dim=1)
    # a trace silent in both has zero residual: it adds 0, and (unlike sqrt at 0) no NaN slope
    live = s > 0
    return torch.sum(torch.sqrt(torch.where(live, s, torch.ones_like(s))) * live)


@pytest.fixture(scope="module")
def c2_slice():
    """Oracle records and autograd gradient of 2 shots x 1000 steps of the 200 x 600 workload
    (the oracle runs its chunks under torch.utils.checkpoint, as the reference does, to bound
    its host memory)."""
    from adfwi_gb300.synthetic import acoustic_gradient_case
    from oracle.acoustic import acoustic_forward
    _threads()
    model, survey, vp_true, vp_init = acoustic_gradient_case(seed=0, device="cuda:0", nt=1000)
    idx = [0, 29]
    prop = A.AcousticPropagator(model, survey, device="cuda:0")
    damp = prop.damp.cpu()
    loc = prop.src_loc[idx]
    rl = prop.rcv_loc
    wav = prop.wavelet.cpu()[idx]
    rho_t = torch.tensor(np.power(vp_true, 0.25) * 310)
    kw = dict(nabc=50, free_surface=False, dx=20.0, dz=20.0, dt=prop.dt)
    with torch.no_grad():
        obs = acoustic_forward(torch.tensor(vp_true), rho_t, damp, loc[:, 0], loc[:, 1], wav, rl[:, 0], rl[:, 1],
                               **kw)["p"]
    model.forward()
    vp = model.vp.detach().cpu().clone().requires_grad_(True)
    out = acoustic_forward(vp, model.rho.detach().cpu(), damp, loc[:, 0], loc[:, 1], wav, rl[:, 0], rl[:, 1],
                           checkpoint_segments=10, checkpoint_chunks=True, **kw)
    loss = normalised_l2(out["p"], obs, prop.dt)
    loss.backward()
    return dict(idx=idx, obs=obs, rec=out["p"].detach(), grad=vp.grad.detach(), loss=float(loss.detach()), model=model,
                survey=survey)


@pytest.mark.parametrize("snapshot_every,adjoint_source", [(0, "array"), (50, "array"), (50, "inject")])
def test_c2_full_grid_fused_l2_gradient_matches_oracle(c2_slice, snapshot_every, adjoint_source):
    """The same misfit through AcousticPropagator.forward_l2 (the CUDA misfit on the plan's
    records, obs normalised by the kernel with the same silent rule; its adjoint source as an
    array or formed inside the adjoint step)."""
    model, survey = c2_slice["model"], c2_slice["survey"]
    prop = A.AcousticPropagator(model, survey, device="cuda:0", snapshot_every=snapshot_every)
    model.vp.grad = None
    loss, rec = prop.forward_l2(c2_slice["obs"].cuda(), shot_index=c2_slice["idx"], silent_rel=1e-3,
                                normalise_obs=True, adjoint_source=adjoint_source)
    loss.backward()
    assert rel(rec["p"], c2_slice["rec"]) <= 1e-5
    assert abs(float(loss.detach()) - c2_slice["loss"]) <= 1e-5 * abs(c2_slice["loss"])
    err = rel(model.vp.grad, c2_slice["grad"])
    assert err <= 1e-4, err


@pytest.mark.parametrize("snapshot_every", [0, 50])
def test_c2_full_grid_normalised_l2_gradient_matches_oracle(c2_slice, snapshot_every):
    model, survey = c2_slice["model"], c2_slice["survey"]
    prop = A.AcousticPropagator(model, survey, device="cuda:0", snapshot_every=snapshot_every)
    model.vp.grad = None
    rec = prop.forward(shot_index=c2_slice["idx"])
    loss = normalised_l2(rec["p"], c2_slice["obs"].cuda(), prop.dt)
    loss.backward()
    assert prop.plan(c2_slice["idx"])[1].snapshot_every == (1000 if snapshot_every == 0 else 50)
    assert rel(rec["p"], c2_slice["rec"]) <= 1e-5
    assert abs(float(loss.detach()) - c2_slice["loss"]) <= 1e-5 * abs(c2_slice["loss"])
    err = rel(model.vp.grad, c2_slice["grad"])
    assert err <= 1e-4, err


# ---------------------------------------------------------------------------- 200 x 400 VTI
def test_c3_full_grid_vti_gradients_match_oracle():
    from adfwi_gb300.synthetic import vti_gradient_case
    from oracle.elastic import elastic_forward
    from oracle.model import elastic_coefficients
    _threads()
    model, survey = vti_gradient_case(seed=0, device="cuda:0", nt=200)
    prop = A.ElasticPropagator(model, survey, device="cuda:0")
    idx = [10]
    gen = torch.Generator().manual_seed(3)
    w = {k: torch.randn((1, 200, prop.rcv_n), generator=gen) for k in ("vx", "vz")}
    rec = prop.forward(shot_index=idx, fd_order=4)
    ((rec["vx"] * w["vx"].cuda()).sum() + (rec["vz"] * w["vz"].cuda()).sum()).backward()
    names = ("vp", "vs", "rho", "eps", "delta", "gamma")
    pars = {k: getattr(model, k).detach().cpu().clone().requires_grad_(True) for k in names}
    co = elastic_coefficients(*(pars[k] for k in names), "vti")
    out = elastic_forward(co, prop.src_loc[idx, 0], prop.src_loc[idx, 1], prop.wavelet.cpu()[idx],
                          prop.moment_tensor.cpu()[idx], prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=prop.nabc,
                          free_surface=True, dx=prop.dx, dz=prop.dz, dt=prop.dt, fd_order=4, abc_type="PML",
                          bcx=prop.bcx.cpu().numpy(), bcz=prop.bcz.cpu().numpy(), damp=None)
    ((out["vx"] * w["vx"]).sum() + (out["vz"] * w["vz"]).sum()).backward()
    for k in ("vx", "vz"):
        assert rel(rec[k], out[k]) <= 1e-5, k
    for k in ("vp", "vs", "rho", "eps", "delta"):
        err = rel(getattr(model, k).grad, pars[k].grad)
        assert err <= 1e-4, (k, err)


# ---------------------------------------------------------------------------- 500 x 1500, FP64
def test_c4_grid_fp64_records_and_gradient_match_oracle():
    from adfwi_gb300.synthetic import linear_gradient_with_anomaly, surface_acquisition
    from oracle.acoustic import acoustic_forward
    _threads()
    nz, nx, dx, nt, dt = 500, 1500, 12.5, 200, 1e-3
    vp = linear_gradient_with_anomaly(nz, nx)
    model = A.AcousticModel(0, 0, nx, nz, dx, dx, vp=vp, rho=np.power(vp, 0.25) * 310, vp_grad=True, nabc=50,
                            device="cuda:0", dtype=torch.float64)
    survey = surface_acquisition(nx, nt, dt, 10.0, 64)
    prop = A.AcousticPropagator(model, survey, device="cuda:0", dtype=torch.float64, snapshot_every=50)
    idx = [31]
    wts = torch.randn((1, nt, nx), generator=torch.Generator().manual_seed(4), dtype=torch.float64)
    rec = prop.forward(shot_index=idx)
    (rec["p"] * wts.cuda()).sum().backward()
    vpo = model.vp.detach().cpu().clone().requires_grad_(True)
    out = acoustic_forward(vpo, model.rho.detach().cpu(), prop.damp.cpu(), prop.src_loc[idx, 0], prop.src_loc[idx, 1],
                           prop.wavelet.cpu()[idx], prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=50,
                           free_surface=False, dx=dx, dz=dx, dt=dt)
    (out["p"] * wts).sum().backward()
    for k in KEYS:
        assert rel(rec[k], out[k]) <= 1e-12, (k, rel(rec[k], out[k]))
    err = rel(model.vp.grad, vpo.grad)
    assert err <= 1e-9, err
