"""Seeded synthetic problems shared by the tests (not a test module)."""
import glob
import os

import numpy as np
import torch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_files(kind=None):
    """Propagator fixtures (acoustic and elastic), or those of one kind."""
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        g = np.load(f)
        if "kind" not in g.files:
            continue
        k = str(g["kind"])
        if (kind is None and k in ("acoustic", "elastic")) or k == kind:
            out.append(f)
    return out


def rel(a, b):
    a = np.asarray(a.detach().cpu() if torch.is_tensor(a) else a, dtype=np.float64)
    b = np.asarray(b.detach().cpu() if torch.is_tensor(b) else b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def layered_vp(nz, nx, rng, vmin=1500.0, vmax=3000.0, n_layers=5, anomaly=250.0):
    z = np.arange(nz)[:, None].astype(np.float64)
    x = np.arange(nx)[None, :].astype(np.float64)
    vp = np.full((nz, nx), vmin)
    bounds = np.sort(rng.integers(2, max(3, nz - 2), size=n_layers))
    vals = np.sort(rng.uniform(vmin, vmax, size=n_layers))
    for b, v in zip(bounds, vals):
        dip = rng.uniform(-0.2, 0.2)
        vp = np.where(z >= b + dip * (x - nx / 2), v, vp)
    sig = max(2.0, min(nz, nx) / 8)
    vp = vp + anomaly * np.exp(-((z - nz / 2) ** 2 + (x - nx / 2) ** 2) / (2 * sig ** 2))
    return vp


def acoustic_problem(A, *, nz=40, nx=56, nabc=12, nt=250, dt=1e-3, dx=10.0, f0=20.0, ns=3, nr=20,
                     free_surface=False, dtype=torch.float32, seed=0, device="cuda:0", vp_grad=True,
                     rho_grad=True, rcv_z=2, src_z=1, **prop_kw):
    """A (model, survey, propagator) triple built through the package API ``A``."""
    rng = np.random.default_rng(seed)
    vp = layered_vp(nz, nx, rng)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    vp = vp.astype(npdt)
    rho = (np.power(vp, 0.25) * 310).astype(npdt)
    model = A.AcousticModel(0, 0, nx, nz, dx, dx, vp=vp, rho=rho, vp_grad=vp_grad, rho_grad=rho_grad,
                            free_surface=free_surface, nabc=nabc, device=device, dtype=dtype)
    src = A.Source(nt=nt, dt=dt, f0=f0)
    _, wav = A.wavelet(nt, dt, f0)
    src.add_sources(src_x=np.linspace(2, nx - 3, ns).astype(int), src_z=np.full(ns, src_z), src_wavelet=wav)
    rcv = A.Receiver(nt=nt, dt=dt)
    rcv.add_receivers(rcv_x=np.linspace(0, nx - 1, nr).astype(int), rcv_z=np.full(nr, rcv_z), rcv_type="pr")
    survey = A.Survey(src, rcv)
    prop = A.AcousticPropagator(model, survey, device=device, dtype=dtype, **prop_kw)
    return model, survey, prop


def oracle_acoustic(prop, model, shot_index=None, segments=1, requires_grad=True):
    """Run the CPU oracle on the same inputs as ``prop`` (after model.forward())."""
    from oracle.acoustic import acoustic_forward
    vp = model.vp.detach().cpu().clone().requires_grad_(requires_grad)
    rho = model.rho.detach().cpu().clone().requires_grad_(requires_grad)
    idx = np.arange(prop.src_n) if shot_index is None else np.atleast_1d(np.arange(prop.src_n)[shot_index])
    out = acoustic_forward(vp, rho, prop.damp.cpu(), prop.src_loc[idx, 0], prop.src_loc[idx, 1],
                           prop.wavelet.cpu()[idx], prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=prop.nabc,
                           free_surface=bool(prop.free_surface), dx=prop.dx, dz=prop.dz, dt=prop.dt,
                           checkpoint_segments=segments)
    return out, vp, rho


def elastic_problem(A, *, nz=30, nx=40, nabc=8, nt=160, dt=5e-4, dx=5.0, f0=40.0, ns=2, nr=12, free_surface=True,
                    fd_order=4, abc_type="PML", iso=False, dtype=torch.float32, seed=0, device="cuda:0", mt=None,
                    **prop_kw):
    """A VTI (or isotropic) elastic (model, survey, propagator) built through the package API ``A``."""
    rng = np.random.default_rng(seed)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    vp = layered_vp(nz, nx, rng, vmin=2000.0, vmax=3200.0, anomaly=200.0).astype(npdt)
    vs = (vp / 1.73).astype(npdt)
    rho = (np.power(vp, 0.25) * 310).astype(npdt)
    eps = np.clip(0.1 + 0.05 * rng.standard_normal((nz, nx)), 0.0, 0.2).astype(npdt)
    delta = np.clip(0.05 + 0.02 * rng.standard_normal((nz, nx)), 0.0, 0.1).astype(npdt)
    gamma = np.zeros((nz, nx), dtype=npdt)
    if iso:
        model = A.IsotropicElasticModel(0, 0, nx, nz, dx, dx, vp=vp, vs=vs, rho=rho, vp_grad=True, vs_grad=True,
                                        rho_grad=True, free_surface=free_surface, abc_type=abc_type, nabc=nabc,
                                        auto_update_rho=False, device=device, dtype=dtype)
    else:
        model = A.AnisotropicElasticModel(0, 0, nx, nz, dx, dx, vp=vp, vs=vs, rho=rho, eps=eps, gamma=gamma,
                                          delta=delta, vp_grad=True, vs_grad=True, rho_grad=True, eps_grad=True,
                                          delta_grad=True, free_surface=free_surface, abc_type=abc_type, nabc=nabc,
                                          device=device, dtype=dtype)
    src = A.Source(nt=nt, dt=dt, f0=f0)
    _, wav = A.wavelet(nt, dt, f0)
    kw = {} if mt is None else {"src_mt": np.asarray(mt)}
    src.add_sources(src_x=np.linspace(4, nx - 5, ns).astype(int), src_z=np.full(ns, 3), src_wavelet=wav, **kw)
    rcv = A.Receiver(nt=nt, dt=dt)
    rcv.add_receivers(rcv_x=np.linspace(2, nx - 3, nr).astype(int), rcv_z=np.full(nr, 1), rcv_type="pr")
    survey = A.Survey(src, rcv)
    prop = A.ElasticPropagator(model, survey, device=device, dtype=dtype, **prop_kw)
    return model, survey, prop


ELASTIC_KEYS = ("txx", "tzz", "txz", "vx", "vz")


def oracle_elastic(prop, model, fd_order=4, segments=1, iso=False):
    """CPU oracle on the same model parameters as ``prop``; returns (records, parameter leaves)."""
    from oracle.elastic import elastic_forward
    from oracle.model import elastic_coefficients
    names = ("vp", "vs", "rho", "eps", "delta", "gamma")
    pars = {k: getattr(model, k).detach().cpu().clone().requires_grad_(True) for k in names}
    co = elastic_coefficients(pars["vp"], pars["vs"], pars["rho"], pars["eps"], pars["delta"], pars["gamma"],
                              getattr(model, "anisotropic_type", "vti"))
    bcx = prop.bcx.cpu().numpy() if prop.bcx is not None else None
    bcz = prop.bcz.cpu().numpy() if prop.bcz is not None else None
    damp = prop.damp.cpu().numpy() if prop.damp is not None else None
    out = elastic_forward(co, prop.src_loc[:, 0], prop.src_loc[:, 1], prop.wavelet.cpu(),
                          prop.moment_tensor.cpu(), prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=prop.nabc,
                          free_surface=bool(prop.free_surface), dx=prop.dx, dz=prop.dz, dt=prop.dt,
                          fd_order=fd_order, abc_type=prop.abc_type, bcx=bcx, bcz=bcz, damp=damp,
                          checkpoint_segments=segments)
    return out, pars
