"""Seeded synthetic models and acquisitions for the benchmark workloads.

No public dataset is involved: every workload is generated from ``numpy.random.default_rng``
with the shapes, sizes and value distributions of the named configurations:

* ``linear_gradient_with_anomaly``: vp linear 1500 -> 3000 m/s with depth plus a Gaussian
  +300 m/s bump (sigma 8 cells) at the centre (the 100 x 100 CPU-runnable case);
* ``layered_faulted``: n dipping interfaces (random dips within +-15 degrees), layer
  velocities uniform in [vmin, vmax] sorted to increase with depth, plus random normal faults
  with 5-20 cell throws (the 200 x 600 gradient case); ``smooth`` gives the Gaussian-smoothed
  starting model;
* ``surface_acquisition``: evenly spaced surface shots and a receiver at every column.
"""
import numpy as np

from .model import AcousticModel, AnisotropicElasticModel
from .survey import Receiver, Source, Survey
from .utils import wavelet


def linear_gradient_with_anomaly(nz, nx, vmin=1500.0, vmax=3000.0, bump=300.0, sigma=8.0):
    z = np.arange(nz)[:, None]
    x = np.arange(nx)[None, :]
    vp = vmin + (vmax - vmin) * z / max(nz - 1, 1) + np.zeros((1, nx))
    vp = vp + bump * np.exp(-((z - nz / 2) ** 2 + (x - nx / 2) ** 2) / (2 * sigma ** 2))
    return vp


def layered_faulted(nz, nx, rng, n_interfaces=12, vmin=1500.0, vmax=4700.0, n_faults=2, max_dip_deg=15.0,
                    throw=(5, 20)):
    """Layered model with dipping interfaces and normal faults (velocity grows with depth)."""
    x = np.arange(nx)[None, :].astype(np.float64)
    z = np.arange(nz)[:, None].astype(np.float64)
    depths = np.sort(rng.uniform(0.04 * nz, 0.96 * nz, size=n_interfaces))
    dips = np.tan(np.deg2rad(rng.uniform(-max_dip_deg, max_dip_deg, size=n_interfaces)))
    vel = np.sort(rng.uniform(vmin, vmax, size=n_interfaces + 1))
    # layer index of every cell: number of interfaces above it
    layer = np.zeros((nz, nx), dtype=np.int64)
    for d, s in zip(depths, dips):
        layer += (z >= d + s * (x - nx / 2)).astype(np.int64)
    # normal faults: cells on the hanging-wall side of a dipping fault plane slip down by `t`
    for _ in range(n_faults):
        x0 = rng.uniform(0.2 * nx, 0.8 * nx)
        fdip = np.tan(np.deg2rad(rng.uniform(50.0, 70.0))) * rng.choice([-1.0, 1.0])
        t = int(rng.integers(throw[0], throw[1] + 1))
        hanging = (x - x0) * fdip > z  # one side of the plane x = x0 + z / fdip
        shifted = np.vstack([np.repeat(layer[:1], t, axis=0), layer[:-t]]) if t < nz else layer
        layer = np.where(hanging, shifted, layer)
    return vel[np.clip(layer, 0, n_interfaces)]


def smooth(v, sigma=10.0):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(v, sigma=sigma, mode="nearest")


def surface_acquisition(nx, nt, dt, f0, n_shots, src_z=2, rcv_z=2, n_rcv=None, moment_tensor=None):
    src = Source(nt=nt, dt=dt, f0=f0)
    _, wav = wavelet(nt, dt, f0)
    sx = np.linspace(0, nx - 1, n_shots + 2)[1:-1].round().astype(int) if n_shots > 1 else np.array([nx // 2])
    kw = {} if moment_tensor is None else {"src_mt": np.asarray(moment_tensor)}
    src.add_sources(src_x=sx, src_z=np.full(len(sx), src_z), src_wavelet=wav, **kw)
    rcv = Receiver(nt=nt, dt=dt)
    n_rcv = nx if n_rcv is None else n_rcv
    rx = np.linspace(0, nx - 1, n_rcv).round().astype(int)
    rcv.add_receivers(rcv_x=rx, rcv_z=np.full(len(rx), rcv_z), rcv_type="pr")
    return Survey(src, rcv)


def acoustic_gradient_case(seed=0, nz=200, nx=600, dx=20.0, nt=3000, dt=1.5e-3, f0=8.0, n_shots=30, nabc=50,
                           device="cuda:0", dtype=None):
    """True and starting models plus survey of the 200 x 600 layered/faulted gradient workload."""
    import torch
    dtype = torch.float32 if dtype is None else dtype
    rng = np.random.default_rng(seed)
    vp_true = layered_faulted(nz, nx, rng)
    vp_init = smooth(vp_true, 10.0)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    vp_true, vp_init = vp_true.astype(npdt), vp_init.astype(npdt)
    rho = (np.power(vp_init, 0.25) * 310).astype(npdt)
    survey = surface_acquisition(nx, nt, dt, f0, n_shots)
    model = AcousticModel(0, 0, nx, nz, dx, dx, vp=vp_init, rho=rho, vp_grad=True, nabc=nabc, device=device,
                          dtype=dtype)
    return model, survey, vp_true, vp_init


def vti_layered(nz, nx, rng, n_layers=8, vmin=2000.0, vmax=4500.0):
    """VTI layered model: vp U(vmin, vmax) increasing with depth, vs = vp/1.73, Gardner rho,
    eps U(0, 0.2) and delta U(0, 0.1) per layer, gamma = 0."""
    depths = np.sort(rng.uniform(0.05 * nz, 0.95 * nz, size=n_layers - 1))
    z = np.arange(nz)[:, None] + np.zeros((1, nx))
    layer = np.zeros((nz, nx), dtype=np.int64)
    for d in depths:
        layer += (z >= d).astype(np.int64)
    vp = np.sort(rng.uniform(vmin, vmax, size=n_layers))[layer]
    eps = rng.uniform(0.0, 0.2, size=n_layers)[layer]
    delta = rng.uniform(0.0, 0.1, size=n_layers)[layer]
    vs = vp / 1.73
    rho = np.power(vp, 0.25) * 310
    return vp, vs, rho, eps, delta, np.zeros((nz, nx))


def vti_gradient_case(seed=0, nz=200, nx=400, dx=10.0, nt=2000, dt=8e-4, f0=15.0, n_shots=20, nabc=40,
                      device="cuda:0", dtype=None, free_surface=True):
    import torch
    dtype = torch.float32 if dtype is None else dtype
    rng = np.random.default_rng(seed)
    vp, vs, rho, eps, delta, gamma = vti_layered(nz, nx, rng)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    cast = [a.astype(npdt) for a in (vp, vs, rho, eps, delta, gamma)]
    model = AnisotropicElasticModel(0, 0, nx, nz, dx, dx, *cast[:3], eps=cast[3], gamma=cast[5], delta=cast[4],
                                    vp_grad=True, vs_grad=True, rho_grad=True, eps_grad=True, delta_grad=True,
                                    free_surface=free_surface, nabc=nabc, device=device, dtype=dtype)
    survey = surface_acquisition(nx, nt, dt, f0, n_shots, src_z=2, rcv_z=1)
    return model, survey
