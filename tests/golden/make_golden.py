"""Generate the golden fixtures in this directory by running the ADFWI reference itself.

This script is test infrastructure. It imports the read-only reference package
(pure Python + PyTorch) on the CPU through a stub importer for the plotting /
optional dependencies that are absent here (matplotlib, h5py, skimage, ...).
None of those stubs touch the propagator arithmetic:
``ADFWI/propagator/acoustic_kernels.py`` and ``elastic_kernels.py`` only need
torch and numpy.

``gradproc.npz`` holds the reference's ``smooth2d`` and ``GradProcessor.forward`` outputs on
seeded inputs. ``acoustic_c1_full.npz`` is the 100 x 100 forward-only configuration at its full
size (PML 50, 10 shots, nt = 1000): its inputs, the reference's forward_wavefield_* maps, every
10th time sample of the pressure records and the FP64 energy of every record trace (the full
records would be 12 MB). ``seismicdata_ref.npz`` is a file written by the reference's
``SeismicData.save``, and ``seismicdata_ours_read_by_ref.npz`` holds what the reference's
``SeismicData.load`` read back from a file written by this package's ``save``. Each propagator fixture holds the inputs of one small case, the reference's record dict
(``AcousticPropagator.forward`` / ``ElasticPropagator.forward``), its damping
arrays, and autograd gradients of a fixed linear functional of the records
(``sum_k <W_k, rec_k>`` with seeded weights), so that gradient parity does
not depend on the singular sqrt-L2 misfit at zero residual.

Usage (from the repository root, in a container that has the reference):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import importlib.abc
import importlib.machinery
import os
import sys
from unittest.mock import MagicMock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_STUBBED = {"matplotlib", "mpl_toolkits", "h5py", "skimage", "geomloss", "pysdtw", "ot",
            "ncg_optimizer", "obspy", "netCDF4", "disba", "seaborn", "torchinfo", "numba", "tqdm"}


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    """Serve MagicMock modules for optional packages the reference imports at module level."""

    def find_spec(self, name, path, target=None):
        if name.split(".")[0] in _STUBBED:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = MagicMock(name=spec.name)
        m.__path__ = []
        m.__spec__ = spec
        return m

    def exec_module(self, module):
        return None


def import_reference(ref_root):
    sys.dont_write_bytecode = True
    sys.meta_path.insert(0, _StubFinder())
    sys.path.insert(0, ref_root)
    import ADFWI  # noqa: F401
    from ADFWI.model import AcousticModel, AnisotropicElasticModel, IsotropicElasticModel
    from ADFWI.survey import Source, Receiver, Survey
    from ADFWI.propagator import AcousticPropagator, ElasticPropagator
    from ADFWI.utils import wavelet
    return dict(AcousticModel=AcousticModel, AnisotropicElasticModel=AnisotropicElasticModel,
                IsotropicElasticModel=IsotropicElasticModel, Source=Source, Receiver=Receiver,
                Survey=Survey, AcousticPropagator=AcousticPropagator,
                ElasticPropagator=ElasticPropagator, wavelet=wavelet)


def layered_vp(nz, nx, vmin, vmax, rng, n_layers=4, anomaly=300.0):
    """Layered velocity increasing with depth plus a Gaussian bump (seeded)."""
    z = np.arange(nz)[:, None].astype(np.float64)
    x = np.arange(nx)[None, :].astype(np.float64)
    vp = np.full((nz, nx), vmin)
    bounds = np.sort(rng.integers(2, nz - 2, size=n_layers))
    vals = np.sort(rng.uniform(vmin, vmax, size=n_layers))
    for b, v in zip(bounds, vals):
        dip = rng.uniform(-0.15, 0.15)
        vp = np.where(z >= b + dip * (x - nx / 2), v, vp)
    vp = vp + anomaly * np.exp(-((z - nz / 2) ** 2 + (x - nx / 2) ** 2) / (2 * 3.0 ** 2))
    return vp


def build_survey(R, nt, dt, f0, src_x, src_z, rcv_x, rcv_z, mt=None):
    src = R["Source"](nt=nt, dt=dt, f0=f0)
    _, wav = R["wavelet"](nt, dt, f0, amp0=1.0)
    kw = {} if mt is None else {"src_mt": mt}
    src.add_sources(src_x=np.asarray(src_x), src_z=np.asarray(src_z), src_wavelet=wav, src_type="mt", **kw)
    rcv = R["Receiver"](nt=nt, dt=dt)
    rcv.add_receivers(rcv_x=np.asarray(rcv_x), rcv_z=np.asarray(rcv_z), rcv_type="pr")
    return R["Survey"](source=src, receiver=rcv), wav


def acoustic_case(R, name, *, nz, nx, nabc, nt, dt, dx, f0, ns, nr, free_surface, segments,
                  dtype_name, seed):
    import torch
    rng = np.random.default_rng(seed)
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    torch.set_default_dtype(dtype)
    vp = layered_vp(nz, nx, 1500.0, 2500.0, rng)
    rho = np.power(vp, 0.25) * 310.0
    if dtype_name == "f32":
        vp = vp.astype(np.float32)
        rho = rho.astype(np.float32)
    model = R["AcousticModel"](0, 0, nx, nz, dx, dx, vp=vp, rho=rho, vp_grad=True, rho_grad=True,
                               free_surface=free_surface, abc_type="PML", nabc=nabc,
                               device="cpu", dtype=dtype)
    src_x = np.linspace(3, nx - 4, ns).astype(int)
    src_z = np.full(ns, 2, dtype=int)
    rcv_x = np.linspace(1, nx - 2, nr).astype(int)
    rcv_z = np.full(nr, 3, dtype=int)
    survey, wav = build_survey(R, nt, dt, f0, src_x, src_z, rcv_x, rcv_z)
    prop = R["AcousticPropagator"](model, survey, device="cpu", dtype=dtype)
    rec = prop.forward(checkpoint_segments=segments)
    weights = {k: rng.standard_normal(rec[k].shape) for k in ("p", "u", "w")}
    loss = sum((rec[k] * torch.tensor(weights[k], dtype=dtype)).sum() for k in ("p", "u", "w"))
    loss.backward()
    out = dict(kind="acoustic", dtype=dtype_name, nz=nz, nx=nx, nabc=nabc, nt=nt, dt=dt, dx=dx,
               f0=f0, free_surface=free_surface, segments=segments,
               vp_in=vp, rho_in=rho,
               vp=model.vp.detach().numpy(), rho=model.rho.detach().numpy(),
               damp=prop.damp.numpy(), wavelet=prop.wavelet.numpy(),
               src_x=src_x, src_z=src_z, rcv_x=rcv_x, rcv_z=rcv_z,
               grad_vp=model.vp.grad.numpy(), grad_rho=model.rho.grad.numpy(), loss=loss.item())
    for k, v in rec.items():
        out["rec_" + k] = v.detach().numpy()
    for k, v in weights.items():
        out["w_" + k] = v
    torch.set_default_dtype(torch.float32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, {k: np.asarray(v).shape for k, v in out.items() if isinstance(v, np.ndarray)})


def elastic_case(R, name, *, nz, nx, nabc, nt, dt, dx, f0, ns, nr, free_surface, fd_order,
                 abc_type, iso, segments, dtype_name, seed, mt=None):
    import torch
    rng = np.random.default_rng(seed)
    dtype = torch.float64 if dtype_name == "f64" else torch.float32
    torch.set_default_dtype(dtype)
    vp = layered_vp(nz, nx, 2000.0, 3200.0, rng, anomaly=200.0)
    vs = vp / 1.73
    rho = np.power(vp, 0.25) * 310.0
    eps = np.clip(0.1 + 0.05 * rng.standard_normal((nz, nx)), 0.0, 0.2)
    delta = np.clip(0.05 + 0.02 * rng.standard_normal((nz, nx)), 0.0, 0.1)
    gamma = np.zeros((nz, nx))
    cast = (lambda a: a.astype(np.float32)) if dtype_name == "f32" else (lambda a: a)
    vp, vs, rho, eps, delta, gamma = map(cast, (vp, vs, rho, eps, delta, gamma))
    if iso:
        model = R["IsotropicElasticModel"](0, 0, nx, nz, dx, dx, vp=vp, vs=vs, rho=rho,
                                           vp_grad=True, vs_grad=True, rho_grad=True,
                                           free_surface=free_surface, abc_type=abc_type, nabc=nabc,
                                           auto_update_rho=False, device="cpu", dtype=dtype)
    else:
        model = R["AnisotropicElasticModel"](0, 0, nx, nz, dx, dx, vp=vp, vs=vs, rho=rho, eps=eps,
                                             gamma=gamma, delta=delta, vp_grad=True, vs_grad=True,
                                             rho_grad=True, eps_grad=True, delta_grad=True,
                                             free_surface=free_surface, abc_type=abc_type,
                                             nabc=nabc, device="cpu", dtype=dtype)
    src_x = np.linspace(4, nx - 5, ns).astype(int)
    src_z = np.full(ns, 3, dtype=int)
    rcv_x = np.linspace(2, nx - 3, nr).astype(int)
    rcv_z = np.full(nr, 1, dtype=int)
    survey, wav = build_survey(R, nt, dt, f0, src_x, src_z, rcv_x, rcv_z, mt=mt)
    prop = R["ElasticPropagator"](model, survey, device="cpu", dtype=dtype)
    rec = prop.forward(fd_order=fd_order, checkpoint_segments=segments)
    comps = ("txx", "tzz", "txz", "vx", "vz")
    weights = {k: rng.standard_normal(rec[k].shape) for k in comps}
    loss = sum((rec[k] * torch.tensor(weights[k], dtype=dtype)).sum() for k in comps)
    loss.backward()
    out = dict(kind="elastic", dtype=dtype_name, nz=nz, nx=nx, nabc=nabc, nt=nt, dt=dt, dx=dx,
               f0=f0, free_surface=free_surface, fd_order=fd_order, abc_type=abc_type, iso=iso,
               segments=segments, vp=vp, vs=vs, rho=rho, eps=eps, delta=delta, gamma=gamma,
               wavelet=prop.wavelet.numpy(), moment_tensor=prop.moment_tensor.numpy(),
               src_x=src_x, src_z=src_z, rcv_x=rcv_x, rcv_z=rcv_z, loss=loss.item())
    if prop.bcx is not None:
        out["bcx"] = prop.bcx.numpy()
        out["bcz"] = prop.bcz.numpy()
    if prop.damp is not None:
        out["damp"] = prop.damp.numpy()
    pars = ("vp", "vs", "rho") if iso else ("vp", "vs", "rho", "eps", "delta")
    for p in pars:
        g = getattr(model, p).grad
        out["grad_" + p] = g.numpy()
    for k, v in rec.items():
        out["rec_" + k] = v.detach().numpy()
    for k, v in weights.items():
        out["w_" + k] = v
    torch.set_default_dtype(torch.float32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, {k: np.asarray(v).shape for k, v in out.items() if isinstance(v, np.ndarray)})


def gradproc_cases(ref_root):
    """Fixtures of the reference's GradProcessor (gradient_process.py:74-134) and smooth2d.

    scipy 1.13 removed ``scipy.signal.hamming`` (the window lives in ``scipy.signal.windows``);
    the land taper of the reference calls the old name, so this script points the old name at
    the window before calling it. Nothing else is changed."""
    import scipy.signal
    if not hasattr(scipy.signal, "hamming"):
        scipy.signal.hamming = scipy.signal.windows.hamming
    from ADFWI.propagator import gradient_process as G
    rng = np.random.default_rng(31)
    out = {"kind": "gradproc"}
    z = rng.standard_normal((37, 53))
    for span in (3, 10, 40):
        out["smooth_in"] = z
        out["smooth_%d" % span] = G.smooth2d(z, span=span)
    cases = [
        ("land_mute_smooth", dict(grad_mute=6, grad_smooth=3, norm_grad=True, forw_illumination=True,
                                  marine_or_land="land"), (48, 64), True, False),
        ("marine_mute_smooth_mask", dict(grad_mute=5, grad_smooth=2, norm_grad=True, forw_illumination=True,
                                         marine_or_land="marine"), (36, 50), True, True),
        ("plain_no_forw", dict(grad_mute=0, grad_smooth=0, norm_grad=False, forw_illumination=True,
                               marine_or_land="land"), (30, 44), False, False),
        ("marine_no_forw_f32", dict(grad_mute=4, grad_smooth=3, norm_grad=True, forw_illumination=True,
                                    marine_or_land="marine"), (40, 45), False, False),
    ]
    for name, kw, (nz, nx), with_forw, with_mask in cases:
        grad = rng.standard_normal((nz, nx)).astype(np.float32)
        forw = (rng.random((nz, nx)) ** 3).astype(np.float32) if with_forw else None
        mask = (rng.random((nz, nx)) > 0.2).astype(np.float32) if with_mask else None
        gp = G.GradProcessor(grad_mask=mask, **kw)
        res = gp.forward(nx=nx, nz=nz, vmax=3000.0, grad=grad.copy(), forw=None if forw is None else forw.copy())
        out[name + "_grad"] = grad
        if forw is not None:
            out[name + "_forw"] = forw
        if mask is not None:
            out[name + "_mask"] = mask
        out[name + "_out"] = np.asarray(res)
        for k, v in kw.items():
            out[name + "_" + k] = v
    np.savez_compressed(os.path.join(HERE, "gradproc.npz"), **out)
    print("gradproc", sorted(out))


def c1_full_case(R):
    """The 100 x 100 forward-only configuration at full size, run by the reference: vp linear
    1500 -> 3000 m/s with depth plus a +300 m/s Gaussian bump (sigma 8 cells) at the centre, rho
    set by the model's own Gardner map, dx = 10 m, PML 50, no free surface, nt = 1000, dt = 1 ms,
    10 Hz Ricker, 10 shots at z = 2 evenly spaced in x, 100 receivers at every x, z = 2."""
    import torch
    torch.set_default_dtype(torch.float32)
    nz = nx = 100
    z = np.arange(nz)[:, None]
    x = np.arange(nx)[None, :]
    vp = 1500.0 + 1500.0 * z / (nz - 1) + np.zeros((1, nx))
    vp = (vp + 300.0 * np.exp(-((z - nz / 2) ** 2 + (x - nx / 2) ** 2) / (2 * 8.0 ** 2))).astype(np.float32)
    rho = (np.power(vp, 0.25) * 310).astype(np.float32)
    model = R["AcousticModel"](0, 0, nx, nz, 10.0, 10.0, vp=vp, rho=rho, free_surface=False, abc_type="PML",
                               nabc=50, device="cpu", dtype=torch.float32)
    src_x = np.linspace(0, nx - 1, 12)[1:-1].round().astype(int)
    src_z = np.full(10, 2, dtype=int)
    rcv_x = np.arange(nx)
    rcv_z = np.full(nx, 2, dtype=int)
    survey, _ = build_survey(R, 1000, 1e-3, 10.0, src_x, src_z, rcv_x, rcv_z)
    prop = R["AcousticPropagator"](model, survey, device="cpu", dtype=torch.float32)
    with torch.no_grad():
        rec = prop.forward()
    out = dict(kind="acoustic_full", nz=nz, nx=nx, nabc=50, nt=1000, dt=1e-3, dx=10.0, f0=10.0,
               free_surface=False, vp_in=vp, src_x=src_x, src_z=src_z, rcv_x=rcv_x, rcv_z=rcv_z,
               damp=prop.damp.numpy(), decimate=10)
    for k in ("p", "u", "w"):
        r = rec[k].numpy()
        out["energy_" + k] = np.sum(r.astype(np.float64) ** 2, axis=1)  # (ns, nr)
    out["rec_p_dec"] = rec["p"].numpy()[:, ::10, :]
    for k in ("p", "u", "w"):
        out["forward_wavefield_" + k] = rec["forward_wavefield_" + k].numpy()
    np.savez_compressed(os.path.join(HERE, "acoustic_c1_full.npz"), **out)
    print("acoustic_c1_full", {k: np.asarray(v).shape for k, v in out.items() if isinstance(v, np.ndarray)})


def seismic_data_files(R):
    """A file written by the reference's SeismicData.save, and what its load reads from a file
    written by this package's SeismicData.save (both from the same seeded survey and records)."""
    import tempfile
    import torch
    from ADFWI.survey import SeismicData as RefSeismicData
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import adfwi_gb300 as A
    sys.path.insert(0, HERE)
    from seismic_case import seismic_data_case

    # the reference's survey and data
    sv_ref, recs = seismic_data_case(R["Source"], R["Receiver"], R["Survey"], R["wavelet"])
    d = RefSeismicData(sv_ref)
    d.record_data({k: torch.tensor(v) for k, v in recs.items()})
    d.save(os.path.join(HERE, "seismicdata_ref.npz"))
    # ours, read back by the reference
    sv_ours, recs2 = seismic_data_case(A.Source, A.Receiver, A.Survey, A.wavelet)
    e = A.SeismicData(sv_ours)
    e.record_data({k: torch.tensor(v) for k, v in recs2.items()})
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "ours.npz")
        e.save(path)
        f = RefSeismicData(sv_ref)
        f.load(path)
    out = {"kind": "seismicdata"}
    for k, v in f.data.items():
        out["data_" + k] = v
    for k in ("src_loc", "rcv_loc", "src_num", "rcv_num", "rcv_type", "src_type", "t", "nt", "dt"):
        out[k] = np.asarray(getattr(f, k))
    np.savez_compressed(os.path.join(HERE, "seismicdata_ours_read_by_ref.npz"), **out)
    print("seismicdata", sorted(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", choices=["gradproc", "c1", "seismicdata"], default=None,
                    help="regenerate one fixture family only")
    ap.add_argument("--read-with-reference", default=None, metavar="NPZ",
                    help="load NPZ with the reference's SeismicData.load and print a JSON digest of its records")
    args = ap.parse_args()
    R = import_reference(args.ref)
    if args.read_with_reference:
        import json
        from ADFWI.survey import SeismicData as RefSeismicData
        sys.path.insert(0, HERE)
        from seismic_case import seismic_data_case
        sv, _ = seismic_data_case(R["Source"], R["Receiver"], R["Survey"], R["wavelet"])
        f = RefSeismicData(sv)
        f.load(args.read_with_reference)
        dig = {k: [list(v.shape), str(v.dtype), float(np.float64(v).sum()), float(np.abs(np.float64(v)).sum())]
               for k, v in f.data.items()}
        print(json.dumps({"data": dig}))
        return
    if args.only == "gradproc":
        gradproc_cases(args.ref)
        return
    if args.only == "c1":
        c1_full_case(R)
        return
    if args.only == "seismicdata":
        seismic_data_files(R)
        return
    import torch
    torch.set_num_threads(min(8, os.cpu_count() or 1))
    ac = dict(nz=24, nx=32, nabc=8, dt=1e-3, dx=10.0, f0=25.0, ns=3, nr=12)
    acoustic_case(R, "acoustic_pml_f32", nt=80, free_surface=False, segments=1, dtype_name="f32", seed=1, **ac)
    acoustic_case(R, "acoustic_fs_seg3_f32", nt=90, free_surface=True, segments=3, dtype_name="f32", seed=2, **ac)
    acoustic_case(R, "acoustic_pml_f64", nt=80, free_surface=False, segments=2, dtype_name="f64", seed=3, **ac)
    el = dict(nz=20, nx=28, nabc=6, dt=5e-4, dx=5.0, f0=40.0, ns=2, nr=9)
    elastic_case(R, "elastic_vti_o4_pml_fs_f32", nt=70, free_surface=True, fd_order=4, abc_type="PML",
                 iso=False, segments=1, dtype_name="f32", seed=11, **el)
    elastic_case(R, "elastic_vti_o6_pml_f32", nt=70, free_surface=False, fd_order=6, abc_type="PML",
                 iso=False, segments=2, dtype_name="f32", seed=12, **el)
    elastic_case(R, "elastic_iso_o4_pml_f32", nt=70, free_surface=False, fd_order=4, abc_type="PML",
                 iso=True, segments=1, dtype_name="f32", seed=13,
                 mt=np.array([[1.0, 0.0, 0.4], [0.0, 1.0, 0.0], [0.4, 0.0, 0.6]]), **el)
    elastic_case(R, "elastic_vti_o4_gerjan_fs_f32", nt=70, free_surface=True, fd_order=4,
                 abc_type="gerjan", iso=False, segments=1, dtype_name="f32", seed=14, **el)
    elastic_case(R, "elastic_vti_o6_sincos_fs_f32", nt=70, free_surface=True, fd_order=6,
                 abc_type="sincos", iso=False, segments=1, dtype_name="f32", seed=15, **el)
    gradproc_cases(args.ref)
    c1_full_case(R)
    seismic_data_files(R)
    # No FP64 elastic fixture: the reference's DiffCoef (elastic_kernels.py:37-56) builds its
    # right-hand side in the default dtype and its matrix in float32, so the elastic propagator
    # raises "expected scalar type Float but found Double" under a float64 default dtype.


if __name__ == "__main__":
    main()
