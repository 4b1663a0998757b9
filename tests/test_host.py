"""Host-side logic on the CPU: boundary profiles, model maps, survey API, the C ABI library
(loads, exports every declared symbol, builds plans and sizes workspaces without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300 import boundary as B
from _cases import golden_files, rel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1])
def test_boundary_profiles_match_reference(path):
    g = np.load(path)
    nz, nx, nabc, dx = int(g["nz"]), int(g["nx"]), int(g["nabc"]), float(g["dx"])
    fs = bool(g["free_surface"])
    cast = np.float64 if str(g["dtype"]) == "f64" else np.float32
    if str(g["kind"]) == "acoustic":
        d = B.bc_pml(nx, nz, dx, dx, nabc, g["vp"].max(), free_surface=False)
        assert np.array_equal(d.astype(cast), g["damp"])
        return
    abc = str(g["abc_type"])
    if abc == "PML":
        bx, bz = B.bc_pml_xz(nx, nz, dx, dx, nabc, g["vp"].max(), free_surface=fs)
        assert np.array_equal(bx.astype(cast), g["bcx"]) and np.array_equal(bz.astype(cast), g["bcz"])
    elif abc == "gerjan":
        assert np.array_equal(B.bc_gerjan(nx, nz, dx, dx, nabc, 0.0053, free_surface=fs).astype(cast), g["damp"])
    else:
        assert np.array_equal(B.bc_sincos(nx, nz, dx, dx, nabc, free_surface=fs).astype(cast), g["damp"])


def test_pml_corner_rule_is_max_of_profiles():
    d = B.bc_pml(30, 20, 10.0, 10.0, 8, 3000.0, free_surface=False)
    pz, px = d[:, 8 + 15], d[8 + 10, :]
    assert np.array_equal(np.maximum(pz[:, None], px[None, :]), d)


@pytest.mark.parametrize("path", golden_files("elastic"), ids=lambda p: p.split("/")[-1])
def test_elastic_model_maps_match_oracle(path):
    from oracle.model import elastic_coefficients
    g = np.load(path)
    iso = bool(g["iso"])
    nz, nx, dx = int(g["nz"]), int(g["nx"]), float(g["dx"])
    if iso:
        m = A.IsotropicElasticModel(0, 0, nx, nz, dx, dx, vp=g["vp"], vs=g["vs"], rho=g["rho"],
                                    auto_update_rho=False)
    else:
        m = A.AnisotropicElasticModel(0, 0, nx, nz, dx, dx, vp=g["vp"], vs=g["vs"], rho=g["rho"], eps=g["eps"],
                                      gamma=g["gamma"], delta=g["delta"])
    m.forward()
    z = lambda k: torch.tensor(g[k] * (0 if iso else 1), dtype=torch.float32)  # noqa: E731
    co = elastic_coefficients(torch.tensor(g["vp"]), torch.tensor(g["vs"]), torch.tensor(g["rho"]),
                              z("eps"), z("delta"), z("gamma"))
    mine = {"C11": m.CC[0], "C13": m.CC[2], "C15": m.CC[4], "C33": m.CC[11], "C35": m.CC[13], "C55": m.CC[18],
            "bx": m.bx, "bz": m.bz}
    for k, v in co.items():
        assert torch.equal(mine[k].detach(), v.detach()), k


def test_acoustic_model_gardner_and_bounds():
    vp = np.full((6, 7), 2000.0, dtype=np.float32)
    vp[2, 3] = 3000.0
    m = A.AcousticModel(0, 0, 7, 6, 5.0, 5.0, vp=vp, rho=np.ones_like(vp), vp_bound=(1500.0, 4000.0), vp_grad=True)
    m.vp.data[0, 0] = 9000.0  # an update that leaves the bounds is clipped by forward()
    m.forward()
    assert float(m.vp.detach().max()) <= 4000.0 + 1e-3
    assert np.allclose(m.rho.detach().numpy(), np.power(m.vp.detach().numpy(), 0.25) * 310)
    assert m.get_bound("vp")[1] >= 4000.0
    with pytest.raises(ValueError):
        m.get_model("vs")
    with pytest.raises(AssertionError):
        A.AcousticModel(0, 0, 7, 6, 5.0, 6.0, vp=vp, rho=vp)


def test_survey_and_seismic_data_roundtrip(tmp_path):
    src = A.Source(nt=50, dt=1e-3, f0=10.0)
    t, w = A.wavelet(50, 1e-3, 10.0)
    src.add_sources(src_x=np.array([1, 5, 9]), src_z=np.array([2, 2, 2]), src_wavelet=w)
    src.add_source(4, 3, w)
    assert src.num == 4 and src.get_wavelet().shape == (4, 50) and src.get_moment_tensor().shape == (4, 3, 3)
    assert np.array_equal(src.get_loc(), np.array([[1, 2], [5, 2], [9, 2], [4, 3]]))
    with pytest.raises(ValueError):
        src.add_source(1, 1, w[:10])
    rcv = A.Receiver(nt=50, dt=1e-3)
    rcv.add_receivers(rcv_x=np.arange(10), rcv_z=np.zeros(10, dtype=int), rcv_type="pr")
    with pytest.raises(ValueError):
        rcv.add_receiver(1, 1, "xx")
    sv = A.Survey(src, rcv)
    d = A.SeismicData(sv)
    d.record_data({"p": torch.ones(4, 50, 10)})
    d.save(str(tmp_path / "d.npz"))
    e = A.SeismicData(sv)
    e.load(str(tmp_path / "d.npz"))
    assert np.array_equal(e.data["p"], np.ones((4, 50, 10)))


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.split("/")[-1])
def test_wavelet_matches_reference(path):
    g = np.load(path)
    _, w = A.wavelet(int(g["nt"]), float(g["dt"]), float(g["f0"]))
    cast = np.float64 if str(g["dtype"]) == "f64" else np.float32
    assert np.array_equal(w.astype(cast), g["wavelet"][0])


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "adfwi_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(adfwi_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native_lib):
    names = _declared_symbols()
    assert "adfwi_acoustic_forward" in names
    missing = [n for n in names if not hasattr(native_lib, n)]
    assert not missing, missing
    assert b"sm_103a" in native_lib.adfwi_version()


def _plan(**kw):
    from adfwi_gb300.acoustic import AcousticPlan
    base = dict(nz=200, nx=600, nabc=50, free_surface=False, src_z=[2] * 30,
                src_x=np.linspace(0, 599, 30).astype(int), rcv_z=[2] * 600, rcv_x=np.arange(600), nt=3000,
                dt=1.5e-3, dtype=torch.float32)
    base.update(kw)
    return AcousticPlan(**base)


def test_plan_workspace_sizing_and_budget(native_lib):
    p = _plan()
    fwd = p.workspace_bytes(False)
    assert 0 < fwd < 1 << 30
    full = _plan(memory_budget=1 << 40)
    assert full.snapshot_every == 3000  # everything fits: no recomputation
    tight = _plan(memory_budget=12 << 30)
    assert 1 <= tight.snapshot_every < 3000
    assert tight.workspace_bytes(True) <= 12 << 30
    fixed = _plan(snapshot_every=50, snapshot_precision="bf16")
    assert fixed.snapshot_every == 50
    assert fixed.workspace_bytes(True) < _plan(snapshot_every=50).workspace_bytes(True)


def test_plan_rejects_bad_geometry(native_lib):
    with pytest.raises(RuntimeError, match="outside"):
        _plan(src_z=[500] * 30)
    with pytest.raises(RuntimeError, match="outside"):
        _plan(rcv_x=np.arange(600) + 100)
    with pytest.raises(ValueError):
        _plan(snapshot_precision="int8")


def test_propagator_refuses_cpu_device():
    vp = np.full((10, 12), 2000.0, dtype=np.float32)
    m = A.AcousticModel(0, 0, 12, 10, 5.0, 5.0, vp=vp, rho=vp, nabc=4)
    src = A.Source(nt=10, dt=1e-3, f0=10.0)
    src.add_source(3, 2, A.wavelet(10, 1e-3, 10.0)[1])
    rcv = A.Receiver(nt=10, dt=1e-3)
    rcv.add_receiver(4, 1, "pr")
    with pytest.raises(RuntimeError, match="CUDA"):
        A.AcousticPropagator(m, A.Survey(src, rcv), device="cpu")


def test_batched_plan_geometry_on_the_host(native_lib):
    """A batched plan (several models, shots grouped by model) builds on the host and sizes a
    workspace with one coefficient block per model; unordered shot models are rejected."""
    from adfwi_gb300.acoustic import AcousticPlan
    kw = dict(nz=20, nx=30, nabc=8, free_surface=False, rcv_z=[2], rcv_x=[4], nt=10, dt=1e-3, dtype=torch.float32)
    one = AcousticPlan(src_z=[1, 1, 1], src_x=[3, 9, 15], **kw)
    two = AcousticPlan(src_z=[1, 1, 1], src_x=[3, 9, 15], shot_model=[0, 0, 1], **kw)
    assert two.nm == 2 and native_lib.adfwi_acoustic_plan_models(two.handle) == 2
    assert two.workspace_bytes(False) > one.workspace_bytes(False)
    with pytest.raises(RuntimeError, match="non-decreasing"):
        AcousticPlan(src_z=[1, 1, 1], src_x=[3, 9, 15], shot_model=[1, 0, 0], **kw)
    with pytest.raises(RuntimeError, match="has no shot"):
        AcousticPlan(src_z=[1, 1], src_x=[3, 9], shot_model=[0, 2], **kw)


@pytest.mark.parametrize("pads", [(3, 2, 4, 1), (0, 5, 2, 2), (2, 0, 0, 3), (0, 0, 0, 0), (1, 1, 1, 1)])
def test_replicate_pad_backward_is_the_fold(pads):
    """The propagators' edge-replicate padding (acoustic_kernels.py:16-37) differentiates by
    the explicit fold, equal to autograd through torch's replicate pad."""
    import torch
    from adfwi_gb300.propagator import _pad_replicate, fold_replicate
    top, bottom, left, right = pads
    g = torch.Generator().manual_seed(1)
    v = torch.randn(7, 9, generator=g, dtype=torch.float64, requires_grad=True)
    w = torch.randn(7 + top + bottom, 9 + left + right, generator=g, dtype=torch.float64)
    ref = torch.nn.functional.pad(v[None, None], (left, right, top, bottom), mode="replicate")[0, 0]
    (ga,) = torch.autograd.grad((ref * w).sum(), v)
    out = _pad_replicate(v, top, bottom, left, right)
    assert torch.equal(out, ref)
    (gb,) = torch.autograd.grad((out * w).sum(), v)
    assert torch.allclose(gb, ga, rtol=0, atol=1e-13)
    assert torch.allclose(fold_replicate(w, *pads), ga, rtol=0, atol=1e-13)


def test_boundary_saving_plan_on_the_host(native_lib):
    """Boundary saving builds its frame tables on the host, reports snapshot_every = -1, sizes a
    gradient workspace between the snapshot and the full-history ones, and refuses batched plans."""
    from adfwi_gb300.acoustic import AcousticPlan, BOUNDARY_SAVING
    kw = dict(nz=30, nx=40, nabc=10, free_surface=False, src_z=[2, 2], src_x=[8, 30], rcv_z=[2] * 40,
              rcv_x=list(range(40)), nt=120, dt=1e-3, dtype=torch.float32)
    bs = AcousticPlan(snapshot_every=BOUNDARY_SAVING, **kw)
    assert bs.snapshot_every == BOUNDARY_SAVING
    full = AcousticPlan(snapshot_every=120, **kw)
    ck = AcousticPlan(snapshot_every=20, **kw)
    assert ck.workspace_bytes(True) < bs.workspace_bytes(True) < full.workspace_bytes(True)
    # forward only, the plans differ by the frame tables (an index per cell and the frame list)
    assert 0 <= bs.workspace_bytes(False) - full.workspace_bytes(False) <= 4 * 2 * 50 * 60 + 512
    with pytest.raises(RuntimeError, match="single-model"):
        AcousticPlan(snapshot_every=BOUNDARY_SAVING, shot_model=[0, 1], **kw)
