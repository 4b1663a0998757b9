"""The CPU oracle reproduces the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference code): records bit-exact, gradients of the
fixture's linear functional within 1e-6 (float32) / 1e-12 (float64)."""
import numpy as np
import pytest
import torch

from _cases import golden_files, rel
from oracle.acoustic import acoustic_forward
from oracle.elastic import elastic_forward
from oracle.model import elastic_coefficients


@pytest.mark.parametrize("path", golden_files("acoustic"), ids=lambda p: p.split("/")[-1])
def test_oracle_acoustic_matches_reference(path):
    g = np.load(path)
    dt_ = torch.float64 if str(g["dtype"]) == "f64" else torch.float32
    vp = torch.tensor(g["vp"], dtype=dt_, requires_grad=True)
    rho = torch.tensor(g["rho"], dtype=dt_, requires_grad=True)
    out = acoustic_forward(vp, rho, torch.tensor(g["damp"]), g["src_x"], g["src_z"],
                           torch.tensor(g["wavelet"], dtype=dt_), g["rcv_x"], g["rcv_z"],
                           nabc=int(g["nabc"]), free_surface=bool(g["free_surface"]), dx=float(g["dx"]),
                           dz=float(g["dx"]), dt=float(g["dt"]), checkpoint_segments=int(g["segments"]))
    for k in out:
        assert np.array_equal(out[k].detach().numpy(), g["rec_" + k]), k
    loss = sum((out[k] * torch.tensor(g["w_" + k], dtype=dt_)).sum() for k in "puw")
    loss.backward()
    tol = 1e-12 if dt_ == torch.float64 else 1e-6
    assert rel(vp.grad, g["grad_vp"]) < tol
    assert rel(rho.grad, g["grad_rho"]) < tol


@pytest.mark.parametrize("path", golden_files("elastic"), ids=lambda p: p.split("/")[-1])
def test_oracle_elastic_matches_reference(path):
    g = np.load(path)
    dt_ = torch.float32
    iso = bool(g["iso"])
    pars = {}
    for k in ("vp", "vs", "rho", "eps", "delta", "gamma"):
        v = g[k] * (0 if iso and k in ("eps", "delta", "gamma") else 1)
        pars[k] = torch.tensor(v, dtype=dt_, requires_grad=True)
    co = elastic_coefficients(pars["vp"], pars["vs"], pars["rho"], pars["eps"], pars["delta"], pars["gamma"])
    out = elastic_forward(co, g["src_x"], g["src_z"], torch.tensor(g["wavelet"], dtype=dt_), g["moment_tensor"],
                          g["rcv_x"], g["rcv_z"], nabc=int(g["nabc"]), free_surface=bool(g["free_surface"]),
                          dx=float(g["dx"]), dz=float(g["dx"]), dt=float(g["dt"]), fd_order=int(g["fd_order"]),
                          abc_type=str(g["abc_type"]), bcx=g["bcx"] if "bcx" in g else None,
                          bcz=g["bcz"] if "bcz" in g else None, damp=g["damp"] if "damp" in g else None,
                          checkpoint_segments=int(g["segments"]))
    for k in out:
        assert np.array_equal(out[k].detach().numpy(), g["rec_" + k]), k
    comps = ("txx", "tzz", "txz", "vx", "vz")
    loss = sum((out[k] * torch.tensor(g["w_" + k], dtype=dt_)).sum() for k in comps)
    loss.backward()
    for p in ("vp", "vs", "rho", "eps", "delta"):
        if "grad_" + p in g:
            assert rel(pars[p].grad, g["grad_" + p]) < 1e-6, p


def test_oracle_refuses_gpu_tensors():
    from oracle.acoustic import _cpu_only
    t = torch.zeros(2)
    _cpu_only(t)
    if torch.cuda.is_available():
        with pytest.raises(RuntimeError):
            _cpu_only(t.cuda())


@pytest.mark.parametrize("path", golden_files("acoustic")[:2], ids=lambda p: p.split("/")[-1])
def test_oracle_checkpointed_chunks_match_reference(path):
    """Running every chunk under torch.utils.checkpoint (the reference's memory-bounded mode)
    gives the fixture's records bit for bit and its gradient to rounding."""
    g = np.load(path)
    dt_ = torch.float64 if str(g["dtype"]) == "f64" else torch.float32
    vp = torch.tensor(g["vp"], dtype=dt_, requires_grad=True)
    rho = torch.tensor(g["rho"], dtype=dt_, requires_grad=True)
    out = acoustic_forward(vp, rho, torch.tensor(g["damp"]), g["src_x"], g["src_z"],
                           torch.tensor(g["wavelet"], dtype=dt_), g["rcv_x"], g["rcv_z"],
                           nabc=int(g["nabc"]), free_surface=bool(g["free_surface"]), dx=float(g["dx"]),
                           dz=float(g["dx"]), dt=float(g["dt"]), checkpoint_segments=int(g["segments"]),
                           checkpoint_chunks=True)
    for k in out:
        assert np.array_equal(out[k].detach().numpy(), g["rec_" + k]), k
    loss = sum((out[k] * torch.tensor(g["w_" + k], dtype=dt_)).sum() for k in "puw")
    loss.backward()
    tol = 1e-12 if dt_ == torch.float64 else 1e-6
    assert rel(vp.grad, g["grad_vp"]) < tol


def c1_inputs():
    """Inputs of the full-size 100 x 100 forward configuration recorded in acoustic_c1_full.npz:
    vp, the Gardner density the reference's model computes from it (float32 numpy, as
    acoustic_model.py:111-118), damping, wavelets and geometry."""
    import os
    from _cases import GOLDEN
    from adfwi_gb300.utils import wavelet
    g = np.load(os.path.join(GOLDEN, "acoustic_c1_full.npz"))
    vp = g["vp_in"]
    rho = np.power(vp, 0.25) * 310
    _, w = wavelet(int(g["nt"]), float(g["dt"]), float(g["f0"]))
    wav = np.tile(w.astype(np.float32), (len(g["src_x"]), 1))
    return g, vp, rho.astype(np.float32), wav


def test_oracle_matches_reference_on_the_full_size_forward_configuration():
    """100 x 100, PML 50 (200 x 200 padded), 10 shots, 100 receivers, nt = 1000: every
    forward_wavefield_* map, every 10th pressure sample and the energy of every p, u, w trace
    equal the reference's bit for bit."""
    g, vp, rho, wav = c1_inputs()
    torch.set_num_threads(max(1, min(16, __import__("os").cpu_count() or 1)))
    with torch.no_grad():
        out = acoustic_forward(torch.tensor(vp), torch.tensor(rho), torch.tensor(g["damp"]), g["src_x"], g["src_z"],
                               torch.tensor(wav), g["rcv_x"], g["rcv_z"], nabc=int(g["nabc"]), free_surface=False,
                               dx=float(g["dx"]), dz=float(g["dx"]), dt=float(g["dt"]))
    for k in ("p", "u", "w"):
        e = np.sum(out[k].numpy().astype(np.float64) ** 2, axis=1)
        assert np.array_equal(e, g["energy_" + k]), k
        assert np.array_equal(out["forward_wavefield_" + k].numpy(), g["forward_wavefield_" + k]), k
    assert np.array_equal(out["p"].numpy()[:, ::int(g["decimate"]), :], g["rec_p_dec"])
