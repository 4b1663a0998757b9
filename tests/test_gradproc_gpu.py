"""GPU gradient processor (adfwi_gb300.gradient) against the reference's own outputs."""
import numpy as np
import pytest
import torch

from _cases import GOLDEN

from adfwi_gb300.gradient import GradProcessor, smooth2d

pytestmark = pytest.mark.gpu
CASES = ("land_mute_smooth", "marine_mute_smooth_mask", "plain_no_forw", "marine_no_forw_f32")


def _fixture():
    return np.load(GOLDEN + "/gradproc.npz")


@pytest.mark.parametrize("span", [3, 10, 40])
def test_smooth2d_kernel_matches_reference(span):
    g = _fixture()
    out = smooth2d(torch.tensor(g["smooth_in"], device="cuda"), span).cpu().numpy()
    ref = g["smooth_%d" % span]
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))


def _processor(g, name):
    kw = {k: g[name + "_" + k].item() for k in ("grad_mute", "grad_smooth", "norm_grad", "forw_illumination",
                                                 "marine_or_land")}
    kw["grad_mask"] = g[name + "_mask"] if name + "_mask" in g else None
    return GradProcessor(**kw)


@pytest.mark.parametrize("name", CASES)
def test_grad_processor_matches_reference(name):
    g = _fixture()
    grad = g[name + "_grad"]
    nz, nx = grad.shape
    forw = g[name + "_forw"] if name + "_forw" in g else None
    ref = g[name + "_out"]
    out = _processor(g, name).forward(nx=nx, nz=nz, vmax=3000.0, grad=grad.copy(), forw=forw)
    assert isinstance(out, np.ndarray) and out.dtype == ref.dtype
    tol = 1e-9 if ref.dtype == np.float64 else 2e-6
    assert np.max(np.abs(out - ref)) <= tol * np.max(np.abs(ref))
    # the same on device tensors, without host round trips
    dev = _processor(g, name).forward(nx=nx, nz=nz, vmax=3000.0, grad=torch.tensor(grad, device="cuda"),
                                      forw=None if forw is None else torch.tensor(forw, device="cuda"))
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), out)
