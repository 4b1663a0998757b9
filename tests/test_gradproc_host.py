"""The gradient-processor oracle against the reference's own outputs (CPU tests)."""
import numpy as np
import pytest

from _cases import GOLDEN

from oracle.gradproc import grad_process, smooth2d

CASES = ("land_mute_smooth", "marine_mute_smooth_mask", "plain_no_forw", "marine_no_forw_f32")


def _fixture():
    return np.load(GOLDEN + "/gradproc.npz")


@pytest.mark.parametrize("span", [3, 10, 40])
def test_smooth2d_oracle_matches_reference(span):
    g = _fixture()
    out = smooth2d(g["smooth_in"], span)
    ref = g["smooth_%d" % span]
    assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))


def _kwargs(g, name):
    kw = {k: g[name + "_" + k].item() for k in ("grad_mute", "grad_smooth", "norm_grad", "forw_illumination",
                                                 "marine_or_land")}
    kw["grad_mask"] = g[name + "_mask"] if name + "_mask" in g else None
    return kw


@pytest.mark.parametrize("name", CASES)
def test_grad_process_oracle_matches_reference(name):
    g = _fixture()
    grad = g[name + "_grad"]
    nz, nx = grad.shape
    forw = g[name + "_forw"] if name + "_forw" in g else None
    out = grad_process(nx, nz, 3000.0, grad, forw, **_kwargs(g, name))
    ref = g[name + "_out"]
    assert out.dtype == ref.dtype
    assert np.max(np.abs(out - ref)) <= 1e-9 * np.max(np.abs(ref))
