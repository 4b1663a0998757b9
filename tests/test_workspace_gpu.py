"""A solve's results do not depend on what its workspace held before: a workspace filled
with NaN bit patterns gives bit-identical records and gradients to a zeroed one, in the
full-history and the snapshot modes of both propagators (GPU tests)."""
import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from _cases import ELASTIC_KEYS, acoustic_problem, elastic_problem

pytestmark = pytest.mark.gpu


def _ws(n, poison):
    return torch.full((n,), 0xFF, dtype=torch.uint8, device="cuda:0") if poison else \
        torch.zeros(n, dtype=torch.uint8, device="cuda:0")


@pytest.mark.parametrize("snapshot_every,precision", [(0, "native"), (37, "native"), (37, "bf16"), (37, "fp16")])
def test_acoustic_ignores_stale_workspace(snapshot_every, precision):
    model, survey, prop = acoustic_problem(A, ns=3, seed=41, snapshot_every=snapshot_every,
                                           snapshot_precision=precision)
    model.forward()
    a1, a2 = prop.coefficients(model)
    _, plan = prop.plan()
    assert (plan.snapshot_every < plan.nt) == (snapshot_every > 0)
    out = []
    for poison in (False, True):
        ws = _ws(plan.workspace_bytes(True), poison)
        rp, ru, rw, fp, fu, fw, _ = plan.run_forward(a1.detach(), a2.detach(), prop.damp, prop.wavelet, True,
                                                     workspace=ws)
        ga1, ga2 = plan.run_backward(a1.detach(), a2.detach(), prop.damp, prop.wavelet, (rp, ru, rw), ws)
        assert plan.status(ws, True) == 0
        out.append([t.cpu().numpy() for t in (rp, ru, rw, fp, fu, fw, ga1, ga2)])
    for a, b in zip(*out):
        assert np.isfinite(a).all() and np.array_equal(a, b)


@pytest.mark.parametrize("abc_type,snapshot_every", [("PML", 0), ("PML", 23), ("gerjan", 0), ("gerjan", 23)])
def test_elastic_ignores_stale_workspace(abc_type, snapshot_every):
    model, survey, prop = elastic_problem(A, abc_type=abc_type, seed=5, snapshot_every=snapshot_every)
    model.forward()
    _, plan = prop.plan()
    coefs, abc = prop.padded_coefficients(model)
    cs = [c.detach() for c in coefs] + [a for a in abc]
    out = []
    for poison in (False, True):
        ws = _ws(plan.workspace_bytes(True), poison)
        rec, fw, ws, ts = plan.run_forward(cs, prop.wavelet, True, workspace=ws)
        grads = plan.run_backward(cs, prop.wavelet, rec, ws)
        out.append([t.cpu().numpy() for t in [rec, fw] + list(grads)])
    for a, b in zip(*out):
        assert np.isfinite(a).all() and np.array_equal(a, b)
