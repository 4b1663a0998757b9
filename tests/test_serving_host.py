"""Host-side logic of the solve server: misfit and pad adjoints against autograd, the arena
book, the admission policy and the seeded request stream (no GPU)."""
import numpy as np
import pytest
import torch

from adfwi_gb300 import serving as S


def _reference_l2(syn, obs, dt):
    """L2 trace misfit on max-normalised traces, written as the reference's FWI loop does
    (acoustic_fwi.py:149-150 normalisation, fwi/misfit/L2.py:26-29 misfit)."""
    syn = syn / torch.max(torch.abs(syn), dim=1, keepdim=True).values
    obs = obs / torch.max(torch.abs(obs), dim=1, keepdim=True).values
    rsd = obs - syn
    return torch.sum(torch.sqrt(torch.sum(rsd * rsd * dt, dim=1)))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_misfit_gradient_matches_autograd(dtype):
    g = torch.Generator().manual_seed(1)
    syn = torch.randn(4, 80, 9, generator=g, dtype=dtype)
    obs = torch.randn(4, 80, 9, generator=g, dtype=dtype)
    syn[1, :, 3] *= -5.0  # traces whose max |value| is a negative sample
    s = syn.clone().requires_grad_(True)
    L = _reference_l2(s, obs, 1.5e-3)
    L.backward()
    loss, gr = S.l2_misfit_grad(syn, S.normalise_traces(obs), 1.5e-3)
    tol = 1e-12 if dtype == torch.float64 else 2e-6
    ref = float(L.detach())
    assert abs(float(loss) - ref) <= tol * abs(ref)
    assert float((gr - s.grad).norm() / s.grad.norm()) <= tol


def test_misfit_skips_silent_traces():
    syn = torch.randn(2, 30, 5, dtype=torch.float64)
    obs = torch.randn(2, 30, 5, dtype=torch.float64)
    syn[0, :, 2] = 0.0
    obs[1, :, 4] = 0.0
    loss, gr = S.l2_misfit_grad(syn, S.normalise_traces(obs), 1e-3)
    assert torch.isfinite(loss) and torch.isfinite(gr).all()
    assert float(gr[0, :, 2].abs().max()) == 0.0


def test_precursor_traces_are_silent():
    syn = torch.randn(2, 40, 6, dtype=torch.float32)
    obs = torch.randn(2, 40, 6, dtype=torch.float32)
    syn[1, :, 0] *= 1e-37  # only the stencil's precursor reached this receiver
    loss, gr = S.l2_misfit_grad(syn, S.normalise_traces(obs, 1e-6), 1e-3, silent_rel=1e-6)
    assert torch.isfinite(gr).all() and float(gr[1, :, 0].abs().max()) == 0.0
    assert float(gr.abs().max()) < 1e3
    _, g0 = S.l2_misfit_grad(syn, S.normalise_traces(obs), 1e-3)  # the reference's rule
    assert float(g0[1, :, 0].abs().max()) > 1e30


def test_fold_is_the_adjoint_of_replicate_padding():
    v = torch.randn(7, 9, dtype=torch.float64, requires_grad=True)
    for n in (1, 3):
        pv = torch.nn.functional.pad(v[None, None], (n, n, n, n), mode="replicate")[0, 0]
        G = torch.randn_like(pv)
        (gv,) = torch.autograd.grad(pv, v, G)
        assert torch.allclose(S.fold_replicate_pad(G, n), gv, rtol=0, atol=1e-13)


def test_arena_book_first_fit_and_coalescing():
    b = S.ArenaBook(10 * 256 + 17)
    assert b.capacity == 2560
    r1 = b.alloc(300)       # 512
    r2 = b.alloc(256)
    r3 = b.alloc(1000)      # 1024
    assert [r[0] for r in (r1, r2, r3)] == [0, 512, 768]
    assert b.alloc(1024) is None and b.largest_free() == 768
    b.free(*r2)
    assert b.alloc(1024) is None     # a 256-byte hole and a 768-byte tail
    b.free(*r1)
    assert b.free_ranges[0] == (0, 768)  # coalesced with the neighbour
    r4 = b.alloc(700)
    assert r4[0] == 0
    b.free(*r3)
    b.free(*r4)
    assert b.free_ranges == [(0, 2560)] and b.used == 0 and b.peak == 1792
    with pytest.raises(RuntimeError):
        b.free(0, 256)


class _Item(object):
    def __init__(self, nbytes):
        self.nbytes = nbytes


def test_admission_backfills_then_turns_strict():
    book = S.ArenaBook(1000 * 256)
    big = book.alloc(600 * 256)  # a running request holds 600 of 1000 units
    q = [(0.0, _Item(500 * 256)), (0.1, _Item(100 * 256)), (0.2, _Item(200 * 256)), (0.3, _Item(300 * 256))]
    got = S.admit(q, book, free_slots=3, now=0.5, max_wait_s=2.0)
    # the oldest (500) does not fit; the two that do are admitted behind its back
    assert [e[0][0] for e in got] == [0.1, 0.2] and [e[0] for e in q] == [0.0, 0.3]
    # the oldest has now waited too long: nothing passes it even though 300 would fit
    got = S.admit(q, book, free_slots=3, now=3.0, max_wait_s=2.0)
    assert got == [] and len(q) == 2
    book.free(*big)
    got = S.admit(q, book, free_slots=1, now=3.1, max_wait_s=2.0)
    assert [e[0][0] for e in got] == [0.0] and [e[0] for e in q] == [0.3]


def test_admission_respects_slots():
    book = S.ArenaBook(1 << 20)
    q = [(float(k), _Item(1024)) for k in range(5)]
    got = S.admit(q, book, free_slots=2, now=0.0, max_wait_s=1.0)
    assert len(got) == 2 and len(q) == 3


def test_synthetic_stream_is_seeded_and_shaped():
    a = S.synthetic_stream(6, rate=50.0, seed=3)
    b = S.synthetic_stream(6, rate=50.0, seed=3)
    ts = [t for t, _, _ in a]
    assert ts == sorted(ts) and ts == [t for t, _, _ in b]
    for (_, tv, r), (_, tv2, r2) in zip(a, b):
        assert np.array_equal(tv, tv2) and np.array_equal(r.vp, r2.vp)
        assert r.meta["shape"] in S.GRIDS and 1 <= r.meta["shots"] <= 16 and r.nt in (1000, 2000, 4000)
        assert r.vp.shape == tv.shape == r.meta["shape"] and len(r.src_x) == r.meta["shots"]
        assert np.all(np.diff(tv.mean(axis=1)) >= -1e-3)  # velocity grows with depth on average


def test_form_batch_packs_the_oldest_requests_of_one_bucket():
    """The oldest waiting request is packed with the later requests of its bucket, in arrival
    order, within the shot and request caps; other buckets wait for their own batch."""
    E = S._Entry
    q = [E(0.0, "a", None, "B1", 4, 10), E(0.1, "b", None, "B2", 8, 10), E(0.2, "c", None, "B1", 8, 10),
         E(0.3, "d", None, "B1", 30, 10), E(0.4, "e", None, "B1", 2, 10), E(0.5, "f", None, "B1", 1, 10)]
    assert S.form_batch(q, 0, 32, 16) == [0, 2, 4, 5]      # d would pass 32 shots: skipped, later ones join
    assert S.form_batch(q, 0, 32, 2) == [0, 2]             # request cap
    assert S.form_batch(q, 1, 32, 16) == [1]               # alone in its bucket
    assert S.form_batch(q, 3, 32, 16) == [3, 4]            # 30 + 2 shots
