"""Solve server on the GPU: results equal the drop-in propagator's, each request's result
is bit-identical alone, in a batch and in a mix, admission keeps to the HBM budget, and a
failing or withdrawn request leaves the others' results unchanged."""
import numpy as np
import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300 import serving as S
from adfwi_gb300.synthetic import smooth

from _cases import layered_vp, rel

pytestmark = pytest.mark.gpu


def _request(seed, nz, nx, ns, nt, nabc=16, dx=10.0, dt=1e-3, f0=18.0, true=False):
    rng = np.random.default_rng(seed)
    vp_true = layered_vp(nz, nx, rng, vmin=1600.0, vmax=3200.0).astype(np.float32)
    vp = vp_true if true else smooth(vp_true, 3.0).astype(np.float32)
    sx = np.linspace(3, nx - 4, ns).round().astype(int)
    req = S.SolveRequest(vp=vp, dx=dx, nt=nt, dt=dt, f0=f0, src_z=np.full(ns, 2), src_x=sx,
                         rcv_z=np.full(nx, 2), rcv_x=np.arange(nx), nabc=nabc, rid=seed)
    return req, vp_true


def _with_obs(server, req, vp_true):
    fwd = S.SolveRequest(vp=vp_true, dx=req.dx, nt=req.nt, dt=req.dt, f0=req.f0, src_z=req.src_z,
                         src_x=req.src_x, rcv_z=req.rcv_z, rcv_x=req.rcv_x, nabc=req.nabc)
    req.obs = server.submit(fwd).result().records
    return req


def test_server_matches_the_drop_in_propagator(native_lib):
    req, vp_true = _request(11, 48, 72, 3, 400)
    with S.SolveServer(hbm_budget=2 << 30, slots=2, snapshot_precision="native", silent_rel=0.0) as srv:
        _with_obs(srv, req, vp_true)
        res = srv.submit(req).result()
    # the same solve through AcousticModel / AcousticPropagator and autograd
    nz, nx = req.vp.shape
    model = A.AcousticModel(0, 0, nx, nz, req.dx, req.dx, vp=req.vp.copy(),
                            rho=(np.power(req.vp, 0.25) * 310).astype(np.float32), vp_grad=True,
                            nabc=req.nabc, device="cuda:0")
    src = A.Source(nt=req.nt, dt=req.dt, f0=req.f0)
    _, wav = A.wavelet(req.nt, req.dt, req.f0)
    src.add_sources(src_x=req.src_x, src_z=req.src_z, src_wavelet=wav)
    rcv = A.Receiver(nt=req.nt, dt=req.dt)
    rcv.add_receivers(rcv_x=req.rcv_x, rcv_z=req.rcv_z, rcv_type="pr")
    prop = A.AcousticPropagator(model, A.Survey(src, rcv), device="cuda:0")
    syn = prop.forward()["p"]
    obs = torch.tensor(req.obs, device="cuda:0")
    syn_n = syn / torch.max(torch.abs(syn), dim=1, keepdim=True).values
    obs_n = obs / torch.max(torch.abs(obs), dim=1, keepdim=True).values
    loss = torch.sum(torch.sqrt(torch.sum((obs_n - syn_n) ** 2 * req.dt, dim=1)))
    loss.backward()
    assert abs(res.loss - loss.item()) <= 1e-5 * abs(loss.item())
    assert rel(res.grad, model.vp.grad) <= 1e-5


def test_forward_records_match_the_drop_in_propagator(native_lib):
    req, vp_true = _request(5, 40, 64, 2, 300, true=True)
    with S.SolveServer(hbm_budget=1 << 30, slots=1) as srv:
        rec = srv.submit(req).result().records
    nz, nx = req.vp.shape
    model = A.AcousticModel(0, 0, nx, nz, req.dx, req.dx, vp=req.vp.copy(),
                            rho=(np.power(req.vp, 0.25) * 310).astype(np.float32), nabc=req.nabc, device="cuda:0")
    src = A.Source(nt=req.nt, dt=req.dt, f0=req.f0)
    _, wav = A.wavelet(req.nt, req.dt, req.f0)
    src.add_sources(src_x=req.src_x, src_z=req.src_z, src_wavelet=wav)
    rcv = A.Receiver(nt=req.nt, dt=req.dt)
    rcv.add_receivers(rcv_x=req.rcv_x, rcv_z=req.rcv_z, rcv_type="pr")
    prop = A.AcousticPropagator(model, A.Survey(src, rcv), device="cuda:0")
    with torch.no_grad():
        ref = prop.forward()["p"].cpu().numpy()
    assert np.array_equal(rec, ref)


SHAPES = [(48, 80, 2, 300), (64, 128, 3, 500), (40, 64, 1, 400), (80, 96, 4, 300), (56, 100, 2, 600)]


def test_each_result_is_the_same_alone_and_in_the_mix(native_lib):
    budget = 256 << 20  # small per-solve budget: the longer solves keep FP24 snapshots
    reqs = [_request(100 + k, *shape) for k, shape in enumerate(SHAPES)]
    with S.SolveServer(hbm_budget=2 << 30, slots=1, per_request_budget=budget) as srv:
        for req, vp_true in reqs:
            _with_obs(srv, req, vp_true)
        alone = [srv.submit(req).result() for req, _ in reqs]
    with S.SolveServer(hbm_budget=2 << 30, slots=3, per_request_budget=budget) as srv:
        futs = [srv.submit(req) for req, _ in reqs]
        mix = [f.result() for f in futs]
        st = srv.stats()
    assert st["peak_concurrency"] >= 2  # the solves really overlapped
    assert any(r.snapshot_every < r_req.nt for r, (r_req, _) in zip(alone, reqs))
    for a, m in zip(alone, mix):
        assert a.rid == m.rid and a.snapshot_every == m.snapshot_every
        assert a.loss == m.loss
        assert np.array_equal(a.grad, m.grad)
        assert np.isfinite(a.grad).all() and np.abs(a.grad).max() > 0


def test_admission_keeps_to_the_budget(native_lib):
    req, vp_true = _request(7, 48, 80, 2, 300)
    with S.SolveServer(hbm_budget=1 << 30, slots=1) as srv:
        _with_obs(srv, req, vp_true)
    need = S.request_bytes(req, "fp24", 64 << 20, 1e-6)
    # room for one solve at a time: the second waits for the first to free its range
    with S.SolveServer(hbm_budget=int(need * 1.5), reserve=0, slots=2, per_request_budget=64 << 20) as srv:
        futs = [srv.submit(req) for _ in range(3)]
        res = [f.result() for f in futs]
        st = srv.stats()
    assert st["peak_concurrency"] == 1 and st["peak_arena_bytes"] <= st["arena_bytes"]
    assert all(np.array_equal(r.grad, res[0].grad) for r in res)
    # a request larger than the whole arena is refused; the server keeps serving
    with S.SolveServer(hbm_budget=need // 2, reserve=0, slots=1, per_request_budget=64 << 20) as srv:
        with pytest.raises(MemoryError):
            srv.submit(req).result()
        bad = S.SolveRequest(vp=req.vp, dx=req.dx, nt=10, dt=req.dt, f0=req.f0, src_z=np.array([2]),
                             src_x=np.array([10 ** 6]), rcv_z=req.rcv_z, rcv_x=req.rcv_x, nabc=req.nabc)
        with pytest.raises(RuntimeError):
            srv.submit(bad).result()


def test_graph_replays_equal_eager_solves_and_take_new_models(native_lib):
    """The second solve of a shape is captured in a CUDA graph and replayed; replays with other
    models of the same shape give exactly the eager results."""
    req_a, vp_true = _request(21, 48, 80, 2, 300)
    with S.SolveServer(hbm_budget=1 << 30, slots=1, graphs=False) as srv:
        _with_obs(srv, req_a, vp_true)
        req_b = S.SolveRequest(**{**req_a.__dict__, "vp": (req_a.vp * 1.03).astype(np.float32), "rid": 99})
        eager = [srv.submit(r).result() for r in (req_a, req_b, req_a)]
    with S.SolveServer(hbm_budget=1 << 30, slots=1, graphs=True) as srv:
        served = [srv.submit(r).result() for r in (req_a, req_b, req_a, req_b)]
        st = srv.stats()
    assert st["graph_replays"] == 3  # solves 2-4: captured at the second, replayed from then on
    for e, g in zip(eager + [eager[1]], served):
        assert e.loss == g.loss and np.array_equal(e.grad, g.grad)
    assert not np.array_equal(served[0].grad, served[1].grad)


def test_idle_shapes_are_evicted_for_room(native_lib):
    """Two shapes that do not fit together: each admission evicts the other's idle range."""
    ra, va = _request(31, 48, 80, 2, 300)
    rb, vb = _request(32, 56, 72, 3, 280)
    with S.SolveServer(hbm_budget=1 << 30, slots=1) as srv:
        _with_obs(srv, ra, va)
        _with_obs(srv, rb, vb)
    need = max(S.request_bytes(r, "fp24", 64 << 20, 1e-6) for r in (ra, rb))
    with S.SolveServer(hbm_budget=int(need * 1.5), reserve=0, slots=1, per_request_budget=64 << 20,
                       graphs=False) as srv:
        ref = [srv.submit(r).result() for r in (ra, rb)]
    with S.SolveServer(hbm_budget=int(need * 1.5), reserve=0, slots=1, per_request_budget=64 << 20) as srv:
        got = [srv.submit(r).result() for r in (ra, rb, ra, rb)]
        assert srv.stats()["peak_arena_bytes"] <= srv.book.capacity
    for e, g in zip(ref + ref, got):
        assert e.loss == g.loss and np.array_equal(e.grad, g.grad)


def _blocker():
    """A long forward solve (another bucket) that holds a server's only slot while other
    requests queue up behind it."""
    return _request(299, 48, 80, 1, 20000, true=True)[0]


def test_batched_requests_equal_their_solves_alone(native_lib):
    """Requests of one bucket (same grid, nt, receivers) with different models and shot counts
    are packed into shared launches; each result is bit-identical to the request solved alone."""
    reqs = [_request(200 + k, 48, 80, ns, 300) for k, ns in enumerate((2, 1, 3, 2))]
    with S.SolveServer(hbm_budget=2 << 30, slots=1, graphs=False) as srv:
        for req, vp_true in reqs:
            _with_obs(srv, req, vp_true)
    with S.SolveServer(hbm_budget=2 << 30, slots=1, graphs=False, max_batch_requests=1) as srv:
        alone = [srv.submit(req).result() for req, _ in reqs]
        assert srv.stats()["requests_per_batch"] == 1
    with S.SolveServer(hbm_budget=2 << 30, slots=1, graphs=False) as srv:
        blocker = srv.submit(_blocker())  # occupies the slot while the others queue up
        futs = [srv.submit(req) for req, _ in reqs]
        blocker.result()
        batched = [f.result() for f in futs]
        st = srv.stats()
    assert st["batches"] == 2 and st["requests_per_batch"] == 2.5  # the blocker, then one batch of four
    for a, b in zip(alone, batched):
        assert a.rid == b.rid and a.loss == b.loss and np.array_equal(a.grad, b.grad)


def test_failing_and_withdrawn_requests_leave_the_others_unchanged(native_lib):
    """A request whose plan rejects its geometry fails at submission, a request withdrawn by
    cancelling its future while it waits never runs, and the requests around them return what
    they return alone."""
    reqs = [_request(300 + k, 48, 80, 2, 300) for k in range(3)]
    with S.SolveServer(hbm_budget=2 << 30, slots=1, graphs=False) as srv:
        for req, vp_true in reqs:
            _with_obs(srv, req, vp_true)
        alone = [srv.submit(req).result() for req, _ in reqs]
    bad = S.SolveRequest(vp=reqs[0][0].vp, dx=10.0, nt=300, dt=1e-3, f0=18.0, src_z=np.array([2]),
                         src_x=np.array([10 ** 6]), rcv_z=np.full(80, 2), rcv_x=np.arange(80), nabc=16)
    with S.SolveServer(hbm_budget=2 << 30, slots=1, graphs=False) as srv:
        blocker = srv.submit(_blocker())
        first = srv.submit(reqs[0][0])
        failed = srv.submit(bad)
        withdrawn = srv.submit(reqs[1][0])
        assert withdrawn.cancel()  # still queued behind the blocker
        last = srv.submit(reqs[2][0])
        blocker.result()
        got = [first.result(), last.result()]
        st = srv.stats()
    with pytest.raises(RuntimeError):
        failed.result()
    assert withdrawn.cancelled() and st["cancelled"] == 1 and st["requests"] == 3
    for a, b in zip((alone[0], alone[2]), got):
        assert a.loss == b.loss and np.array_equal(a.grad, b.grad)


def test_iterating_clients_replay_graphs_and_match_eager_solves(native_lib):
    """Closed-loop FWI clients (gradient -> model update -> next gradient): each client's
    batches repeat, so with graphs they replay from the third iteration on, and every loss and
    model of every iteration is bit-identical to an eager server's."""
    clients = []
    for seed, (nz, nx, ns, nt) in ((31, (40, 64, 3, 300)), (32, (36, 56, 2, 260))):
        req, vp_true = _request(seed, nz, nx, ns, nt)
        clients.append((0.0, vp_true, req))
    hist = {}
    for graphs in (True, False):
        with S.SolveServer(hbm_budget=2 << 30, slots=2, snapshot_precision="native", graphs=graphs) as srv:
            if not hist:
                S.observed_data(srv, clients)
            srv.reset_stats()
            hist[graphs] = S.run_fwi_clients(srv, clients, 4, step=10.0)
            st = srv.stats()
        if graphs:
            assert st["graph_replays"] >= 2 * len(clients), st
        else:
            assert st["graph_replays"] == 0
    for ha, hb in zip(hist[True], hist[False]):
        assert len(ha) == 4
        for (la, va), (lb, vb) in zip(ha, hb):
            assert la == lb and np.array_equal(va, vb)
        assert ha[-1][0] < ha[0][0]  # the misfit decreases along the iterations
