"""Continuous-batching server for iso-acoustic forward and gradient solves of mixed sizes.

Requests (a model, its shots and, for a gradient solve, its observed data) arrive at any
time. When a solve slot is free, the server packs the oldest waiting request with the later
waiting requests of its bucket (same grid, time axis, wavelet, receivers and snapshot
interval) into one batched plan, whose persistent step kernels advance every shot of every
packed request in the same launches (each request on its own velocity model); it admits the
batch as soon as its device memory fits the HBM budget, runs every admitted batch on its own
CUDA stream so that batches overlap on the GPU, and reports per-request latency (arrival to
result) beside throughput.

Memory. The budget is one device arena allocated once. Each admitted batch takes one
contiguous, 256-byte aligned range of it (first fit) holding everything of its solve that
scales with the problem: the snapshot workspace, the three record arrays, the observed data
and its adjoint source, and the coefficient, damping, wavelet and gradient planes of each of
its models. The range stays resident until the batch completes. Admission is therefore exact (a request starts
only when its range can be carved), and no solve allocates or frees its large buffers through
a caching allocator (which synchronises the whole device when it runs out of cached blocks).
Short-lived temporaries of the misfit go through PyTorch's allocator and are covered by the
reserve left outside the arena.

Scheduling is first-come-first-served with backfill: a waiting request that fits may start
before an older one that does not fit yet, until the oldest has waited ``max_wait_s``; from
then on requests start strictly in arrival order so large requests cannot starve. A batch
that does not fit sheds its newest members first. A request larger than the whole arena, or
whose geometry its plan rejects, fails at submission; a cancelled future withdraws its request
while it waits; a failing batch fails only its own requests' futures.

Determinism. A request's snapshot interval depends only on its own shape (every request gets
the same ``per_request_budget``, and the interval is part of its bucket), a batched plan groups
each request's shots as a plan of that request alone would, the kernels are deterministic
(fixed-order reductions, no atomics), and each request's misfit runs over its own traces with
fixed-order reductions, so a request returns bit-identical records, loss and gradient whether
it runs alone, in a batch or next to other batches.
"""
import collections
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from .acoustic import AcousticPlan
from .boundary import bc_pml
from .utils import wavelet as _wavelet

_ALIGN = 256


def _aligned(n):
    return (int(n) + _ALIGN - 1) // _ALIGN * _ALIGN


@dataclass
class SolveRequest:
    """One iso-acoustic solve: records of ``vp`` (forward) or loss and dL/dvp (gradient).

    ``vp`` (nz, nx) in m/s on a square grid of spacing ``dx``; rho follows Gardner
    (310 vp^0.25, not differentiated) as ``AcousticModel.forward`` does; PML damping of
    ``nabc`` cells built from max(vp); sources ``(src_z, src_x)`` and receivers
    ``(rcv_z, rcv_x)`` are model cells; every shot fires the same Ricker wavelet of peak
    frequency ``f0``. ``obs`` (ns, nt, nr) makes it a gradient solve: the misfit is the L2
    trace misfit on max-normalised traces.
    """
    vp: np.ndarray
    dx: float
    nt: int
    dt: float
    f0: float
    src_z: np.ndarray
    src_x: np.ndarray
    rcv_z: np.ndarray
    rcv_x: np.ndarray
    obs: Optional[np.ndarray] = None
    nabc: int = 50
    free_surface: bool = False
    rid: int = -1
    meta: dict = field(default_factory=dict)


@dataclass
class SolveResult:
    rid: int
    loss: Optional[float]
    grad: Optional[np.ndarray]
    records: Optional[np.ndarray]
    t_arrival: float
    t_admit: float
    t_done: float
    cell_updates: int
    arena_bytes: int
    snapshot_every: int

    @property
    def latency(self):
        return self.t_done - self.t_arrival


# ------------------------------------------------------------------------------------------
# misfit and chain rule without autograd (no solve goes through the shared autograd thread);
# the server itself calls the fused CUDA misfit (adfwi_gb300.misfit), these PyTorch forms
# state the same arithmetic and check it
# ------------------------------------------------------------------------------------------
def _live_traces(m, silent_rel):
    """Traces (rows of the per-trace peaks ``m``, shape (ns, nr)) that carry signal: peak > 0
    and above ``silent_rel`` times the peak of their shot gather."""
    return (m > 0) & (m > silent_rel * m.amax(dim=1, keepdim=True))


def normalise_traces(d, silent_rel=0.0):
    """Divide every trace (dim 1 = time) by its max |value| (acoustic_fwi.py:149-150).
    Traces that are silent (zero everywhere, or with a peak at most ``silent_rel`` times
    their shot gather's peak) are set to zero; the reference divides them by their own tiny
    or zero peak."""
    m = torch.max(torch.abs(d), dim=1).values
    live = _live_traces(m, silent_rel)
    return d / torch.where(live, m, torch.ones_like(m))[:, None, :] * live[:, None, :]


def l2_misfit_grad(syn, obs_n, dt, silent_rel=0.0):
    """Loss and dLoss/dsyn of ``Misfit_waveform_L2`` (fwi/misfit/L2.py:26-29) applied to
    max-normalised synthetic traces: L = sum_{s,r} sqrt(sum_t (obs_n - syn/m)^2 dt) with
    m = max_t |syn|. The sums over time and traces are taken in FP64; the gradient follows
    the reference's autograd (the max routes its share to the arg-max sample).

    Silent synthetic traces (zero everywhere, or with a peak at most ``silent_rel`` times
    their shot gather's peak: only the stencil's numerical precursor ahead of the first
    arrival reaches them) are taken as zero: they add their observed trace's norm to the
    loss and nothing to the gradient. The reference normalises them by their own peak, which
    turns a precursor of ~1e-38 into an adjoint source of ~1e35 (overflow, NaN gradients).
    Returns (loss as a 0-d FP64 tensor, gradient in syn's dtype)."""
    mx, imx = syn.max(dim=1)
    mn, imn = syn.min(dim=1)
    use_min = (-mn) > mx
    m = torch.where(use_min, -mn, mx)                     # (ns, nr), >= 0
    idx = torch.where(use_min, imn, imx)
    sgn = torch.where(use_min, -torch.ones_like(m), torch.ones_like(m))
    live = _live_traces(m, silent_rel)
    syn_n = syn / torch.where(live, m, torch.ones_like(m))[:, None, :] * live[:, None, :]
    rsd = (obs_n - syn_n).double()                        # (ns, nt, nr)
    nrm = torch.sqrt(torch.sum(rsd * rsd, dim=1) * dt)    # (ns, nr)
    loss = nrm.sum()
    live = live & (nrm > 0)
    inv = torch.where(live, 1.0 / torch.where(live, nrm, torch.ones_like(nrm)), torch.zeros_like(nrm))
    g_n = rsd * (-dt) * inv[:, None, :]                   # dL / d(syn/m), zero on silent traces
    m64 = torch.where(live, m, torch.ones_like(m)).double()
    g = g_n / m64[:, None, :]
    corr = -(g_n * syn.double()).sum(dim=1) / (m64 * m64) * sgn.double()
    g.scatter_add_(1, idx[:, None, :], corr[:, None, :])
    return loss, g.to(syn.dtype)


def fold_replicate_pad(g, n):
    """Adjoint of edge-replicate padding by n cells (acoustic_kernels.py:16-37): the padded
    strips fold into the edge rows / columns and the corner blocks into the corner cells."""
    from .propagator import fold_replicate
    return fold_replicate(g, n, n, n, n)


def _pad(v, n):
    return torch.nn.functional.pad(v[None, None], (n, n, n, n), mode="replicate")[0, 0]


# ------------------------------------------------------------------------------------------
# device arena
# ------------------------------------------------------------------------------------------
class ArenaBook(object):
    """First-fit bookkeeping of 256-byte aligned ranges in ``capacity`` bytes (host only).
    Not thread-safe by itself: the server calls it under its lock."""

    def __init__(self, capacity):
        self.capacity = int(capacity) // _ALIGN * _ALIGN
        self.free_ranges = [(0, self.capacity)] if self.capacity else []  # sorted, coalesced
        self.used = 0
        self.peak = 0

    def alloc(self, nbytes):
        n = _aligned(nbytes)
        for k, (off, size) in enumerate(self.free_ranges):
            if size >= n:
                if size == n:
                    del self.free_ranges[k]
                else:
                    self.free_ranges[k] = (off + n, size - n)
                self.used += n
                self.peak = max(self.peak, self.used)
                return off, n
        return None

    def free(self, off, n):
        fr = self.free_ranges
        k = 0
        while k < len(fr) and fr[k][0] < off:
            k += 1
        if (k < len(fr) and off + n > fr[k][0]) or (k > 0 and fr[k - 1][0] + fr[k - 1][1] > off):
            raise RuntimeError("arena range (%d, %d) overlaps a free range: double free" % (off, n))
        fr.insert(k, (off, n))
        if k + 1 < len(fr) and fr[k][0] + fr[k][1] == fr[k + 1][0]:
            fr[k] = (fr[k][0], fr[k][1] + fr[k + 1][1])
            del fr[k + 1]
        if k > 0 and fr[k - 1][0] + fr[k - 1][1] == fr[k][0]:
            fr[k - 1] = (fr[k - 1][0], fr[k - 1][1] + fr[k][1])
            del fr[k]
        self.used -= n

    def largest_free(self):
        return max((s for _, s in self.free_ranges), default=0)


def admit(queue, book, free_slots, now, max_wait_s, size=lambda e: e[1].nbytes):
    """Admission step: carve ``book`` ranges for entries of ``queue`` (arrival-ordered
    tuples whose first item is the arrival time) into at most ``free_slots`` slots, first
    come first served with backfill; once the oldest entry has waited more than
    ``max_wait_s`` nothing may pass it. Removes the admitted entries from ``queue`` and
    returns [(entry, offset, bytes)]."""
    out = []
    strict = bool(queue) and now - queue[0][0] > max_wait_s
    i = 0
    while i < len(queue) and len(out) < free_slots:
        got = book.alloc(size(queue[i]))
        if got is not None:
            out.append((queue.pop(i),) + got)
            continue
        if strict:
            break
        i += 1
    return out


class _Carver(object):
    """Hands out typed views of consecutive 256-byte aligned pieces of an arena range."""

    def __init__(self, buf, off, end):
        self.buf, self.off, self.end = buf, off, end

    def take(self, shape, dtype):
        n = int(np.prod(shape)) * torch.empty((), dtype=dtype).element_size()
        if self.off + n > self.end:
            raise RuntimeError("solve footprint exceeds its arena range")
        v = self.buf[self.off:self.off + n].view(dtype).view(*shape)
        self.off += _aligned(n)
        return v


# ------------------------------------------------------------------------------------------
# batches: requests of one bucket packed into one batched plan, with its arena buffers and
# (after the second use of the same composition) a captured CUDA graph
# ------------------------------------------------------------------------------------------
def _i64(a):
    return np.asarray(a, dtype=np.int64).tobytes()


def _alone_plan(req, snapshot_precision, per_request_budget):
    """The plan of ``req`` solved alone (host only): checks its geometry."""
    vp = np.asarray(req.vp)
    if vp.ndim != 2:
        raise ValueError("vp must be a 2-D (nz, nx) array")
    nz, nx = vp.shape
    return AcousticPlan(nz=nz, nx=nx, nabc=req.nabc, free_surface=req.free_surface, src_z=req.src_z,
                        src_x=req.src_x, rcv_z=req.rcv_z, rcv_x=req.rcv_x, nt=req.nt, dt=req.dt,
                        dtype=torch.float32, snapshot_precision=snapshot_precision, memory_budget=per_request_budget)


def _shape_key(req, grad, snapshot_precision, silent_rel):
    """Requests that may share launches: same mode, grid, spacing, time axis, wavelet, absorbing
    frame and receivers (their sources and models may differ)."""
    return (bool(grad), tuple(np.shape(req.vp)), float(req.dx), int(req.nt), float(req.dt), float(req.f0),
            int(req.nabc), bool(req.free_surface), _i64(req.rcv_z), _i64(req.rcv_x), str(snapshot_precision),
            float(silent_rel))


def bucket_snapshot_every(req, snapshot_precision, batch_budget, max_batch_shots):
    """Snapshot interval of every solve of ``req``'s bucket: the one a batch of ``max_batch_shots``
    shots of this shape gets under ``batch_budget`` bytes. Fixing it per bucket keeps a request's
    result independent of the batch it is packed into (host only)."""
    vp = np.asarray(req.vp)
    nz, nx = vp.shape
    n = int(max_batch_shots)
    return AcousticPlan(nz=nz, nx=nx, nabc=req.nabc, free_surface=req.free_surface,
                        src_z=np.full(n, int(np.asarray(req.src_z)[0])), src_x=np.full(n, int(np.asarray(req.src_x)[0])),
                        rcv_z=req.rcv_z, rcv_x=req.rcv_x, nt=req.nt, dt=req.dt, dtype=torch.float32,
                        snapshot_precision=snapshot_precision, memory_budget=batch_budget).snapshot_every


def _batch_signature(bucket, reqs):
    return (bucket,) + tuple((len(r.src_x), _i64(r.src_z), _i64(r.src_x)) for r in reqs)


def request_bytes(req, snapshot_precision, per_request_budget, silent_rel=1e-6, max_batch_shots=32):
    """Device bytes of ``req`` solved alone by a server with these settings (host only)."""
    K = bucket_snapshot_every(req, snapshot_precision, per_request_budget, max_batch_shots)
    grad = req.obs is not None
    return _Batch([req], _shape_key(req, grad, snapshot_precision, silent_rel) + (K,), K, snapshot_precision,
                  silent_rel).nbytes


def _pad_models(v, n):
    """Edge-replicate padding by n cells of a stack of models (nm, nz, nx)."""
    return torch.nn.functional.pad(v[:, None], (n, n, n, n), mode="replicate")[:, 0]


class _Batch(object):
    """Requests of one bucket solved together: one batched plan (one model per request, the
    requests' shots in order), one arena range with every buffer of the solve, and the CUDA
    graph of the whole device-side solve once the same composition has been solved twice.

    Each request's shots are grouped as a plan of its model alone groups them and every request
    keeps its own snapshot interval (part of the bucket), so a request's records, loss and
    gradient are bit-identical whether it is solved alone or packed with others.

    The device-side solve (``_enqueue``) takes the models, their densities, their damping frames
    and the observed data from fixed buffers (the host computes density and damping exactly as
    AcousticModel / AcousticPropagator do) and does every other step on the GPU -- the padded
    coefficients, forward, the per-request misfits, adjoint and the chain rule to dL/dvp -- so
    one captured graph replays it for any models of the same composition."""

    def __init__(self, reqs, bucket, snapshot_every, snapshot_precision, silent_rel):
        r0 = reqs[0]
        self.nz, self.nx = np.shape(r0.vp)
        self.nm = len(reqs)
        self.ns_r = [len(r.src_x) for r in reqs]
        self.ranges = []
        s0 = 0
        for n in self.ns_r:
            self.ranges.append((s0, s0 + n))
            s0 += n
        self.ns, self.nr = s0, len(r0.rcv_x)
        self.grad = bucket[0]
        self.nt, self.dt, self.dx, self.f0, self.nabc = int(r0.nt), float(r0.dt), float(r0.dx), float(r0.f0), \
            int(r0.nabc)
        self.silent_rel = float(silent_rel)
        self.bucket = bucket
        self.key = _batch_signature(bucket, reqs)
        shot_model = np.concatenate([np.full(n, m) for m, n in enumerate(self.ns_r)])
        self.plan = AcousticPlan(nz=self.nz, nx=self.nx, nabc=self.nabc, free_surface=r0.free_surface,
                                 src_z=np.concatenate([np.asarray(r.src_z) for r in reqs]),
                                 src_x=np.concatenate([np.asarray(r.src_x) for r in reqs]), rcv_z=r0.rcv_z,
                                 rcv_x=r0.rcv_x, nt=self.nt, dt=self.dt, dtype=torch.float32,
                                 snapshot_precision=snapshot_precision, snapshot_every=snapshot_every,
                                 shot_model=shot_model)
        self.ws_bytes = self.plan.workspace_bytes(self.grad)
        self.nzp, self.nxp = self.plan.grid_shape()
        rec = self.ns * self.nt * self.nr * 4
        grid = self.nm * self.nzp * self.nxp * 4
        model = self.nm * self.nz * self.nx * 4
        self.nbytes = (_aligned(self.ws_bytes) + 3 * _aligned(rec) + (2 * _aligned(rec) if self.grad else 0)
                       + 3 * _aligned(grid) + 5 * _aligned(model) + _aligned(self.ns * self.nt * 4) + 2 * _ALIGN)
        self.cells = [n * self.nzp * self.nxp * self.nt for n in self.ns_r]
        self.off = self.n = None
        self.bound = False
        self.graph = None
        self.uses = 0

    # -- arena buffers and the batch's constant data (once per arena range)
    def _bind(self, arena, device):
        cv = _Carver(arena, self.off, self.off + self.n)
        shp = (self.ns, self.nt, self.nr)
        gshp = (self.nm, self.nzp, self.nxp)
        mshp = (self.nm, self.nz, self.nx)
        self.ws = cv.take((self.ws_bytes,), torch.uint8)
        self.recs = tuple(cv.take(shp, torch.float32) for _ in range(3))
        self.a1, self.a2, self.damp = (cv.take(gshp, torch.float32) for _ in range(3))
        self.fw = tuple(cv.take(mshp, torch.float32) for _ in range(3))
        self.vp_d = cv.take(mshp, torch.float32)
        self.rho_d = cv.take(mshp, torch.float32)
        self.wav = cv.take((self.ns, self.nt), torch.float32)
        self.dx_t = torch.full((), self.dx, dtype=torch.float32, device=device)  # divisor of alpha1
        self.one = cv.take((1,), torch.float64)  # scale of the misfit's adjoint source
        self.one.fill_(1.0)
        if self.grad:
            self.obs = cv.take(shp, torch.float32)
            self.adj = cv.take(shp, torch.float32)  # the misfit's adjoint source
        _, w = _wavelet(self.nt, self.dt, self.f0)
        self.wav.copy_(torch.from_numpy(np.ascontiguousarray(np.tile(w, (self.ns, 1)), dtype=np.float32)))
        self.bound = True

    def _load(self, reqs):
        """Copy the requests' models, their Gardner densities (310 vp^0.25, evaluated on the host
        in float32 as AcousticModel.forward does), damping frames and observed data into the fixed
        buffers."""
        for m, req in enumerate(reqs):
            vp = np.ascontiguousarray(req.vp, dtype=np.float32)
            self.vp_d[m].copy_(torch.from_numpy(vp))
            self.rho_d[m].copy_(torch.from_numpy(np.power(vp, 0.25) * 310))
            self.damp[m].copy_(torch.from_numpy(np.ascontiguousarray(
                bc_pml(self.nx, self.nz, self.dx, self.dx, self.nabc, vp.max(), free_surface=False),
                dtype=np.float32)))
            if self.grad:
                s0, s1 = self.ranges[m]
                self.obs[s0:s1].copy_(torch.from_numpy(np.ascontiguousarray(req.obs, dtype=np.float32)))

    def _enqueue(self, h):
        """The whole solve on the current stream (handle h): device work only, no host sync."""
        nb = self.nabc
        c, den = _pad_models(self.vp_d, nb), _pad_models(self.rho_d, nb)
        t1 = den * c
        # divisor as a device tensor: true division, as the drop-in propagator computes alpha1
        self.a1.copy_(t1 * c * self.dt / self.dx_t)
        self.a2.copy_(self.dt / (den * self.dx))
        self.plan.run_forward(self.a1, self.a2, self.damp, self.wav, self.grad, workspace=self.ws, records=self.recs,
                              fw=self.fw, stream=h)
        if not self.grad:
            return
        # each request's misfit over its own traces, its adjoint source in one pass, the adjoint
        self.out_loss = self.plan.l2_loss(self.recs[0], self.obs, self.ws, self.silent_rel, True, stream=h)
        self.plan.l2_sources(self.recs[0], self.obs, self.ws, self.one, True, adj=self.adj, stream=h)
        ga1, _ = self.plan.run_backward(self.a1, self.a2, self.damp, self.wav, (self.adj, None, None), self.ws,
                                        stream=h)
        # alpha1 = ((den c) c) dt / dx; alpha2 and rho do not depend on vp
        g_t2 = ga1 * (self.dt / self.dx)
        self.out_grad = [fold_replicate_pad(g_t2[m] * t1[m] + g_t2[m] * c[m] * den[m], nb) for m in range(self.nm)]

    def run(self, reqs, arena, stream, capture_stream, device, use_graphs):
        """Solve ``reqs`` in this batch's arena range and wait; returns [(loss, grad, records)]."""
        if not self.bound:
            self._bind(arena, device)
        with torch.cuda.stream(stream):
            self._load(reqs)
        if use_graphs and self.graph is None and self.uses >= 1:
            # second solve of this composition: capture the device-side solve once, replay it from now on
            capture_stream.wait_stream(stream)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.stream(capture_stream):
                g.capture_begin(capture_error_mode="thread_local")
                try:
                    self._enqueue(capture_stream.cuda_stream)
                finally:
                    g.capture_end()
            self.graph = g
            stream.wait_stream(capture_stream)
        with torch.cuda.stream(stream):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._enqueue(stream.cuda_stream)
            code = self.plan.status(self.ws, self.grad, stream=stream.cuda_stream)
            if code != 0:
                raise RuntimeError("solve of requests %s: a pipeline wait timed out on the GPU (status %d)"
                                   % ([r.rid for r in reqs], code))
            self.uses += 1
            if not self.grad:
                rec = self.recs[0].cpu().numpy()
                return [(None, None, rec[s0:s1]) for s0, s1 in self.ranges]
            losses = self.out_loss.cpu().numpy()
            grads = torch.stack(self.out_grad).cpu().numpy()
            return [(float(losses[m]), grads[m], None) for m in range(self.nm)]


# ------------------------------------------------------------------------------------------
# server
# ------------------------------------------------------------------------------------------
class _Entry(object):
    """A queued request: arrival time, the request, its future, its bucket and shot count."""
    __slots__ = ("t", "req", "fut", "bucket", "shots", "snapshot_every")

    def __init__(self, t, req, fut, bucket, shots, snapshot_every):
        self.t, self.req, self.fut, self.bucket, self.shots, self.snapshot_every = t, req, fut, bucket, shots, \
            snapshot_every


def _member_order(e):
    return (-e.shots, _i64(e.req.src_z), _i64(e.req.src_x))


def form_batch(queue, i, max_shots, max_requests):
    """Entries of ``queue`` (arrival order) that join ``queue[i]`` in one batch: later entries of
    the same bucket, in arrival order, while the batch keeps to ``max_shots`` shots and
    ``max_requests`` requests. Returns their indices, ``i`` first."""
    head = queue[i]
    idx, shots = [i], head.shots
    for j in range(i + 1, len(queue)):
        if len(idx) >= max_requests:
            break
        e = queue[j]
        if e.bucket == head.bucket and shots + e.shots <= max_shots:
            idx.append(j)
            shots += e.shots
    return idx


class SolveServer(object):
    """Admit, batch, overlap and complete solves under an HBM budget (module docstring).

    Continuous batching: when a slot is free, the oldest waiting request is packed with the later
    waiting requests of its bucket (same grid, time axis, wavelet, receivers and snapshot
    interval; ``max_batch_shots`` shots and ``max_batch_requests`` requests at most) into one
    batched plan, whose launches advance all their shots together; batches on different slots
    overlap on the GPU. A request's result does not depend on its batch.

    ``graphs``: keep each solved batch (plan, arena range, buffers) after it completes and
    capture its device-side solve in a CUDA graph at its second use; later batches of the same
    composition copy in their models and data and replay the graph. Idle batches keep their
    arena ranges until admission needs the room (least recently used first)."""

    def __init__(self, device="cuda:0", hbm_budget=150 << 30, slots=4, snapshot_precision="fp24",
                 per_request_budget=None, max_wait_s=2.0, reserve=None, silent_rel=1e-6, graphs=True,
                 max_batch_shots=32, max_batch_requests=16):
        if not torch.cuda.is_available():
            raise RuntimeError("SolveServer needs a CUDA device (adfwi_gb300 has no CPU implementation)")
        self.device = torch.device(device)
        self.budget = int(hbm_budget)
        reserve = int(reserve if reserve is not None else min(self.budget // 10, 16 << 30))
        self.book = ArenaBook(self.budget - reserve)
        self.arena = torch.empty(self.book.capacity, dtype=torch.uint8, device=self.device)
        self.slots = int(slots)
        self.snapshot_precision = snapshot_precision
        # device bytes that one batch of max_batch_shots shots may take (sets each bucket's
        # snapshot interval)
        self.per_request_budget = int(per_request_budget if per_request_budget is not None
                                      else max(1 << 30, self.book.capacity // max(1, self.slots)))
        self.max_wait_s = float(max_wait_s)
        self.silent_rel = float(silent_rel)
        self.graphs = bool(graphs)
        self.max_batch_shots = int(max_batch_shots)
        self.max_batch_requests = int(max_batch_requests)
        self._cv = threading.Condition()
        self._queue = []      # _Entry, arrival order
        self._ready = []      # (batch, [entries], t_admit)
        self._idle = collections.OrderedDict()  # id(batch) -> batch, least recently used first
        self._planned = collections.OrderedDict()  # signature -> planned batch without a range yet
        self._bucket_K = {}   # shape key -> snapshot interval of the bucket
        self._running = 0
        self._closed = False
        self._next_id = 0
        self.completed: List[SolveResult] = []
        self.failed = 0
        self.cancelled = 0
        self.peak_running = 0
        self.graph_replays = 0
        self.batches = 0
        self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.slots)]
        self._capture_streams = [torch.cuda.Stream(device=self.device) for _ in range(self.slots)]
        self._workers = [threading.Thread(target=self._worker, args=(k,), daemon=True, name="adfwi-solve-%d" % k)
                         for k in range(self.slots)]
        for w in self._workers:
            w.start()

    # -------------------------------------------------------------- client side
    def submit(self, req: SolveRequest, t_arrival=None) -> Future:
        """Queue a request; the future resolves to a SolveResult (or raises the solve's error).
        Cancelling the future before its solve starts withdraws the request."""
        fut = Future()
        t = time.perf_counter() if t_arrival is None else t_arrival
        grad = req.obs is not None
        try:
            alone = _alone_plan(req, self.snapshot_precision, self.per_request_budget)
            if grad and tuple(np.shape(req.obs)) != (alone.ns, req.nt, alone.nr):
                raise ValueError("obs has shape %s, expected %s" % (np.shape(req.obs), (alone.ns, req.nt, alone.nr)))
            skey = _shape_key(req, grad, self.snapshot_precision, self.silent_rel)
            with self._cv:
                K = self._bucket_K.get(skey)
            if K is None:
                K = bucket_snapshot_every(req, self.snapshot_precision, self.per_request_budget, self.max_batch_shots)
                with self._cv:
                    self._bucket_K[skey] = K
            bucket = skey + (K,)
            need = _Batch([req], bucket, K, self.snapshot_precision, self.silent_rel).nbytes
        except Exception as e:
            fut.set_exception(e)
            return fut
        if need > self.book.capacity:
            fut.set_exception(MemoryError("request %d needs %d bytes of device memory, more than the %d-byte arena"
                                          % (req.rid, need, self.book.capacity)))
            return fut
        with self._cv:
            if self._closed:
                raise RuntimeError("the server is closed")
            if req.rid < 0:
                req.rid = self._next_id
            self._next_id += 1
            self._queue.append(_Entry(t, req, fut, bucket, len(req.src_x), K))
            self._admit_locked()
            self._cv.notify_all()
        return fut

    def close(self, wait=True):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        if wait:
            for w in self._workers:
                w.join()
        with self._cv:
            for batch in list(self._idle.values()):
                self.book.free(batch.off, batch.n)
            self._idle.clear()
            if wait:
                # the workers have stopped and every batch is done: drop the cached batches
                # (their buffers and graphs) and the arena, so that the device memory is free for
                # whatever comes next even while this object is still referenced
                self._planned.clear()
                self.arena = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def reset_stats(self):
        with self._cv:
            self.completed = []
            self.failed = 0
            self.cancelled = 0
            self.graph_replays = 0
            self.batches = 0
            self.peak_running = self._running
            self.book.peak = self.book.used

    def stats(self):
        done = list(self.completed)
        if not done:
            return {}
        lat = np.array([r.latency for r in done])
        t0 = min(r.t_arrival for r in done)
        t1 = max(r.t_done for r in done)
        cells = sum(r.cell_updates for r in done)
        return {"requests": len(done), "failed": self.failed, "cancelled": self.cancelled,
                "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                "mean_s": float(lat.mean()), "makespan_s": t1 - t0, "gcell_per_s": cells / (t1 - t0) / 1e9,
                "peak_arena_bytes": self.book.peak, "arena_bytes": self.book.capacity,
                "peak_concurrency": self.peak_running, "graph_replays": self.graph_replays, "batches": self.batches,
                "requests_per_batch": len(done) / max(1, self.batches)}

    # -------------------------------------------------------------- scheduling
    def _take_idle(self, key):
        for bid, batch in self._idle.items():
            if batch.key == key:
                del self._idle[bid]
                return batch
        return None

    def _alloc_evicting(self, nbytes):
        got = self.book.alloc(nbytes)
        while got is None and self._idle:
            _, old = self._idle.popitem(last=False)  # least recently used idle batch
            self.book.free(old.off, old.n)
            got = self.book.alloc(nbytes)
        return got

    def _admit_locked(self):
        now = time.perf_counter()
        free = self.slots - self._running - len(self._ready)
        q = self._queue
        # withdrawn requests leave the queue
        keep = [e for e in q if not e.fut.cancelled()]
        self.cancelled += len(q) - len(keep)
        q[:] = keep
        strict = bool(q) and now - q[0].t > self.max_wait_s
        i = 0
        while i < len(q) and free > 0:
            idx = form_batch(q, i, self.max_batch_shots, self.max_batch_requests)
            admitted, dropped = None, False
            while idx and admitted is None:  # shed the newest members until the batch's range fits
                # members in a canonical order (most shots first, then geometry), so that the
                # same set of request shapes makes the same batch composition, whatever their
                # arrival order, and reuses its graph
                members = sorted((q[j] for j in idx), key=_member_order)
                reqs = [e.req for e in members]
                key = _batch_signature(members[0].bucket, reqs)
                batch = self._take_idle(key)
                if batch is None:
                    batch = self._planned.pop(key, None)
                    if batch is None:
                        try:
                            batch = _Batch(reqs, members[0].bucket, members[0].snapshot_every,
                                           self.snapshot_precision, self.silent_rel)
                        except Exception as e:  # a batch that cannot be planned: its head fails alone
                            if len(idx) == 1:
                                q[i].fut.set_exception(e)
                                del q[i]
                                self.failed += 1
                                dropped = True
                                break
                            idx = idx[:1]
                            continue
                    got = self._alloc_evicting(batch.nbytes)
                    if got is None:
                        self._remember_planned(key, batch)
                        idx = idx[:-1]
                        continue
                    batch.off, batch.n = got
                admitted = (batch, members)
            if dropped:
                continue
            if admitted is None:
                if strict:
                    break  # the oldest request has waited too long: nothing may pass it
                i += 1
                continue
            for j in sorted(idx, reverse=True):
                del q[j]
            self._ready.append((admitted[0], admitted[1], now))
            free -= 1

    def _remember_planned(self, key, batch):
        """Keep a planned batch that did not fit yet (host tables only), so that the next
        admission attempt does not plan it again."""
        self._planned[key] = batch
        while len(self._planned) > 64:
            self._planned.popitem(last=False)

    def _worker(self, k):
        stream, cstream = self._streams[k], self._capture_streams[k]
        while True:
            with self._cv:
                while True:
                    self._admit_locked()
                    if self._ready:
                        break
                    if self._closed and not self._queue:
                        return
                    self._cv.wait(timeout=0.05)
                batch, members, t_admit = self._ready.pop(0)
                self._running += 1
                self.peak_running = max(self.peak_running, self._running)
            out = err = None
            replayed = False
            try:
                out = batch.run([e.req for e in members], self.arena, stream, cstream, self.device, self.graphs)
                replayed = batch.graph is not None  # this solve ran as a graph replay (its composition's second use on)
            except Exception as e:  # the other batches keep running; the futures carry the error
                err = e
            t_done = time.perf_counter()
            try:
                stream.synchronize()  # the range may be reused only once this solve's work is done
            except Exception as e:
                err = err or e
            results = []
            if err is None:
                for m, (e, (loss, grad, rec)) in enumerate(zip(members, out)):
                    results.append(SolveResult(e.req.rid, loss, grad, rec, e.t, t_admit, t_done, batch.cells[m],
                                               batch.n, batch.plan.snapshot_every))
            with self._cv:
                self._running -= 1
                if self.graphs and err is None:
                    self._idle[id(batch)] = batch  # keep the batch (and its graph) for the next one like it
                else:
                    self.book.free(batch.off, batch.n)
                if err is None:
                    self.completed.extend(results)
                    self.graph_replays += int(replayed)
                    self.batches += 1
                else:
                    self.failed += len(members)
                self._admit_locked()
                self._cv.notify_all()
            for m, e in enumerate(members):
                if err is None:
                    e.fut.set_result(results[m])
                else:
                    e.fut.set_exception(err)


def replay(server, timed_requests):
    """Submit ``[(t_offset_s, SolveRequest), ...]`` at their arrival offsets from now and
    wait for all; returns the results in submission order."""
    t0 = time.perf_counter()
    futs = []
    for t, req in timed_requests:
        delay = t0 + t - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        futs.append(server.submit(req, t_arrival=t0 + t))
    return [f.result() for f in futs]


# ------------------------------------------------------------------------------------------
# synthetic request streams
# ------------------------------------------------------------------------------------------
GRIDS = ((100, 300), (200, 600), (300, 900), (500, 1500))


def random_layered_vp(rng, nz, nx, vmin=1500.0, vmax=4500.0):
    """Random layered model: 4-11 dipping interfaces and 0-2 normal faults, velocities
    uniform in [vmin, vmax] sorted to increase with depth."""
    from .synthetic import layered_faulted
    return layered_faulted(nz, nx, rng, n_interfaces=int(rng.integers(4, 12)), vmin=vmin, vmax=vmax,
                           n_faults=int(rng.integers(0, 3))).astype(np.float32)


def synthetic_stream(n, rate, seed=0, grids=GRIDS, shots=(1, 16), nts=(1000, 2000, 4000), dt=1e-3, f0=10.0,
                     nabc=50):
    """``n`` seeded requests with Poisson arrivals of ``rate`` per second: grid uniform over
    ``grids``, shot count uniform in ``shots`` (evenly spaced at z=2), nt uniform over
    ``nts``, a receiver at every column (z=2), PML of ``nabc`` cells. Returns
    [(t_offset, true_vp, request)]; the request's ``vp`` is the Gaussian-smoothed (sigma 10
    cells) true model and its ``obs`` is left for ``observed_data`` to fill."""
    from .synthetic import smooth
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        nz, nx = grids[int(rng.integers(len(grids)))]
        ns = int(rng.integers(shots[0], shots[1] + 1))
        nt = int(nts[int(rng.integers(len(nts)))])
        true_vp = random_layered_vp(rng, nz, nx)
        dx = 12.5 if nz >= 300 else 10.0
        sx = np.linspace(0, nx - 1, ns + 2)[1:-1].round().astype(int) if ns > 1 else np.array([nx // 2])
        req = SolveRequest(vp=smooth(true_vp, 10.0).astype(np.float32), dx=dx, nt=nt, dt=dt, f0=f0,
                           src_z=np.full(len(sx), 2), src_x=sx, rcv_z=np.full(nx, 2), rcv_x=np.arange(nx),
                           nabc=nabc, rid=k, meta={"shape": (nz, nx), "shots": ns, "nt": nt})
        out.append((t, true_vp, req))
    return out


def observed_data(server, stream):
    """Fill each request's ``obs`` with the records of its true model, served as forward
    solves by ``server`` (all submitted at once)."""
    futs = []
    for _, true_vp, req in stream:
        fwd = SolveRequest(vp=true_vp, dx=req.dx, nt=req.nt, dt=req.dt, f0=req.f0, src_z=req.src_z, src_x=req.src_x,
                           rcv_z=req.rcv_z, rcv_x=req.rcv_x, nabc=req.nabc, free_surface=req.free_surface)
        futs.append(server.submit(fwd))
    for (_, _, req), f in zip(stream, futs):
        req.obs = f.result().records
    return stream


# ------------------------------------------------------------------------------------------
# closed-loop FWI clients
# ------------------------------------------------------------------------------------------
FWI_CLIENTS = (((200, 600), 8, 2000), ((100, 300), 4, 1000), ((300, 900), 6, 2000), ((100, 300), 12, 2000))


def fwi_clients(seed=0, shapes=FWI_CLIENTS, dt=1e-3, f0=10.0, nabc=50):
    """One gradient request per client shape ((nz, nx), shots, nt): a smoothed random layered
    starting model, its true model, evenly spaced surface shots and a receiver at every column.
    Returns [(true_vp, request)]; ``observed_data`` fills the observed records."""
    from .synthetic import smooth
    rng = np.random.default_rng(seed)
    out = []
    for k, ((nz, nx), ns, nt) in enumerate(shapes):
        true_vp = random_layered_vp(rng, nz, nx)
        dx = 12.5 if nz >= 300 else 10.0
        sx = np.linspace(0, nx - 1, ns + 2)[1:-1].round().astype(int) if ns > 1 else np.array([nx // 2])
        req = SolveRequest(vp=smooth(true_vp, 10.0).astype(np.float32), dx=dx, nt=nt, dt=dt, f0=f0,
                           src_z=np.full(len(sx), 2), src_x=sx, rcv_z=np.full(nx, 2), rcv_x=np.arange(nx),
                           nabc=nabc, rid=k, meta={"shape": (nz, nx), "shots": ns, "nt": nt})
        out.append((0.0, true_vp, req))
    return out


def run_fwi_clients(server, clients, iterations, step=20.0):
    """Closed-loop FWI: every client submits a gradient solve, takes a normalised
    steepest-descent step of ``step`` m/s (vp -= step * grad / max|grad|, kept in
    [1000, 6000] m/s) and submits the next iteration, ``iterations`` times; the clients run
    concurrently, one thread each. A client's requests keep their shape, so its solves reuse
    the same batch and, from its third iteration on, replay that batch's CUDA graph. Returns
    each client's [(loss, vp)] per iteration."""
    import copy
    results = [None] * len(clients)
    errors = []

    def client(k):
        try:
            req = copy.copy(clients[k][2])
            hist = []
            for _ in range(iterations):
                res = server.submit(req).result()
                g = res.grad
                gm = float(np.abs(g).max())
                vp = req.vp - (step * g / gm if gm > 0 else 0.0)
                hist.append((res.loss, req.vp))
                req = copy.copy(req)
                req.vp = np.clip(vp, 1000.0, 6000.0).astype(np.float32)
            results[k] = hist
        except Exception as e:  # reported to the caller after every client has stopped
            errors.append(e)

    threads = [threading.Thread(target=client, args=(k,), name="fwi-client-%d" % k) for k in range(len(clients))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    return results
