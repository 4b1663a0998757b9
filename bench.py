#!/usr/bin/env python
"""Benchmark of the GB300 propagator hot path: fwd+adjoint gradient throughput.

Workload (one "step"): one full-waveform-inversion gradient evaluation on the 200 x 600
layered/faulted iso-acoustic model (dx = 20 m, PML 50 -> 300 x 700 padded cells), 30 surface
shots, 600 receivers, nt = 3000, dt = 1.5 ms, 8 Hz Ricker, FP32: forward solve on the smoothed
starting model, per-trace normalisation and the L2 misfit against data observed on the true
model (the CUDA misfit passes on the plan's records and its adjoint source), then the
hand-written checkpointed adjoint back to dL/dvp. Inputs are seeded synthetic
stand-ins with those shapes and distributions (no public dataset).

Metric: Gcell-updates/s = shots * nzp * nxp * nt / time per gradient step.
  value: device time (CUDA events) with every input resident in HBM;
  e2e:   the same step through the public API with the model and the observed data copied
         from pinned host memory each step and the gradient + loss read back.

Arms: the default arm runs the CUDA library; ``--impl reference`` times the CPU oracle
(the reference's algorithm restated in PyTorch, CPU, all host threads) on a bounded sample
of the same workload.

Multi-GPU (torchrun, N > 1): every rank solves its own copy of the workload (shots are
independent; no collective on the data path), timing is the max over ranks, value = all
ranks' cell-updates / that time ("weak" scaling).
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+adjoint Gcell-updates/s"
UNIT = "Gcell-updates/s"
WORKLOAD = ("iso-acoustic forward + L2-misfit adjoint gradient: 200x600 layered model with 12 dipping "
            "interfaces and 2 normal faults, dx=20 m, PML 50 (300x700 padded), nt=3000, dt=1.5 ms, 8 Hz Ricker, "
            "30 surface shots, 600 receivers, FP32, checkpointed hand-written adjoint")
# Algorithmic bytes per cell-update of each kernel class (the figures the roofline uses):
#   forward step: read+write p, u, w (24 B) + the two per-cell coefficients (8 B);
#   adjoint step: adjoint state read+write (24 B) + coefficients (8 B) + reloaded forward
#                 state (12 B) + gradient accumulators read+write (8 B).
ALGO_BYTES = {"acoustic_fwd_step": 32.0, "acoustic_adj_step": 52.0}
# Gradient step total per cell-update (forward 32 + recompute 32 + segment store 12 + adjoint 52).
GRAD_BYTES = 128.0
# Elastic VTI gradient, algorithmic bytes per cell-update: forward 64 (5 fields r/w 40 + C11, C13,
# C33, C55, bx, bz 24) + recompute 64 + stored states 20 + adjoint 132 (state 40, coefficients 24,
# reloaded forward states 20, six gradient accumulators r/w 48); the same figure for every
# snapshot interval, split-field PML terms not counted.
EL_GRAD_BYTES = 280.0


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of each kernel from the committed ncu summaries (or {})."""
    out = {}
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return out
    for fn in sorted(os.listdir(pdir)):
        if not fn.endswith((".md", ".txt")):
            continue
        with open(os.path.join(pdir, fn)) as f:
            for line in f:
                m = re.match(r"\s*traffic_bytes_per_launch\s+(\S+)\s+([0-9.eE+]+)\s+cells_per_launch\s+([0-9.eE+]+)",
                             line)
                if m:
                    out[m.group(1)] = (float(m.group(2)), float(m.group(3)))
    return out


class ClockSampler(object):
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", "adfwi_clocks_%d_%d.csv" % (os.getpid(), index))

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gpu_arm(args, world, rank, local):
    import adfwi_gb300 as A
    from adfwi_gb300 import _native as N
    from adfwi_gb300.synthetic import acoustic_gradient_case

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    model, survey, vp_true, vp_init = acoustic_gradient_case(seed=0, device=str(dev), nt=args.nt)
    free, _ = torch.cuda.mem_get_info(dev)
    prop = A.AcousticPropagator(model, survey, device=str(dev), memory_budget=int(args.memory_fraction * free))
    nt, dt, ns = prop.nt, prop.dt, prop.src_n
    nzp, nxp = prop.nz + 2 * prop.nabc, prop.nx + 2 * prop.nabc
    cells = ns * nzp * nxp * nt
    # observed data on the true model (setup, untimed)
    with torch.no_grad():
        model.vp.data.copy_(torch.as_tensor(vp_true, device=dev))
        obs = prop.forward()["p"]
        obs = (obs / torch.max(torch.abs(obs), dim=1, keepdim=True).values).contiguous()
    vp0 = torch.as_tensor(vp_init, device=dev)

    def step(obs_dev):
        model.vp.data.copy_(vp0)
        model.vp.grad = None
        # forward solve + normalised L2 misfit (obs normalised once at setup, as acoustic_fwi.py
        # does), its adjoint source in one pass, then the adjoint
        loss, _ = prop.forward_l2(obs_dev)
        loss.backward()
        return loss

    _, plan = prop.plan()
    K = plan.snapshot_every
    for _ in range(args.warmup):
        step(obs)
    torch.cuda.synchronize(dev)

    # -- value: inputs resident in HBM, device time over exactly `steps` steps
    barrier(world)
    torch.cuda.synchronize(dev)
    n0 = N.launch_count()
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            loss = step(obs)
        e1.record()
        torch.cuda.synchronize(dev)
    barrier(world)
    launches = N.launch_count() - n0
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, world, dev)
    ms_step = ms / args.steps
    value = world * cells / (ms_step * 1e-3) / 1e9

    # -- e2e: public API with host buffers (pinned), copies inside the timed region
    vp_host = torch.as_tensor(vp_init).pin_memory()
    obs_host = obs.cpu().pin_memory()
    obs_dev = torch.empty_like(obs)
    grad_host = torch.empty(model.vp.shape, dtype=model.vp.dtype).pin_memory()
    h2d = vp_host.numel() * vp_host.element_size() + obs_host.numel() * obs_host.element_size()
    d2h = grad_host.numel() * grad_host.element_size() + 4
    barrier(world)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vp0.copy_(vp_host, non_blocking=True)
        obs_dev.copy_(obs_host, non_blocking=True)
        loss = step(obs_dev)
        grad_host.copy_(model.vp.grad, non_blocking=True)
        _ = float(loss.item())
    torch.cuda.synchronize(dev)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e_value = world * cells * args.steps / e2e_s / 1e9

    # -- roofline: per-kernel-class device time from CUDA events around every launch
    N.profile_start(True)
    for _ in range(max(1, min(args.steps, 2))):
        step(obs)
    torch.cuda.synchronize(dev)
    stats = N.profile_stop()
    peak, peak_kind = peaks()
    timed = {k: v for k, v in stats.items() if k in ALGO_BYTES and v[1] > 0}
    roof = None
    if timed:
        dom = max(timed, key=lambda k: timed[k][2])
        launches_dom, tl, tot_ms = timed[dom]
        avg_s = tot_ms / tl * 1e-3
        cells_launch = ns * nzp * nxp
        algo = ALGO_BYTES[dom] * cells_launch
        achieved = algo / avg_s / 1e9
        tr = ncu_traffic().get(dom)
        traffic = None
        if tr is not None:
            traffic = tr[0] * cells_launch / tr[1]  # scale a smaller capture by the cells processed
        roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": algo, "avg_launch_ms": round(avg_s * 1e3, 5),
                "kernel_share": {k: round(v[2] / sum(x[2] for x in stats.values()), 4) for k, v in stats.items()}}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered/faulted model, Ricker sources)",
        "config": {"workload": WORKLOAD, "shots": ns, "nt": nt, "grid_padded": [nzp, nxp], "receivers": prop.rcv_n,
                   "snapshot_every": K, "snapshot_precision": "native",
                   "l2": "working set larger than L2 (fields + segment history >> 129 MB), no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk.summary(),
        "loss": float(loss.item()),
    }
    return line


def _device_time(fn, dev, warmup, reps):
    """Mean device time (CUDA events on the current stream) of fn() over reps calls after warmup."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1) / reps


def _kernel_roofline(N, stats, cls, cells_launch):
    """Roofline of one kernel class from the library's per-launch event timing."""
    peak, kind = peaks()
    if cls not in stats or stats[cls][1] == 0:
        return None
    _, tl, tot = stats[cls]
    avg_s = tot / tl * 1e-3
    algo = ALGO_BYTES[cls] * cells_launch
    tr = ncu_traffic().get(cls)
    return {"bound": "hbm", "kernel": cls, "achieved": round(algo / avg_s / 1e9, 1), "peak": peak, "unit": "GB/s",
            "frac": round(algo / avg_s / 1e9 / peak, 4), "peak_source": kind,
            "traffic": None if tr is None else tr[0] * cells_launch / tr[1],
            "algorithmic_bytes_per_launch": algo, "avg_launch_ms": round(avg_s * 1e3, 5)}


def fp64_error(args, dev, memory_fraction):
    """Error of the headline FP32 gradient (and records, loss) against an FP64 run of the same
    scheme on the same inputs (untimed): the 200 x 600 workload in both precisions."""
    import adfwi_gb300 as A
    from adfwi_gb300.synthetic import acoustic_gradient_case
    res = {}
    for dtype in (torch.float64, torch.float32):
        model, survey, vp_true, vp_init = acoustic_gradient_case(seed=0, device=str(dev), nt=args.nt, dtype=dtype)
        free, _ = torch.cuda.mem_get_info(dev)
        prop = A.AcousticPropagator(model, survey, device=str(dev), dtype=dtype,
                                    memory_budget=int(memory_fraction * free))
        with torch.no_grad():
            model.vp.data.copy_(torch.as_tensor(vp_true, device=dev))
            obs = prop.forward()["p"]
            obs = (obs / torch.max(torch.abs(obs), dim=1, keepdim=True).values).contiguous()
        model.vp.data.copy_(torch.as_tensor(vp_init, device=dev))
        loss, rec = prop.forward_l2(obs)
        loss.backward()
        res[dtype] = (rec["p"].detach().double(), model.vp.grad.detach().double(), float(loss.detach()),
                      prop.plan()[1].snapshot_every)
        del model, prop, rec, obs
        torch.cuda.empty_cache()
    r64, g64, l64, k64 = res[torch.float64]
    r32, g32, l32, _ = res[torch.float32]
    rel = lambda a, b: float((a - b).norm() / b.norm())  # noqa: E731
    return {"grad_vp_rel_l2": rel(g32, g64), "records_p_rel_l2": rel(r32, r64), "loss_rel": abs(l32 - l64) / abs(l64),
            "fp64_snapshot_every": k64,
            "how": "same inputs, FP64 stencils and FP64 history/snapshots on the GPU; relative L2 over the whole array"}


def forward_legs(args, dev):
    """Forward-only solves (records, no gradient): the 100 x 100 configuration in full (PML 50,
    200 x 200 padded, 10 shots, 100 receivers, nt = 1000, dt = 1 ms, 10 Hz) and the 200 x 600
    workload's forward (30 shots, 300 x 700 padded, 600 receivers, nt = 3000)."""
    import adfwi_gb300 as A
    from adfwi_gb300 import _native as N
    from adfwi_gb300.synthetic import acoustic_gradient_case, linear_gradient_with_anomaly, surface_acquisition
    out = {}
    vp1 = linear_gradient_with_anomaly(100, 100).astype(np.float32)
    m1 = A.AcousticModel(0, 0, 100, 100, 10.0, 10.0, vp=vp1, rho=np.power(vp1, 0.25) * 310, nabc=50, device=str(dev))
    p1 = A.AcousticPropagator(m1, surface_acquisition(100, 1000, 1e-3, 10.0, 10), device=str(dev))
    m2, s2, _, _ = acoustic_gradient_case(seed=0, device=str(dev), nt=args.nt)
    p2 = A.AcousticPropagator(m2, s2, device=str(dev))
    for name, model, prop, reps in (("c1_100x100", m1, p1, 10), ("c2_200x600", m2, p2, 3)):
        nzp, nxp = prop.nz + 2 * prop.nabc, prop.nx + 2 * prop.nabc
        cells = prop.src_n * nzp * nxp * prop.nt

        def solve():
            with torch.no_grad():
                return prop.forward()

        ms = _device_time(solve, dev, 2, reps)
        # e2e: vp from pinned host memory in, the three record arrays back to pinned host memory
        vp_host = model.vp.detach().cpu().pin_memory()
        recs_host = [torch.empty((prop.src_n, prop.nt, prop.rcv_n)).pin_memory() for _ in range(3)]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(reps):
            model.vp.data.copy_(vp_host, non_blocking=True)
            r = solve()
            for h, k in zip(recs_host, "puw"):
                h.copy_(r[k], non_blocking=True)
            torch.cuda.synchronize(dev)
        e2e = cells * reps / (time.perf_counter() - t0) / 1e9
        N.profile_start(True)
        solve()
        torch.cuda.synchronize(dev)
        roof = _kernel_roofline(N, N.profile_stop(), "acoustic_fwd_step", prop.src_n * nzp * nxp)
        l2 = 4 * 3 * 2 * prop.src_n * nzp * nxp > 129e6
        out[name] = {"value": round(cells / (ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_solve": round(ms, 3),
                     "reps": reps, "shots": prop.src_n, "nt": prop.nt, "grid_padded": [nzp, nxp],
                     "receivers": prop.rcv_n,
                     "e2e": {"value": round(e2e, 3), "unit": UNIT,
                             "h2d_bytes_per_step": vp_host.numel() * 4,
                             "d2h_bytes_per_step": sum(h.numel() * 4 for h in recs_host)},
                     "roofline": roof if l2 else None,
                     "roofline_note": None if l2 else "fields fit in L2 (129 MB): no HBM roofline reported"}
    return out


def checkpointed_leg(args, dev):
    """Checkpointed gradient on the 500 x 1500 precision configuration (dx = 12.5 m, PML 50 ->
    600 x 1600 padded, nt = 6000, dt = 1 ms, 10 Hz Ricker, snapshots every 50 steps, 1500
    receivers): FP32 stencils with the snapshots in FP32, BF16 and FP16 (one max-abs scale per
    snapshot, shot and field) and FP24 (float32 rounded to a 15-bit mantissa, 3 bytes), timed; errors of records and dL/dvp (L = sum of records x fixed
    random traces) against an FP64 run of the same scheme with FP64 snapshots (untimed)."""
    import adfwi_gb300 as A
    from adfwi_gb300.synthetic import linear_gradient_with_anomaly, surface_acquisition
    nz, nx, dx, nt, dt, f0 = 500, 1500, 12.5, args.ckpt_nt, 1e-3, 10.0
    vp = linear_gradient_with_anomaly(nz, nx)
    sv = surface_acquisition(nx, nt, dt, f0, 64)
    idx = np.arange(0, 64, 64 // args.ckpt_shots)[:args.ckpt_shots]
    gen = torch.Generator(device=dev).manual_seed(0)
    wts = torch.randn((len(idx), nt, nx), generator=gen, device=dev, dtype=torch.float64)
    runs = [("fp64", torch.float64, "native"), ("fp32", torch.float32, "native"),
            ("fp32_bf16", torch.float32, "bf16"), ("fp32_fp16", torch.float32, "fp16"),
            ("fp32_fp24", torch.float32, "fp24")]
    got = {}
    for name, dtype, prec in runs:
        npdt = np.float64 if dtype == torch.float64 else np.float32
        model = A.AcousticModel(0, 0, nx, nz, dx, dx, vp=vp.astype(npdt), rho=(np.power(vp, 0.25) * 310).astype(npdt),
                                vp_grad=True, nabc=50, device=str(dev), dtype=dtype)
        prop = A.AcousticPropagator(model, sv, device=str(dev), dtype=dtype, snapshot_precision=prec,
                                    snapshot_every=50, ring_depth=args.ring_depth)
        w = wts.to(dtype)

        def grad():
            model.vp.grad = None
            rec = prop.forward(shot_index=idx)
            (rec["p"] * w).sum().backward()
            return rec

        ms = None
        if name != "fp64":
            grad()  # warm-up (plan, first launches)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
        rec = grad()
        if name != "fp64":
            e1.record()
        torch.cuda.synchronize(dev)
        if name != "fp64":
            ms = e0.elapsed_time(e1)
        got[name] = (rec["p"].detach().double(), model.vp.grad.detach().double(), ms)
        del model, prop, rec
        torch.cuda.empty_cache()
    peak, kind = peaks()
    cells = len(idx) * (nz + 100) * (nx + 100) * nt
    r64, g64, _ = got["fp64"]
    rel = lambda a, b: float((a - b).norm() / b.norm())  # noqa: E731
    res = {}
    for name, (r, g, ms) in got.items():
        if name == "fp64":
            continue
        v = cells / (ms * 1e-3) / 1e9
        res[name] = {"value": round(v, 3), "unit": UNIT, "ms_per_gradient": round(ms, 1),
                     "records_rel_l2_vs_fp64": rel(r, r64), "grad_vp_rel_l2_vs_fp64": rel(g, g64),
                     "roofline": {"bound": "hbm", "bytes_per_cell_update": GRAD_BYTES,
                                  "achieved": round(v * GRAD_BYTES, 1), "peak": peak, "unit": "GB/s",
                                  "frac": round(v * GRAD_BYTES / peak, 4), "peak_source": kind,
                                  "scope": "whole checkpointed gradient (forward, recompute, adjoint, snapshots)"}}
    return {"workload": "checkpointed gradient, 500x1500 model (600x1600 padded), nt=%d, snapshots every 50 steps, "
                        "%d of the 64 surface shots (every %dth), 1500 receivers" % (nt, len(idx), 64 // args.ckpt_shots),
            "shots": len(idx), "nt": nt, "snapshot_every": 50,
            "ring": {0: "automatic (deep: padded grid >= 1400 cells wide)", 1: "shallow", 2: "deep"}[args.ring_depth],
            "results": res}


def headline_checkpointed_leg(args, dev):
    """The headline gradient (200 x 600, 30 shots, nt = 3000, normalised L2 through forward_l2)
    in the memory-bounded forms -- snapshots every 50 steps with the segments recomputed in the
    adjoint (FP32 and FP24 snapshots), and boundary saving (the absorbing frame of every step
    kept, the interior rebuilt backwards) -- against the full-history gradient of the headline
    (which the 280 GB of HBM allows): time, workspace and gradient difference."""
    import adfwi_gb300 as A
    from adfwi_gb300.synthetic import acoustic_gradient_case
    model, survey, vp_true, vp_init = acoustic_gradient_case(seed=0, device=str(dev), nt=args.nt)
    cells = 30 * 300 * 700 * args.nt
    with torch.no_grad():
        model.vp.data.copy_(torch.as_tensor(vp_true, device=dev))
        obs = A.AcousticPropagator(model, survey, device=str(dev)).forward()["p"]
        obs = (obs / torch.max(torch.abs(obs), dim=1, keepdim=True).values).contiguous()
    vp0 = torch.as_tensor(vp_init, device=dev)
    out, grads = {}, {}
    runs = (("full_history", 0, "native"), ("fp32_every_50", 50, "native"), ("fp24_every_50", 50, "fp24"),
            ("boundary_saving", -1, "native"))
    for name, K, prec in runs:
        free, _ = torch.cuda.mem_get_info(dev)
        # built on the starting model: the damping frame takes max(vp) at construction, as the
        # reference's propagator does, so every run here gets the same frame
        model.vp.data.copy_(vp0)
        prop = A.AcousticPropagator(model, survey, device=str(dev), snapshot_every=K, snapshot_precision=prec,
                                    memory_budget=int(args.memory_fraction * free))

        def step():
            model.vp.data.copy_(vp0)
            model.vp.grad = None
            loss, _ = prop.forward_l2(obs)
            loss.backward()

        ms = _device_time(step, dev, 1, 2)
        grads[name] = model.vp.grad.detach().double().clone()
        plan = prop.plan()[1]
        out[name] = {"value": round(cells / (ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_gradient": round(ms, 1),
                     "snapshot_every": plan.snapshot_every,
                     "workspace_gb": round(plan.workspace_bytes(True) / 2 ** 30, 2)}
        del prop
        torch.cuda.empty_cache()
    g0 = grads["full_history"]
    for name in ("fp32_every_50", "fp24_every_50", "boundary_saving"):
        out[name]["grad_vp_rel_l2_vs_full_history"] = float((grads[name] - g0).norm() / g0.norm())
        out[name]["bit_identical_to_full_history"] = bool(torch.equal(grads[name], g0))
    return out


def plain_gpu_leg(args, dev):
    """The plain GPU path against the library on one gradient sample: the 200 x 600 workload
    (30 shots, 300 x 700 padded, 600 receivers) cut to 100 time steps, L = sum of the pressure
    records x fixed random traces. The plain path is the reference's algorithm as PyTorch tensor
    operations (the oracle's loop, bit-identical to the reference's records on the CPU) on CUDA
    tensors, each time chunk under torch.utils.checkpoint as the reference's propagator runs it,
    with autograd for the gradient."""
    import adfwi_gb300 as A
    from adfwi_gb300.synthetic import acoustic_gradient_case
    from oracle.acoustic import acoustic_forward
    nt = 100
    model, survey, _, _ = acoustic_gradient_case(seed=0, device=str(dev), nt=nt)
    prop = A.AcousticPropagator(model, survey, device=str(dev), memory_budget=60 << 30)
    cells = prop.src_n * (prop.nz + 2 * prop.nabc) * (prop.nx + 2 * prop.nabc) * nt
    wts = torch.randn((prop.src_n, nt, prop.rcv_n), generator=torch.Generator().manual_seed(0)).to(dev)

    def ours():
        model.vp.grad = None
        (prop.forward()["p"] * wts).sum().backward()

    def plain():
        model.forward()
        vp = model.vp.detach().clone().requires_grad_(True)
        out = acoustic_forward(vp, model.rho.detach(), prop.damp, prop.src_loc[:, 0], prop.src_loc[:, 1],
                               prop.wavelet, prop.rcv_loc[:, 0], prop.rcv_loc[:, 1], nabc=prop.nabc,
                               free_surface=False, dx=prop.dx, dz=prop.dz, dt=prop.dt, allow_gpu=True,
                               checkpoint_chunks=True)
        (out["p"] * wts).sum().backward()

    t_plain = _device_time(plain, dev, 1, 2)
    t_ours = _device_time(ours, dev, 2, 5)
    return {"sample": "30 shots x 300x700 padded x %d steps, forward + gradient" % nt,
            "plain_gpu_gcell_per_s": round(cells / (t_plain * 1e-3) / 1e9, 3),
            "library_gcell_per_s": round(cells / (t_ours * 1e-3) / 1e9, 3),
            "speedup_vs_plain_gpu": round(t_plain / t_ours, 2),
            "plain_path": "oracle loop (reference arithmetic in PyTorch ops) on CUDA, chunks under "
                          "torch.utils.checkpoint, autograd backward"}


def serving_arm(args, dev):
    """Served stream of mixed-size forward+gradient requests (Poisson arrivals, grids from
    {100x300, 200x600, 300x900, 500x1500}, 1-16 shots, nt in {1000, 2000, 4000}, random layered
    vp, FP32 stencils with FP24 snapshots, PML 50, 150 GB HBM admission budget): the
    continuous-batching server (same-bucket requests packed into shared launches, batches
    overlapped on several streams) at each arrival rate, against the same stream solved one
    request at a time (one slot, no packing) at the highest rate."""
    from adfwi_gb300 import serving as S
    rates = [float(r) for r in str(args.serve_rates).split(",") if r]
    budget = 150 << 30
    out = {"served": {}}
    results = {}
    per_req = None
    stream = S.synthetic_stream(args.serve_requests, max(rates), seed=0)
    modes = [("served@%g" % r, r, args.serve_slots, 32) for r in rates] + [("one_at_a_time", max(rates), 1, 1)]
    for name, rate, slots, mbr in modes:
        timed = [(t * max(rates) / rate, req) for t, _, req in stream]  # the same requests, arrivals rescaled
        with S.SolveServer(device=dev, hbm_budget=budget, slots=slots, snapshot_precision="fp24",
                           per_request_budget=per_req, max_batch_requests=mbr) as srv:
            per_req = srv.per_request_budget
            if not results:
                S.observed_data(srv, stream)  # observed data of the true models (setup, untimed)
            srv.reset_stats()
            results[name] = S.replay(srv, timed)
            st = srv.stats()
        rec = {"arrival_rate_per_s": rate, "p50_s": round(st["p50_s"], 4), "p99_s": round(st["p99_s"], 4),
               "mean_s": round(st["mean_s"], 4), "throughput_gcell_per_s": round(st["gcell_per_s"], 3),
               "requests_per_s": round(st["requests"] / st["makespan_s"], 3), "slots": slots,
               "batches": st["batches"], "requests_per_batch": round(st["requests_per_batch"], 2),
               "peak_concurrency": st["peak_concurrency"], "peak_arena_gb": round(st["peak_arena_bytes"] / 2 ** 30, 2),
               "graph_replays": st["graph_replays"]}
        if name == "one_at_a_time":
            out[name] = rec
        else:
            out["served"][name] = rec
    ref = results["one_at_a_time"]
    same = all(a.loss == b.loss and np.array_equal(a.grad, b.grad)
               for name in results for a, b in zip(results[name], ref))
    top = out["served"]["served@%g" % max(rates)]
    if args.fwi_iterations > 0:
        out["fwi_clients"] = fwi_clients_leg(args, dev, budget)
    out.update({"requests": args.serve_requests, "hbm_budget_gb": budget / 2 ** 30,
                "arena_gb": round(srv.book.capacity / 2 ** 30, 2), "per_request_budget_gb": round(per_req / 2 ** 30, 2),
                "snapshot_precision": "fp24", "bit_identical_alone_vs_mix": bool(same),
                "graph_replays": sum(v["graph_replays"] for v in out["served"].values()),
                "speedup_vs_one_at_a_time": round(top["throughput_gcell_per_s"]
                                                  / out["one_at_a_time"]["throughput_gcell_per_s"], 3),
                "sample": "first %d requests of the seeded 2000-request stream" % args.serve_requests})
    return out


def fwi_clients_leg(args, dev, budget):
    """Closed-loop FWI clients on the server (``serving.run_fwi_clients``): four clients with
    fixed shapes (200x600 8 shots nt 2000, 100x300 4 shots nt 1000, 300x900 6 shots nt 2000,
    100x300 12 shots nt 2000), each iterating gradient -> model update -> next gradient, served
    with and without CUDA graphs. Every client's requests keep one shape, so its batches repeat
    and, with graphs, replay from the third iteration on; the two runs give the same bits."""
    from adfwi_gb300 import serving as S
    clients = S.fwi_clients(seed=1)
    with S.SolveServer(device=dev, hbm_budget=budget, slots=args.serve_slots, snapshot_precision="fp24") as srv:
        S.observed_data(srv, clients)
    out, hists = {}, {}
    for graphs in (True, False):
        with S.SolveServer(device=dev, hbm_budget=budget, slots=args.serve_slots, snapshot_precision="fp24",
                           graphs=graphs) as srv:
            srv.reset_stats()
            t0 = time.perf_counter()
            hists[graphs] = S.run_fwi_clients(srv, clients, args.fwi_iterations)
            wall = time.perf_counter() - t0
            st = srv.stats()
        out["graphs" if graphs else "eager"] = {
            "throughput_gcell_per_s": round(st["gcell_per_s"], 3), "wall_s": round(wall, 3),
            "p50_s": round(st["p50_s"], 4), "p99_s": round(st["p99_s"], 4), "requests": st["requests"],
            "graph_replays": st["graph_replays"], "batches": st["batches"]}
    same = all(a[0] == b[0] and np.array_equal(a[1], b[1])
               for ha, hb in zip(hists[True], hists[False]) for a, b in zip(ha, hb))
    out.update({"clients": len(clients), "iterations": args.fwi_iterations, "bit_identical_graphs_vs_eager": bool(same),
                "loss_first_last": [[round(h[0][0], 6), round(h[-1][0], 6)] for h in hists[True]],
                "speedup_graphs_vs_eager": round(out["eager"]["wall_s"] / out["graphs"]["wall_s"], 3)})
    return out


def elastic_arm(args, dev):
    """VTI-elastic velocity-stress gradient (200 x 400, dx = 10 m, PML 40 + free surface -> 242 x 480
    padded cells, 4th order, nt = 2000, dt = 0.8 ms, 15 Hz Ricker explosive sources, 20 shots,
    400 receivers; vx / vz records weighted by fixed random traces; gradients for vp, vs, rho,
    eps and delta through the hand-written adjoint)."""
    import adfwi_gb300 as A
    from adfwi_gb300.synthetic import vti_gradient_case
    model, survey = vti_gradient_case(seed=0, device=str(dev), nt=args.elastic_nt)
    prop = A.ElasticPropagator(model, survey, device=str(dev))
    nt, ns = prop.nt, prop.src_n
    gen = torch.Generator().manual_seed(0)
    w = {k: torch.randn((ns, nt, prop.rcv_n), generator=gen).to(dev) for k in ("vx", "vz")}

    def step():
        for par in ("vp", "vs", "rho", "eps", "delta"):
            getattr(model, par).grad = None
        rec = prop.forward(fd_order=4)
        loss = (rec["vx"] * w["vx"]).sum() + (rec["vz"] * w["vz"]).sum()
        loss.backward()
        return rec

    rec = step()
    nzp, nxp = prop.padded_coefficients(model, 4)[0][0].shape
    cells = ns * nzp * nxp * nt
    reps = max(3, min(args.steps, 5))
    ms = _device_time(step, dev, 1, reps)
    _, plan = prop.plan(None, 4)
    value = cells / (ms * 1e-3) / 1e9
    # e2e: the five model parameters from pinned host memory in, their gradients back out
    pars = ("vp", "vs", "rho", "eps", "delta")
    host_in = {k: getattr(model, k).detach().cpu().pin_memory() for k in pars}
    host_out = {k: torch.empty_like(host_in[k]).pin_memory() for k in pars}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(reps):
        for k in pars:
            getattr(model, k).data.copy_(host_in[k], non_blocking=True)
        step()
        for k in pars:
            host_out[k].copy_(getattr(model, k).grad, non_blocking=True)
        torch.cuda.synchronize(dev)
    e2e = cells * reps / (time.perf_counter() - t0) / 1e9
    peak, peak_kind = peaks()
    achieved = value * EL_GRAD_BYTES
    out = {"workload": "VTI elastic gradient (vp, vs, rho, eps, delta): 200x400, PML 40 + free surface "
                       "(242x480 padded), 4th order, nt=%d, dt=0.8 ms, 20 shots, 400 receivers, FP32" % nt,
           "value": round(value, 3), "unit": UNIT, "ms_per_gradient": round(ms, 2),
           "steps": reps, "snapshot_every": plan.snapshot_every, "grid_padded": [int(nzp), int(nxp)],
           "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": sum(v.numel() * 4 for v in host_in.values()),
                   "d2h_bytes_per_step": sum(v.numel() * 4 for v in host_out.values())},
           "roofline": {"bound": "hbm", "bytes_per_cell_update": EL_GRAD_BYTES, "achieved": round(achieved, 1),
                        "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                        "scope": "whole gradient (all elastic kernels), algorithmic bytes per cell-update"}}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = elastic_cpu_sample(args.elastic_cpu_steps)
    return out


def elastic_cpu_sample(n_steps, min_seconds=5.0):
    """CPU oracle (the reference's elastic loop restated in PyTorch, all host threads) on a bounded
    sample of the VTI workload: 1 shot x n_steps steps of the 242 x 480 padded grid, forward +
    autograd backward to vp, vs, rho, eps, delta, repeated until min_seconds of work."""
    from adfwi_gb300.boundary import bc_pml_xz
    from adfwi_gb300.synthetic import surface_acquisition, vti_layered
    from oracle.elastic import elastic_forward
    from oracle.model import elastic_coefficients
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    rng = np.random.default_rng(0)
    arrs = vti_layered(200, 400, rng)
    sv = surface_acquisition(400, n_steps, 8e-4, 15.0, 20, src_z=2, rcv_z=1)
    bcx, bcz = bc_pml_xz(400, 200, 10.0, 10.0, 40, arrs[0].max(), free_surface=True)
    loc = sv.source.get_loc()[[10]]
    rl = sv.receiver.get_loc()
    done, t_all, reps = 0, 0.0, 0
    while t_all < min_seconds and reps < 20:
        pars = [torch.tensor(a.astype(np.float32), requires_grad=True) for a in arrs]
        t0 = time.perf_counter()
        co = elastic_coefficients(*pars, "vti")
        out = elastic_forward(co, loc[:, 0], loc[:, 1], torch.tensor(sv.source.get_wavelet()[:1], dtype=torch.float32),
                              torch.tensor(sv.source.get_moment_tensor()[:1], dtype=torch.float32), rl[:, 0], rl[:, 1],
                              nabc=40, free_surface=True, dx=10.0, dz=10.0, dt=8e-4, fd_order=4, abc_type="PML",
                              bcx=bcx, bcz=bcz, damp=None)
        (out["vx"].square().sum() + out["vz"].square().sum()).backward()
        t_all += time.perf_counter() - t0
        done += 242 * 480 * n_steps
        reps += 1
    return {"value": round(done / t_all / 1e9, 5), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d x (1 shot x %d steps) of the 242x480 padded VTI gradient, CPU oracle forward + autograd "
                      "backward, %.1f s" % (reps, n_steps, t_all)}


def precision_study(args):
    """Snapshot precision against the FP64 instance of the same scheme on the 500 x 1500 model
    (linear 1500 -> 3000 m/s with a +300 m/s Gaussian anomaly, dx = 12.5 m, PML 50, nt = 6000,
    dt = 1 ms, 10 Hz Ricker): FP32 stencils with checkpoints every 50 steps kept in FP32, BF16 and
    FP16 (per-snapshot max-abs scale), against FP64 stencils and FP64 checkpoints. Shots: every
    8th of the 64 evenly spaced surface shots. Errors: relative L2 of the pressure records and of
    dL/dvp for L = sum(records x fixed random traces)."""
    import adfwi_gb300 as A
    from adfwi_gb300.synthetic import linear_gradient_with_anomaly, surface_acquisition
    dev = torch.device("cuda", 0)
    nz, nx, dx, nt, dt, f0 = 500, 1500, 12.5, args.precision_nt, 1e-3, 10.0
    vp = linear_gradient_with_anomaly(nz, nx)
    sv64 = surface_acquisition(nx, nt, dt, f0, 64)
    idx = np.arange(0, 64, 8)
    gen = torch.Generator().manual_seed(0)
    wts = torch.randn((len(idx), nt, nx), generator=gen, dtype=torch.float64)
    out = {}
    runs = [("fp64", torch.float64, "native"), ("fp32", torch.float32, "native"), ("fp32_bf16", torch.float32, "bf16"),
            ("fp32_fp16", torch.float32, "fp16")]
    for name, dtype, prec in runs:
        npdt = np.float64 if dtype == torch.float64 else np.float32
        model = A.AcousticModel(0, 0, nx, nz, dx, dx, vp=vp.astype(npdt), rho=(np.power(vp, 0.25) * 310).astype(npdt),
                                vp_grad=True, nabc=50, device=str(dev), dtype=dtype)
        prop = A.AcousticPropagator(model, sv64, device=str(dev), dtype=dtype, snapshot_precision=prec,
                                    snapshot_every=50)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        rec = prop.forward(shot_index=idx)
        (rec["p"] * wts.to(dev, dtype)).sum().backward()
        torch.cuda.synchronize(dev)
        out[name] = {"rec": rec["p"].detach().double().cpu(), "grad": model.vp.grad.detach().double().cpu(),
                     "s": time.perf_counter() - t0}
        del model, prop, rec
        torch.cuda.empty_cache()
    ref = out["fp64"]
    rel = lambda a, b: float((a - b).norm() / b.norm())  # noqa: E731
    res = {name: {"records_rel_l2": rel(v["rec"], ref["rec"]), "grad_vp_rel_l2": rel(v["grad"], ref["grad"]),
                  "seconds": round(v["s"], 2)} for name, v in out.items() if name != "fp64"}
    return {"study": "snapshot precision vs FP64 GPU run", "grid": [nz, nx], "dx": dx, "nt": nt, "shots": len(idx),
            "snapshot_every": 50, "fp64_seconds": round(ref["s"], 2), "results": res}


def cpu_sample(n_steps, threads):
    """Time the CPU oracle on a bounded sample: 1 shot of the gradient workload, n_steps steps,
    forward + autograd backward (the reference's own gradient mechanism)."""
    from adfwi_gb300.synthetic import layered_faulted, smooth, surface_acquisition
    from oracle.acoustic import acoustic_forward
    from adfwi_gb300.boundary import bc_pml
    torch.set_num_threads(threads)
    rng = np.random.default_rng(0)
    vp_true = layered_faulted(200, 600, rng)
    vp = smooth(vp_true, 10.0).astype(np.float32)
    rho = (np.power(vp, 0.25) * 310).astype(np.float32)
    sv = surface_acquisition(600, n_steps, 1.5e-3, 8.0, 30)
    damp = torch.tensor(bc_pml(600, 200, 20.0, 20.0, 50, vp.max(), free_surface=False), dtype=torch.float32)
    wav = torch.tensor(sv.source.get_wavelet()[:1], dtype=torch.float32)
    loc = sv.source.get_loc()[:1]
    rl = sv.receiver.get_loc()
    vpt = torch.tensor(vp, requires_grad=True)
    t0 = time.perf_counter()
    out = acoustic_forward(vpt, torch.tensor(rho), damp, loc[:, 0], loc[:, 1], wav, rl[:, 0], rl[:, 1], nabc=50,
                           free_surface=False, dx=20.0, dz=20.0, dt=1.5e-3)
    out["p"].square().sum().backward()
    t = time.perf_counter() - t0
    cells = 1 * 300 * 700 * n_steps
    return cells / t / 1e9, t


def reference_arm(args):
    threads = os.cpu_count() or 1
    n_steps = args.cpu_sample_steps
    cpu_sample(min(20, n_steps), threads)  # warm the allocator / thread pool
    for _ in range(args.warmup):
        cpu_sample(n_steps, threads)
    vals = []
    t_all = 0.0
    for _ in range(args.steps):
        v, t = cpu_sample(n_steps, threads)
        vals.append(v)
        t_all += t
    value = args.steps * 300 * 700 * n_steps / t_all / 1e9
    sample = "1 shot x %d steps of the 300x700 padded gradient workload (forward + autograd backward)" % n_steps
    return {"impl": "reference", "metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_all / args.steps * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded layered/faulted model, Ricker sources)",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample, "port_vs_reference_cpu": port_vs_reference()},
            "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def port_vs_reference():
    """The committed timing of the reference's own CPU propagator against this port on the same
    slice and threads (tests/golden/cpu_timing_ref_vs_port.json; the reference itself cannot run
    where the benchmark does), or None."""
    path = os.path.join(ROOT, "tests", "golden", "cpu_timing_ref_vs_port.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return {"port_over_reference_speed": d["port_over_reference_speed"], "threads": d["threads"],
                "machine": d["machine"], "sample": d["sample"]}
    except Exception:
        return None


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--memory-fraction", type=float, default=0.7,
                    help="share of free HBM the gradient workspace may use (snapshot / history sizing)")
    ap.add_argument("--cpu-sample-steps", type=int, default=300)
    ap.add_argument("--nt", type=int, default=3000,
                    help="time steps of the gradient workload (the measured configuration has 3000; fewer steps "
                         "keep the same per-launch shapes for small profiling captures)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=48,
                    help="requests of the served mixed-size stream (0 skips the serving measurement)")
    ap.add_argument("--serve-rates", default="10,500",
                    help="Poisson arrival rates of the served stream (1/s), comma separated")
    ap.add_argument("--serve-slots", type=int, default=4, help="concurrent solves of the server")
    ap.add_argument("--fwi-iterations", type=int, default=8,
                    help="iterations of the closed-loop FWI clients on the server (0 skips them)")
    ap.add_argument("--no-elastic", action="store_true", help="skip the VTI-elastic gradient measurement")
    ap.add_argument("--elastic-only", action="store_true", help="run only the VTI-elastic gradient measurement")
    ap.add_argument("--elastic-nt", type=int, default=2000,
                    help="time steps of the elastic workload (2000 measured; fewer for profiling captures)")
    ap.add_argument("--elastic-cpu-steps", type=int, default=100)
    ap.add_argument("--no-extra-legs", action="store_true",
                    help="skip the forward-only, checkpointed, FP64-error and plain-GPU legs")
    ap.add_argument("--ckpt-nt", type=int, default=6000, help="time steps of the checkpointed 500x1500 leg")
    ap.add_argument("--ckpt-shots", type=int, default=8, help="shots (of 64) of the checkpointed 500x1500 leg")
    ap.add_argument("--ckpt-only", action="store_true", help="run only the checkpointed 500x1500 leg")
    ap.add_argument("--ring-depth", type=int, default=0, choices=[0, 1, 2],
                    help="TMA ring of the checkpointed leg's step kernels (0 = automatic, 1 shallow, 2 deep)")
    ap.add_argument("--precision", action="store_true",
                    help="run only the snapshot-precision study (BF16 / FP16 / FP32 checkpoints vs FP64)")
    ap.add_argument("--precision-nt", type=int, default=6000)
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.precision:
        if rank == 0:
            print(json.dumps(precision_study(args)), flush=True)
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args)), flush=True)
        return
    if args.elastic_only:
        if rank == 0:
            torch.cuda.set_device(local)
            print(json.dumps(elastic_arm(args, torch.device("cuda", local))), flush=True)
        return
    if args.ckpt_only:
        if rank == 0:
            torch.cuda.set_device(local)
            print(json.dumps(checkpointed_leg(args, torch.device("cuda", local))), flush=True)
        return
    line = gpu_arm(args, world, rank, local)
    if world == 1 and not args.no_extra_legs:
        dev = torch.device("cuda", local)
        torch.cuda.empty_cache()
        line["accuracy_vs_fp64"] = fp64_error(args, dev, args.memory_fraction)
        torch.cuda.empty_cache()
        line["forward_only"] = forward_legs(args, dev)
        torch.cuda.empty_cache()
        line["checkpointed"] = checkpointed_leg(args, dev)
        torch.cuda.empty_cache()
        line["headline_checkpointed"] = headline_checkpointed_leg(args, dev)
        torch.cuda.empty_cache()
        line["plain_gpu"] = plain_gpu_leg(args, dev)
    if world == 1 and not args.no_elastic:
        torch.cuda.empty_cache()
        line["elastic"] = elastic_arm(args, torch.device("cuda", local))
    if world == 1 and args.serve_requests > 0:
        torch.cuda.empty_cache()
        line["serving"] = serving_arm(args, torch.device("cuda", local))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # bounded sample: repeat a 1-shot slice of the workload until >= 10 s of CPU work
        threads = os.cpu_count() or 1
        done, t_all, reps = 0, 0.0, 0
        while t_all < 10.0 and reps < 50:
            _, t = cpu_sample(args.cpu_sample_steps, threads)
            done += 300 * 700 * args.cpu_sample_steps
            t_all += t
            reps += 1
        line["cpu_baseline"] = {"value": round(done / t_all / 1e9, 5), "unit": UNIT, "cores": threads,
                                "kind": "port", "port_vs_reference_cpu": port_vs_reference(),
                                "sample": "%d x (1 shot x %d steps) of the 300x700 padded gradient workload, CPU "
                                          "oracle forward + autograd backward, %.1f s" % (reps, args.cpu_sample_steps,
                                                                                          t_all)}
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
