"""Time the reference's own CPU propagator against the oracle port on the same slice.

Test infrastructure, run in a container that has the reference (it cannot travel to the GPU
host, where the CPU baseline therefore times the port): one shot x N steps of the 200 x 600
gradient workload (300 x 700 padded, 600 receivers, dt 1.5 ms, 8 Hz Ricker), FP32, forward
records plus the autograd backward of sum(p^2), with the same thread count for both. The
reference runs through its public API (AcousticModel / Survey / AcousticPropagator.forward,
default checkpointing); the port is oracle.acoustic.acoustic_forward, the loop the CPU baseline
of bench.py times. Writes cpu_timing_ref_vs_port.json beside this script.

Usage (repository root): python tests/golden/time_reference_cpu.py [--ref DIR] [--steps N]
"""
import argparse
import json
import os
import platform
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def slice_inputs(n_steps):
    from adfwi_gb300.synthetic import layered_faulted, smooth
    from adfwi_gb300.utils import wavelet
    rng = np.random.default_rng(0)
    vp = smooth(layered_faulted(200, 600, rng), 10.0).astype(np.float32)
    rho = (np.power(vp, 0.25) * 310).astype(np.float32)
    _, wav = wavelet(n_steps, 1.5e-3, 8.0)
    sx = np.linspace(0, 599, 32)[1:-1].round().astype(int)[:1]
    rx = np.arange(600)
    return vp, rho, np.asarray(wav, dtype=np.float32), sx, rx


def time_reference(R, n_steps):
    import torch
    vp, rho, wav, sx, rx = slice_inputs(n_steps)
    model = R["AcousticModel"](0, 0, 600, 200, 20.0, 20.0, vp=vp, rho=rho, vp_grad=True, free_surface=False,
                               abc_type="PML", nabc=50, device="cpu", dtype=torch.float32)
    src = R["Source"](nt=n_steps, dt=1.5e-3, f0=8.0)
    src.add_sources(src_x=sx, src_z=np.full(len(sx), 2), src_wavelet=wav, src_type="mt")
    rcv = R["Receiver"](nt=n_steps, dt=1.5e-3)
    rcv.add_receivers(rcv_x=rx, rcv_z=np.full(len(rx), 2), rcv_type="pr")
    prop = R["AcousticPropagator"](model, R["Survey"](source=src, receiver=rcv), device="cpu",
                                   dtype=torch.float32)
    t0 = time.perf_counter()
    rec = prop.forward()
    rec["p"].square().sum().backward()
    return time.perf_counter() - t0


def time_port(n_steps):
    import torch
    from adfwi_gb300.boundary import bc_pml
    from oracle.acoustic import acoustic_forward
    vp, rho, wav, sx, rx = slice_inputs(n_steps)
    damp = torch.tensor(bc_pml(600, 200, 20.0, 20.0, 50, vp.max(), free_surface=False), dtype=torch.float32)
    vpt = torch.tensor(vp, requires_grad=True)
    t0 = time.perf_counter()
    out = acoustic_forward(vpt, torch.tensor(rho), damp, sx, np.full(len(sx), 2), torch.tensor(wav[None]),
                           rx, np.full(len(rx), 2), nabc=50, free_surface=False, dx=20.0, dz=20.0, dt=1.5e-3)
    out["p"].square().sum().backward()
    return time.perf_counter() - t0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    import torch
    from make_golden import import_reference
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    R = import_reference(args.ref)
    time_reference(R, 20)
    time_port(20)
    ref = [time_reference(R, args.steps) for _ in range(args.reps)]
    port = [time_port(args.steps) for _ in range(args.reps)]
    cells = 300 * 700 * args.steps
    out = {"sample": "1 shot x %d steps of the 300x700 padded gradient workload, FP32, forward + autograd "
                     "backward of sum(p^2)" % args.steps,
           "threads": threads, "machine": platform.machine(), "processor": platform.processor(),
           "reference_s": [round(t, 3) for t in ref], "port_s": [round(t, 3) for t in port],
           "reference_gcell_per_s": round(cells / statistics.median(ref) / 1e9, 5),
           "port_gcell_per_s": round(cells / statistics.median(port) / 1e9, 5),
           "port_over_reference_speed": round(statistics.median(ref) / statistics.median(port), 3)}
    with open(os.path.join(HERE, "cpu_timing_ref_vs_port.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
