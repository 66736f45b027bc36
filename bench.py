#!/usr/bin/env python3
"""Benchmark of the reshape + split-3D-FFT hot path on one GB300.

Workload (one step): a 512x512x512 complex128 global array on an 8x8 virtual
processor grid (64 virtual ranks) moves through the decomposition chain
block -> rotate -> factor_reverse (two reshapes), then the split 3D FFT runs
forward and inverse on the factor_reverse decomposition.  Inputs are seeded
uniform[-1,1) values resident in HBM (2 GiB per array, larger than L2, so no
L2 flush is needed between steps).

Prints one JSON line (see the keys below).  ``--impl reference`` times the
reference algorithm on the host cores instead (the CPU restatement under
oracle/, since the reference itself needs MPI and FFTW, absent on the box).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SIDE = 512
GRID = (8, 8)
P = GRID[0] * GRID[1]
ROT = (1, 170)        # rotate amounts on dims 0 and 1 (1 and L/3)
FREV = ((16, 32), (32, 16))  # factor_reverse (A, B) on dims 0 and 1


def specs(n=N_SIDE, grid=GRID, rot=ROT, frev=FREV):
    g0, g1 = grid
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g0, n, g1, n)
    rotd = "packed:rotate(%d,block(%d,%d))|rotate(%d,block(%d,%d))|local(%d)" % (rot[0], n, g0, rot[1], n, g1, n)
    frv = "packed:frev(%d,%d,block(%d,%d))|frev(%d,%d,block(%d,%d))|local(%d)" % (
        frev[0][0], frev[0][1], n, g0, frev[1][0], frev[1][1], n, g1, n)
    return blk, rotd, frv


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_key):
    """DRAM bytes per launch of a kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(kernel_key)
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flops_per_transform(n_total):
    return 5.0 * n_total * math.log2(n_total)


# ----------------------------------------------------------------------------- GPU arm

def run_gpu(args):
    import numpy as np
    import torch

    from decomp_mpi_gb300 import api

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    blk, rotd, frv = specs()
    comm = api.Comm(P)
    D0 = api.decomp_from_spec(comm, blk)
    D1 = api.decomp_from_spec(comm, rotd)
    D2 = api.decomp_from_spec(comm, frv)
    r01 = api.ReshapePlan(comm, 16, D0, D1)
    r12 = api.ReshapePlan(comm, 16, D1, D2)
    n_total = N_SIDE ** 3
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    gen = torch.Generator(device=dev)
    gen.manual_seed(1)
    a0 = torch.empty(P * r01.src_pitch, dtype=torch.complex128, device=dev)
    a0.real.uniform_(-1, 1, generator=gen)
    a0.imag.uniform_(-1, 1, generator=gen)
    a1 = torch.empty(P * r01.dest_pitch, dtype=torch.complex128, device=dev)
    a2 = torch.empty(P * r12.dest_pitch, dtype=torch.complex128, device=dev)

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    reshape_ms = []

    def step(record=False):
        if record:
            ev[0].record(stream)
        r01.run(a0.data_ptr(), a1.data_ptr(), sh)
        if record:
            ev[1].record(stream)
            ev[2].record(stream)
        r12.run(a1.data_ptr(), a2.data_ptr(), sh)
        if record:
            ev[3].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    total_ms = t0.elapsed_time(t1)
    # per-kernel durations (same stream, separate pass so the headline loop has no extra events)
    for _ in range(args.steps):
        step(record=True)
        torch.cuda.synchronize()
        reshape_ms.append(ev[0].elapsed_time(ev[1]))
        reshape_ms.append(ev[2].elapsed_time(ev[3]))
    clk = clocks.stop()

    # correctness spot check of this run: reshape back and compare (bit-exact permutation)
    r20 = api.ReshapePlan(comm, 16, D2, D0)
    back = torch.empty_like(a0)
    r20.run(a2.data_ptr(), back.data_ptr(), sh)
    torch.cuda.synchronize()
    from oracle import oracle as O  # the checker only
    off = torch.from_numpy(O.global_offsets(P, blk, r01.src_pitch, (N_SIDE,) * 3).ravel()).to(dev)
    exact = bool(torch.equal(back[off], a0[off]))

    ms_per_step = total_ms / args.steps
    bytes_step = r01.bytes_moved + r12.bytes_moved
    gbs = bytes_step / (ms_per_step * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    per_launch_ms = statistics.mean(reshape_ms)
    achieved = r01.bytes_moved / (per_launch_ms * 1e-3) / 1e9

    # end to end through the C-ABI with host buffers: H2D input, two reshapes, D2H result
    host_in = torch.empty(a0.numel(), dtype=torch.complex128, pin_memory=True)
    host_in.copy_(a0.cpu())
    host_out = torch.empty(a2.numel(), dtype=torch.complex128, pin_memory=True)
    for _ in range(max(1, args.warmup // 2)):
        a0.copy_(host_in, non_blocking=True)
        step()
        host_out.copy_(a2, non_blocking=True)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        a0.copy_(host_in, non_blocking=True)
        step()
        host_out.copy_(a2, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e = {"value": round(bytes_step / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GB/s",
           "h2d_bytes_per_step": host_in.numel() * 16, "d2h_bytes_per_step": host_out.numel() * 16,
           "ms_per_step": round(e2e_ms, 4)}

    cpu = cpu_baseline(args, sample_only=True)
    line = {
        "metric": "reshape GB/s (block->rotate->factor_reverse chain, 512^3 complex128, 8x8 virtual grid)",
        "value": round(gbs, 2),
        "unit": "GB/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128",
        "data": "synthetic: uniform[-1,1) complex128, seed 1, resident in HBM",
        "config": {"workload": "512^3 complex128, 8x8 virtual grid, reshape block->rotate(1,170)->"
                               "factor_reverse((16,32),(32,16))", "virtual_ranks": P,
                   "l2": "inputs (2 GiB) larger than L2, no flush", "parallelism": "virtual grid on one GPU"},
        "bit_exact_roundtrip": exact,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": ncu_traffic("reshape_512c128_block_to_rotate"),
                     "kernel": "k1_permute (block->rotate reshape), algorithmic bytes 2*N*16"},
        "e2e": e2e,
        "gpu_launches": (r01.launches + r12.launches) * args.steps,
        "clocks": clk,
        "cpu_baseline": cpu,
        "plans": [r01.describe(), r12.describe()],
    }
    print(json.dumps(line))


# ----------------------------------------------------------------------------- CPU arm (reference algorithm)

def cpu_baseline(args, sample_only=False):
    """The reference's reshape algorithm (oracle restatement: per-peer typemaps, pack and unpack)
    on the host cores, over a bounded sample: the same chain at 256^3 on the same 8x8 grid."""
    import numpy as np

    from oracle import oracle as O

    n = 256
    blk, rotd, frv = specs(n=n, rot=(1, 85), frev=((16, 16), (32, 8)))
    threads = os.cpu_count() or 1
    sp, p1, p2 = O.pitch_of(P, blk), O.pitch_of(P, rotd), O.pitch_of(P, frv)
    rng = np.random.default_rng(1)
    a0 = rng.uniform(-1, 1, P * sp) + 1j * rng.uniform(-1, 1, P * sp)
    a1 = np.zeros(P * p1, np.complex128)
    a2 = np.zeros(P * p2, np.complex128)
    pl1 = O.ReshapePlanCPU(P, blk, rotd, 16)
    pl2 = O.ReshapePlanCPU(P, rotd, frv, 16)
    pl1.run(a0, sp, a1, p1, threads)
    reps = 2 if sample_only else max(1, args.steps)
    t = time.perf_counter()
    for _ in range(reps):
        pl1.run(a0, sp, a1, p1, threads)
        pl2.run(a1, p1, a2, p2, threads)
    dt = (time.perf_counter() - t) / reps
    gbs = 2 * 2 * (n ** 3) * 16 / dt / 1e9
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "reshape chain block->rotate->factor_reverse at 256^3 complex128 on the 8x8 virtual grid, "
                      "reference algorithm restated in C (per-peer typemaps, pack + unpack), %d threads" % threads,
            "ms_per_step": round(dt * 1e3, 2)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cpu = cpu_baseline(args)
    line = {
        "metric": "reshape GB/s (block->rotate->factor_reverse chain, 512^3 complex128, 8x8 virtual grid)",
        "value": cpu["value"], "unit": "GB/s", "n_gpus": int(args.gpus), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": cpu["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic: uniform[-1,1) complex128, seed 1",
        "config": {"workload": "512^3 complex128, 8x8 virtual grid, reshape block->rotate->factor_reverse "
                               "(bounded CPU sample at 256^3)", "virtual_ranks": P},
        "impl": "reference", "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 and int(os.environ.get("RANK", "0")) != 0:
        return  # one GPU per run in this build: extra ranks do no work
    run_gpu(args)


if __name__ == "__main__":
    main()
