#!/usr/bin/env python3
"""Benchmark of the reshape + split-3D-FFT hot path on one GB300.

Workload (one step), the plain FP64 drop-in at scale: a 512x512x512
complex128 global array on an 8x8 virtual processor grid (64 virtual ranks)
moves through the decomposition chain block -> rotate -> factor_reverse (two
reshapes), then the split 3D FFT runs forward and inverse on the
factor_reverse decomposition.  Inputs are seeded uniform[-1,1) values
resident in HBM (2 GiB per array, larger than the 129 MB L2, so no L2 flush
is needed between steps).

Prints one JSON line.  ``value`` is GFLOP/s of the whole step (two 3D
transforms at 5 N log2 N flops each, divided by the time of the full step,
reshapes included); the reshape GB/s and the FFT-only GFLOP/s are reported
beside it.  ``--impl reference`` times the reference algorithm on the host
cores instead (the CPU restatement under oracle/: the reference itself needs
MPI and FFTW, which the GPU machine does not have).
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


def specs(n=N_SIDE, grid=GRID):
    """block -> rotate(1, n/3) -> factor_reverse((16, n/16), (n/16, 16)) on dims 0 and 1; dim 2 local."""
    g0, g1 = grid
    rot = (1, n // 3)
    frev = ((16, n // 16), (n // 16, 16))
    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g0, n, g1, n)
    rotd = "packed:rotate(%d,block(%d,%d))|rotate(%d,block(%d,%d))|local(%d)" % (rot[0], n, g0, rot[1], n, g1, n)
    frv = "packed:frev(%d,%d,block(%d,%d))|frev(%d,%d,block(%d,%d))|local(%d)" % (
        frev[0][0], frev[0][1], n, g0, frev[1][0], frev[1][1], n, g1, n)
    return blk, rotd, frv


def workload_name(n):
    return ("%d^3 complex128, 8x8 virtual grid: reshape block->rotate(1,%d)->factor_reverse((16,%d),(%d,16)), "
            "split 3D FFT forward + inverse" % (n, n // 3, n // 16, n // 16))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(key):
    """DRAM bytes per launch of a kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(key)
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
    import torch

    from decomp_mpi_gb300 import api

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    n = args.n
    blk, rotd, frv = specs(n)
    comm = api.Comm(P)
    D0 = api.decomp_from_spec(comm, blk)
    D1 = api.decomp_from_spec(comm, rotd)
    D2 = api.decomp_from_spec(comm, frv)
    r01 = api.ReshapePlan(comm, 16, D0, D1)
    r12 = api.ReshapePlan(comm, 16, D1, D2)
    n_total = n ** 3
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    gen = torch.Generator(device=dev)
    gen.manual_seed(1)
    a0 = torch.empty(P * r01.src_pitch, dtype=torch.complex128, device=dev)
    a0.real.uniform_(-1, 1, generator=gen)
    a0.imag.uniform_(-1, 1, generator=gen)
    a1 = torch.empty(P * r01.dest_pitch, dtype=torch.complex128, device=dev)
    a2 = torch.empty(P * r12.dest_pitch, dtype=torch.complex128, device=dev)

    # workspace sized as the reference requires: 2 * extent per rank
    probe = api.SplitPlan(D2, 1 << 20, 1 << 40, 1 << 21)
    length = 2 * probe.extent
    probe.free()
    work = torch.empty(P * length, dtype=torch.complex128, device=dev)
    sp = api.SplitPlan(D2, a2.data_ptr(), length, work.data_ptr())

    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]

    def step(record=False):
        if record:
            ev[0].record(stream)
        r01.run(a0.data_ptr(), a1.data_ptr(), sh)
        r12.run(a1.data_ptr(), a2.data_ptr(), sh)
        if record:
            ev[1].record(stream)
        sp.run(api.FFTW_FORWARD, sh)
        if record:
            ev[2].record(stream)
        sp.run(api.FFTW_BACKWARD, sh)
        if record:
            ev[3].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.4)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    total_ms = t0.elapsed_time(t1)
    clk = clocks.stop()

    # component times (a separate pass with events between the parts)
    res_ms, fwd_ms, inv_ms = [], [], []
    for _ in range(max(2, min(args.steps, 5))):
        step(record=True)
        torch.cuda.synchronize()
        res_ms.append(ev[0].elapsed_time(ev[1]))
        fwd_ms.append(ev[1].elapsed_time(ev[2]))
        inv_ms.append(ev[2].elapsed_time(ev[3]))
    # per-pass kernel durations of the dominant kernel (FFT pass), same stream
    sp.set_timing(True)
    step()
    torch.cuda.synchronize()
    sp.run(api.FFTW_FORWARD, sh)
    torch.cuda.synchronize()
    pass_fwd = sp.pass_times(api.FFTW_FORWARD)
    sp.run(api.FFTW_BACKWARD, sh)
    torch.cuda.synchronize()
    pass_inv = sp.pass_times(api.FFTW_BACKWARD)
    sp.set_timing(False)

    # native FP64 arithmetic on the same plan, for comparison
    sp.set_arith(api.ARITH_FP64)
    nat_fwd, nat_inv = [], []
    for i in range(3):
        ev[1].record(stream)
        sp.run(api.FFTW_FORWARD, sh)
        ev[2].record(stream)
        sp.run(api.FFTW_BACKWARD, sh)
        ev[3].record(stream)
        torch.cuda.synchronize()
        if i:
            nat_fwd.append(ev[1].elapsed_time(ev[2]))
            nat_inv.append(ev[2].elapsed_time(ev[3]))
    sp.set_arith(api.ARITH_DF)
    # the other pass schedule on the same plan, for comparison
    other = api.SCHEDULE_SPLIT if sp.schedule == api.SCHEDULE_LINES else api.SCHEDULE_LINES
    used = sp.schedule
    alt_fwd, alt_inv = [], []
    try:
        sp.set_schedule(other)
        for i in range(3):
            ev[1].record(stream)
            sp.run(api.FFTW_FORWARD, sh)
            ev[2].record(stream)
            sp.run(api.FFTW_BACKWARD, sh)
            ev[3].record(stream)
            torch.cuda.synchronize()
            if i:
                alt_fwd.append(ev[1].elapsed_time(ev[2]))
                alt_inv.append(ev[2].elapsed_time(ev[3]))
    except Exception:  # the other schedule does not apply to this shape
        pass
    sp.set_schedule(used)

    # correctness of this run: forward then inverse returns N times the input
    r01.run(a0.data_ptr(), a1.data_ptr(), sh)
    r12.run(a1.data_ptr(), a2.data_ptr(), sh)
    ref = a2.clone()
    sp.run(api.FFTW_FORWARD, sh)
    sp.run(api.FFTW_BACKWARD, sh)
    torch.cuda.synchronize()
    from oracle import oracle as O  # the checker only
    off = torch.from_numpy(O.global_offsets(P, frv, r12.dest_pitch, (n,) * 3).ravel()).to(dev)
    back = a2[off] / n_total
    want = ref[off]
    rt_err = float((torch.linalg.vector_norm(back - want) / torch.linalg.vector_norm(want)).item())
    del off, back, want, ref

    ms_per_step = total_ms / args.steps
    flops_step = 2 * flops_per_transform(n_total)
    gflops = flops_step / (ms_per_step * 1e-3) / 1e9
    reshape_bytes = r01.bytes_moved + r12.bytes_moved
    reshape_gbs = reshape_bytes / (statistics.median(res_ms) * 1e-3) / 1e9
    fft_ms = statistics.median(fwd_ms) + statistics.median(inv_ms)
    fft_gflops = flops_step / (fft_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    launches = pass_fwd + pass_inv
    avg_pass_ms = statistics.mean(launches)
    pass_bytes = 2.0 * n_total * 16  # algorithmic bytes of one pass: read + write the array once
    achieved = pass_bytes / (avg_pass_ms * 1e-3) / 1e9
    fp64_peak = api.load().dmg_probe_fma_tflops(0)
    pass_tflops = flops_per_transform(n_total) / len(pass_fwd) / (avg_pass_ms * 1e-3) / 1e12

    # end to end through the C-ABI with host buffers: H2D input, the step, D2H result
    host_in = torch.empty(a0.numel(), dtype=torch.complex128, pin_memory=True)
    host_in.copy_(a0.cpu())
    host_out = torch.empty(a2.numel(), dtype=torch.complex128, pin_memory=True)
    for _ in range(2):
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
    e2e = {"value": round(flops_step / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GFLOP/s",
           "h2d_bytes_per_step": host_in.numel() * 16, "d2h_bytes_per_step": host_out.numel() * 16,
           "ms_per_step": round(e2e_ms, 3)}

    cpu = cpu_baseline(args, reps=1)
    line = {
        "metric": "3D FFT GFLOP/s (5 N log2 N per transform) + reshape GB/s",
        "value": round(gflops, 2),
        "unit": "GFLOP/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "arithmetic": "complex128 data; double-float (pairs of FP32, 48-bit significand) on the FP32 pipes, "
                      "input scaled by a power of two; native FP64 timed beside it",
        "data": "synthetic: uniform[-1,1) complex128, seed 1, resident in HBM",
        "config": {"workload": workload_name(n), "virtual_ranks": P, "dat_pitch": r12.dest_pitch,
                   "work_length_per_rank": length, "l2": "inputs (2 GiB) larger than L2, no flush",
                   "parallelism": "8x8 virtual grid on one GPU"},
        "fft_gflops": round(fft_gflops, 2),
        "reshape_gbs": round(reshape_gbs, 1),
        "reshape_frac_of_hbm": round(reshape_gbs / peak, 4),
        "ms_breakdown": {"reshapes": round(statistics.median(res_ms), 3),
                         "fft_forward": round(statistics.median(fwd_ms), 3),
                         "fft_inverse": round(statistics.median(inv_ms), 3)},
        "fft_pass_ms": [round(x, 3) for x in launches],
        "native_fp64_ms": {"fft_forward": round(statistics.median(nat_fwd), 3),
                           "fft_inverse": round(statistics.median(nat_inv), 3)},
        "schedule": "lines" if used == api.SCHEDULE_LINES else "split",
        "other_schedule_ms": ({"schedule": "lines" if other == api.SCHEDULE_LINES else "split",
                               "fft_forward": round(statistics.median(alt_fwd), 3),
                               "fft_inverse": round(statistics.median(alt_inv), 3)} if alt_fwd else None),
        "roundtrip_rel_l2": rt_err,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": ncu_traffic("fft_pass_512c128"),
                     "kernel": "fft_pass_kernel<df> (one double-float FFT pass over the array: 2*N*16 B algorithmic)",
                     "fp64_equivalent": {"achieved_tflops": round(pass_tflops, 3),
                                         "native_fp64_peak_tflops": round(fp64_peak, 3),
                                         "note": "5 N log2(n) flops per pass at FP64 accuracy; the native FP64 "
                                                 "peak is the in-library FMA probe"}},
        "e2e": e2e,
        "gpu_launches": (r01.launches + r12.launches + sp.launches(api.FFTW_FORWARD)
                         + sp.launches(api.FFTW_BACKWARD)) * args.steps,
        "clocks": clk,
        "cpu_baseline": cpu,
        "plans": {"reshape": [r01.describe(), r12.describe()], "split": sp.describe()},
    }
    print(json.dumps(line))


# ----------------------------------------------------------------------------- CPU arm (reference algorithm)

def cpu_baseline(args, reps=1, n=256):
    """The reference's algorithm on the host cores over a bounded sample of the workload: the same
    chain and split FFT at n^3 on the same 8x8 grid, restated in C (per-peer typemaps packed and
    unpacked for the reshapes; FFT stages on the oracle's FP64 FFT, standing in for FFTW)."""
    import numpy as np

    from oracle import oracle as O

    blk, rotd, frv = specs(n)
    threads = os.cpu_count() or 1
    sp0, p1, p2 = O.pitch_of(P, blk), O.pitch_of(P, rotd), O.pitch_of(P, frv)
    rng = np.random.default_rng(1)
    a0 = rng.uniform(-1, 1, P * sp0) + 1j * rng.uniform(-1, 1, P * sp0)
    a1 = np.zeros(P * p1, np.complex128)
    a2 = np.zeros(P * p2, np.complex128)
    pl1 = O.ReshapePlanCPU(P, blk, rotd, 16)
    pl2 = O.ReshapePlanCPU(P, rotd, frv, 16)
    wl = 4 * (n ** 3) // P + 64  # at least twice the extent of A and B on every rank
    fft = O.SplitPlanCPU(P, frv, wl)
    work = np.zeros(P * wl, np.complex128)

    def one():
        pl1.run(a0, sp0, a1, p1, threads)
        pl2.run(a1, p1, a2, p2, threads)
        fft.run(a2, p2, work, -1, threads)
        fft.run(a2, p2, work, +1, threads)

    t = time.perf_counter()
    for _ in range(reps):
        one()
    dt = (time.perf_counter() - t) / reps
    flops = 2 * flops_per_transform(n ** 3)
    return {"value": round(flops / dt / 1e9, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": "the same step at %d^3 complex128 on the 8x8 virtual grid (64 ranks on %d threads): "
                      "reshape chain with the reference's per-peer typemaps (pack + unpack) and the split FFT "
                      "with the oracle's FP64 FFT in place of FFTW" % (n, threads),
            "ms_per_step": round(dt * 1e3, 2)}


def run_reference(args):
    if int(os.environ.get("RANK", "0")) != 0:
        return
    cpu = cpu_baseline(args, reps=max(1, min(args.steps, 5)))
    line = {
        "metric": "3D FFT GFLOP/s (5 N log2 N per transform) + reshape GB/s",
        "value": cpu["value"], "unit": "GFLOP/s", "n_gpus": int(args.gpus), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": cpu["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: uniform[-1,1) complex128, seed 1",
        "config": {"workload": workload_name(args.n) + " (bounded CPU sample at 256^3)", "virtual_ranks": P},
        "impl": "reference", "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def sweep_specs(shape, g):
    """block and block<->interleave/rotate/factor_reverse decompositions on a g x g grid (dims 0, 1; dim 2 local)."""
    L0, L1, L2 = shape

    def il(L):
        A = 2 * g if L % (2 * g) == 0 else g
        return "interleave(block(%d,%d),%d)" % (A, g, L // A)

    blk = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (L0, g, L1, g, L2)
    other = {
        "interleave": "packed:%s|%s|local(%d)" % (il(L0), il(L1), L2),
        "rotate": "packed:rotate(%d,block(%d,%d))|rotate(1,block(%d,%d))|local(%d)" % (L0 // 3, L0, g, L1, g, L2),
        "factor_reverse": "packed:frev(16,%d,block(%d,%d))|frev(%d,16,block(%d,%d))|local(%d)" % (
            L0 // 16, L0, g, L1 // 16, L1, g, L2),
    }
    return blk, other


def run_sweep(args):
    """Reshape bandwidth sweep: element value = global linear index, every transition both ways,
    GB/s = 2 * N * element size / time; each case is checked to round-trip exactly."""
    import torch

    from decomp_mpi_gb300 import api

    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    peak, peak_kind = measured_peaks()
    shapes = [(256, 256, 256), (512, 512, 1024), (1024, 1024, 512)]
    if args.quick:
        shapes = shapes[:1]
    for shape in shapes:
        N = shape[0] * shape[1] * shape[2]
        for g in (4, 16, 32):
            blk, others = sweep_specs(shape, g)
            comm = api.Comm(g * g)
            B = api.decomp_from_spec(comm, blk)
            for kind, spec in others.items():
                D = api.decomp_from_spec(comm, spec)
                for dtype, tdt in (("int64", torch.int64), ("complex64", torch.complex64)):
                    for name, (s, d) in (("block->" + kind, (B, D)), (kind + "->block", (D, B))):
                        pl = api.ReshapePlan(comm, 8, s, d)
                        back = api.ReshapePlan(comm, 8, d, s)
                        src = torch.empty(g * g * pl.src_pitch, dtype=torch.int64, device=dev)
                        src.copy_(torch.arange(src.numel(), device=dev))
                        if tdt == torch.complex64:
                            src = src.view(torch.complex64)
                        dst = torch.empty(g * g * pl.dest_pitch, dtype=src.dtype, device=dev)
                        rt = torch.empty_like(src)
                        for _ in range(3):
                            pl.run(src.data_ptr(), dst.data_ptr(), stream.cuda_stream)
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        reps = 5
                        e0.record(stream)
                        for _ in range(reps):
                            pl.run(src.data_ptr(), dst.data_ptr(), stream.cuda_stream)
                        e1.record(stream)
                        back.run(dst.data_ptr(), rt.data_ptr(), stream.cuda_stream)
                        torch.cuda.synchronize()
                        ms = e0.elapsed_time(e1) / reps
                        gbs = pl.bytes_moved / (ms * 1e-3) / 1e9
                        # these decompositions have no padding: every source slot moves and comes back
                        assert g * g * pl.src_pitch == N and pl.elements == N
                        exact = bool(torch.equal(rt, src))
                        print(json.dumps({"sweep": "reshape", "shape": list(shape), "grid": "%dx%d" % (g, g),
                                          "transition": name, "dtype": dtype, "ms": round(ms, 4),
                                          "gbs": round(gbs, 1), "frac_of_hbm": round(gbs / peak, 4),
                                          "peak_kind": peak_kind, "elements": N, "roundtrip_exact": exact,
                                          "plan": pl.describe()}), flush=True)
                        del src, dst, rt
                        pl.free()
                        back.free()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sweep", action="store_true", help="reshape bandwidth sweep (one JSON line per case)")
    ap.add_argument("--quick", action="store_true", help="with --sweep: the 256^3 shapes only")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_SIDE, help="cube side (the headline workload is 512)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 and int(os.environ.get("RANK", "0")) != 0:
        return  # one GPU per run in this build: extra ranks do no work
    if args.sweep:
        run_sweep(args)
        return
    run_gpu(args)


if __name__ == "__main__":
    main()
