#!/usr/bin/env python3
"""Benchmark of the reshape + split-3D-FFT hot path on one GB300.

Workload (one step), the plain FP64 drop-in at scale: a 512x512x512
complex128 global array on an 8x8 virtual processor grid (64 virtual ranks)
moves through the decomposition chain block -> rotate -> factor_reverse (two
reshapes), then the split 3D FFT runs forward and inverse on the
factor_reverse decomposition.  Inputs are seeded uniform[-1,1) values
resident in HBM (2 GiB per array, larger than the 129 MB L2, so no L2 flush
is needed between steps).

With ``--gpus N`` under ``torch.distributed.run`` every rank runs its own
replica of the workload on its own GPU (the path does not shard across GPUs:
the processor grid is virtual, inside one GPU's memory).  The timed region is
bracketed by a barrier on every rank, its duration is the maximum over the
ranks, and ``value`` counts the transforms of all replicas.

Prints one JSON line.  ``value`` is GFLOP/s of the whole step in native
FP64 arithmetic, the reference's (two 3D transforms at 5 N log2 N flops
each, divided by the time of the full step, reshapes included); the reshape
GB/s and the FFT-only GFLOP/s are reported beside it, the same step in
double-float arithmetic under ``double_float``, and (unless --no-extras) a
reshape-sweep subset and a bounded served stream.  ``--impl reference``
times the reference algorithm for the same workload on the host cores
instead (the CPU restatement under oracle/: the reference itself needs MPI
and FFTW, which the GB300 host does not have).
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

    def __init__(self, index=None):
        self.proc = None
        self.lines = []
        self.index = index if index is not None else os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-i", self.index,
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

# GB300's nominal FP64 rate (an FMA counted as two flops); the FP64 passes are bound by this pipe
FP64_PEAK_TFLOPS = 1.25


class Workload:
    """The headline workload on one GPU: the 512^3 complex128 array (seed 1) in the block decomposition, the
    two reshape plans of the chain, the split FFT plan on the factor_reverse decomposition and its
    workspace (2 x extent per rank, as the reference requires)."""

    def __init__(self, n, dev):
        import torch

        from decomp_mpi_gb300 import api

        self.api = api
        self.n = n
        self.N = n ** 3
        blk, rotd, frv = specs(n)
        self.frv = frv
        self.comm = api.Comm(P)
        self.D = [api.decomp_from_spec(self.comm, s) for s in (blk, rotd, frv)]
        self.r01 = api.ReshapePlan(self.comm, 16, self.D[0], self.D[1])
        self.r12 = api.ReshapePlan(self.comm, 16, self.D[1], self.D[2])
        self.stream = torch.cuda.current_stream(dev)
        self.sh = self.stream.cuda_stream
        gen = torch.Generator(device=dev)
        gen.manual_seed(1)
        self.a0 = torch.empty(P * self.r01.src_pitch, dtype=torch.complex128, device=dev)
        self.a0.real.uniform_(-1, 1, generator=gen)
        self.a0.imag.uniform_(-1, 1, generator=gen)
        self.a1 = torch.empty(P * self.r01.dest_pitch, dtype=torch.complex128, device=dev)
        self.a2 = torch.empty(P * self.r12.dest_pitch, dtype=torch.complex128, device=dev)
        probe = api.SplitPlan(self.D[2], 1 << 20, 1 << 40, 1 << 21)
        self.length = 2 * probe.extent
        probe.free()
        self.work = torch.empty(P * self.length, dtype=torch.complex128, device=dev)
        self.sp = api.SplitPlan(self.D[2], self.a2.data_ptr(), self.length, self.work.data_ptr())
        self.ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def step(self, record=False):
        api, ev, sh = self.api, self.ev, self.sh
        if record:
            ev[0].record(self.stream)
        self.r01.run(self.a0.data_ptr(), self.a1.data_ptr(), sh)
        self.r12.run(self.a1.data_ptr(), self.a2.data_ptr(), sh)
        if record:
            ev[1].record(self.stream)
        self.sp.run(api.FFTW_FORWARD, sh)
        if record:
            ev[2].record(self.stream)
        self.sp.run(api.FFTW_BACKWARD, sh)
        if record:
            ev[3].record(self.stream)

    def launches(self):
        api = self.api
        return (self.r01.launches + self.r12.launches + self.sp.launches(api.FFTW_FORWARD)
                + self.sp.launches(api.FFTW_BACKWARD))

    def timed(self, reps, steps, warmup):
        """W untimed steps, then K steps between a barrier and a synchronize on both sides (CUDA events on
        the launching stream); the slowest replica's milliseconds."""
        import torch
        for _ in range(warmup):
            self.step()
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        reps.barrier()
        torch.cuda.synchronize()
        t0.record(self.stream)
        for _ in range(steps):
            self.step()
        t1.record(self.stream)
        torch.cuda.synchronize()
        reps.barrier()
        return reps.max([t0.elapsed_time(t1)])[0]

    def breakdown(self, nrep):
        """Median milliseconds of the two reshapes, the forward and the inverse (events between the parts), and
        the per-pass milliseconds of one forward and one inverse run (events around each pass)."""
        import torch
        api, ev, sp = self.api, self.ev, self.sp
        res_ms, fwd_ms, inv_ms = [], [], []
        for _ in range(nrep):
            self.step(record=True)
            torch.cuda.synchronize()
            res_ms.append(ev[0].elapsed_time(ev[1]))
            fwd_ms.append(ev[1].elapsed_time(ev[2]))
            inv_ms.append(ev[2].elapsed_time(ev[3]))
        sp.set_timing(True)
        sp.run(api.FFTW_FORWARD, self.sh)
        torch.cuda.synchronize()
        pf = sp.pass_times(api.FFTW_FORWARD)
        sp.run(api.FFTW_BACKWARD, self.sh)
        torch.cuda.synchronize()
        pi = sp.pass_times(api.FFTW_BACKWARD)
        sp.set_timing(False)
        return {"reshapes": statistics.median(res_ms), "fft_forward": statistics.median(fwd_ms),
                "fft_inverse": statistics.median(inv_ms), "pass_fwd": pf, "pass_inv": pi}

    def roundtrip_error(self):
        """Forward then inverse of the chain's output returns N times it: relative L2 of the difference
        (on the device, over the slots the decomposition holds)."""
        import torch
        api = self.api
        self.r01.run(self.a0.data_ptr(), self.a1.data_ptr(), self.sh)
        self.r12.run(self.a1.data_ptr(), self.a2.data_ptr(), self.sh)
        ref = self.a2.clone()
        self.sp.run(api.FFTW_FORWARD, self.sh)
        self.sp.run(api.FFTW_BACKWARD, self.sh)
        torch.cuda.synchronize()
        d = self.a2 / self.N - ref
        # padding slots (none in this decomposition) hold the same garbage on both sides
        err = float((torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)).item())
        del ref, d
        return err


def e2e_pipelined(w, reps, steps):
    """End to end through the C-ABI with host buffers: every step uploads its input from pinned host memory and
    reads its result (the inverse's output) back.  Two device buffer sets; step k+1's upload and step k's
    download run on copy streams while the kernels of the neighbouring step run, with events ordering every
    reuse of a buffer.  Returns (pipelined ms per step, serial ms per step, h2d bytes, d2h bytes)."""
    import torch
    api, stream, sh, sp = w.api, w.stream, w.sh, w.sp
    dev = w.a0.device
    host_in = torch.empty(w.a0.numel(), dtype=torch.complex128, pin_memory=True)
    host_in.copy_(w.a0.cpu())
    host_out = [torch.empty(w.a2.numel(), dtype=torch.complex128, pin_memory=True) for _ in range(2)]
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # serial: copy, step, copy on one stream
    for _ in range(2):
        w.a0.copy_(host_in, non_blocking=True)
        w.step()
        host_out[0].copy_(w.a2, non_blocking=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        w.a0.copy_(host_in, non_blocking=True)
        w.step()
        host_out[0].copy_(w.a2, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    serial_ms = e0.elapsed_time(e1) / steps

    sets = [(w.a0, w.a1, w.a2, w.work)] + [(torch.empty_like(w.a0), torch.empty_like(w.a1),
                                            torch.empty_like(w.a2), torch.empty_like(w.work))]
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    ev_up = [torch.cuda.Event() for _ in range(2)]
    ev_comp = [torch.cuda.Event() for _ in range(2)]
    ev_down = [torch.cuda.Event() for _ in range(2)]

    def step_on(k):
        b0, b1, b2, wk = sets[k % 2]
        w.r01.run(b0.data_ptr(), b1.data_ptr(), sh)
        w.r12.run(b1.data_ptr(), b2.data_ptr(), sh)
        sp.set_buffers(b2.data_ptr(), wk.data_ptr())
        sp.run(api.FFTW_FORWARD, sh)
        sp.run(api.FFTW_BACKWARD, sh)

    def pipelined(nsteps, timed):
        if timed:
            e0.record(stream)
        up.wait_stream(stream)
        down.wait_stream(stream)
        with torch.cuda.stream(up):
            sets[0][0].copy_(host_in, non_blocking=True)
        ev_up[0].record(up)
        for k in range(nsteps):
            s = k % 2
            stream.wait_event(ev_up[s])
            if k >= 2:
                stream.wait_event(ev_down[s])  # step k-2's result has left this set
            step_on(k)
            ev_comp[s].record(stream)
            if k + 1 < nsteps:
                if k >= 1:
                    up.wait_event(ev_comp[1 - s])  # step k-1 has consumed the other set's input
                with torch.cuda.stream(up):
                    sets[1 - s][0].copy_(host_in, non_blocking=True)
                ev_up[1 - s].record(up)
            down.wait_event(ev_comp[s])
            with torch.cuda.stream(down):
                host_out[s].copy_(sets[s][2], non_blocking=True)
            ev_down[s].record(down)
        stream.wait_stream(down)
        stream.wait_stream(up)
        if timed:
            e1.record(stream)
        torch.cuda.synchronize()

    pipelined(3, False)
    reps.barrier()
    pipelined(steps, True)
    reps.barrier()
    e2e_ms, serial_ms = reps.max([e0.elapsed_time(e1) / steps, serial_ms])
    sp.set_buffers(w.a2.data_ptr(), w.work.data_ptr())
    del sets
    return e2e_ms, serial_ms, host_in.numel() * 16, host_out[0].numel() * 16


def transform_roof(N, bd64, bddf, peak):
    """The whole forward transform against the split FFT's algorithmic bytes, 4 N s (two HBM round trips, the
    reshapes and the twiddle fused), and against the FP64 pipe (5 N log2 N flops)."""
    out = {"algorithmic_bytes": 4 * N * 16, "flops": flops_per_transform(N)}
    for key, bd in (("fp64", bd64), ("double_float", bddf)):
        t = bd["fft_forward"] * 1e-3
        gbs = 4 * N * 16 / t / 1e9
        out[key] = {"forward_ms": round(bd["fft_forward"], 3), "achieved_gbs": round(gbs, 1),
                    "hbm_frac": round(gbs / peak, 4),
                    "fp64_pipe_frac": round(flops_per_transform(N) / t / 1e12 / FP64_PEAK_TFLOPS, 4)}
    return out


def run_gpu(args):
    import torch

    from decomp_mpi_gb300 import api
    from decomp_mpi_gb300.replicas import Replicas

    # one replica of the whole workload per GPU (the path does not shard across GPUs)
    reps = Replicas()
    dev = torch.device("cuda:%d" % reps.local_rank)
    torch.cuda.set_device(dev)
    reps.init("nccl")
    n = args.n
    w = Workload(n, dev)
    sp = w.sp
    W = reps.world
    flops_step = 2 * flops_per_transform(w.N)
    peak, peak_kind = measured_peaks()

    # ---- the headline: native FP64 arithmetic
    sp.set_arith(api.ARITH_FP64)
    clocks = ClockSampler(reps.gpu_index())
    clocks.start()
    time.sleep(0.4)
    total_ms = w.timed(reps, args.steps, args.warmup)
    clk = clocks.stop()
    launches_per_step = w.launches()
    bd64 = w.breakdown(max(2, min(args.steps, 5)))
    rt64 = w.roundtrip_error()

    # ---- double-float arithmetic (pairs of FP32 on the FP32 pipes): a second, named form
    sp.set_arith(api.ARITH_DF)
    df_total_ms = w.timed(reps, args.steps, args.warmup)
    bddf = w.breakdown(max(2, min(args.steps, 5)))
    rtdf = w.roundtrip_error()
    df_launches = w.launches()

    # ---- end to end through the C-ABI with host buffers, FP64
    sp.set_arith(api.ARITH_FP64)
    e2e_steps = max(args.steps, 10)
    e2e_ms, serial_ms, h2d, d2h = e2e_pipelined(w, reps, e2e_steps)

    ms_per_step = total_ms / args.steps
    df_ms_per_step = df_total_ms / args.steps
    reshape_bytes = w.r01.bytes_moved + w.r12.bytes_moved
    reshape_gbs = reshape_bytes / (bd64["reshapes"] * 1e-3) / 1e9
    pass_bytes = 2.0 * w.N * 16  # algorithmic bytes of one pass: the array read and written once

    def pass_roof(bd):
        launches = bd["pass_fwd"] + bd["pass_inv"]
        avg = statistics.mean(launches)
        achieved = pass_bytes / (avg * 1e-3) / 1e9
        tflops = flops_per_transform(w.N) / len(bd["pass_fwd"]) / (avg * 1e-3) / 1e12
        return launches, avg, achieved, tflops

    l64, avg64, ach64, tf64 = pass_roof(bd64)
    ldf, avgdf, achdf, tfdf = pass_roof(bddf)
    plans = {"reshape": [w.r01.describe(), w.r12.describe()], "split": sp.describe()}
    w_N = w.N
    wl = w.length
    dat_pitch = w.r12.dest_pitch
    del w, sp
    torch.cuda.empty_cache()

    if not reps.leader:
        reps.close()
        return
    extras = {}
    if not args.no_extras:
        extras["reshape_sweep_subset"] = [
            {k: c[k] for k in ("shape", "grid", "transition", "ms", "gbs", "frac_of_hbm", "placement_exact",
                               "roundtrip_exact")}
            for c in sweep_cases([(1024, 1024, 512)], [32], ["int64"])]
        torch.cuda.empty_cache()
        extras["served_stream"] = serve_study(args, njobs=args.jobs)
        torch.cuda.empty_cache()
        extras["precision_form"] = precision_study(1024)
        torch.cuda.empty_cache()
        extras["grouped_small"] = group_study()
        torch.cuda.empty_cache()
        extras["plan_compare"] = compare_study(256, 64)
        torch.cuda.empty_cache()
    cpu = cpu_baseline(args, reps=3)
    line = {
        "metric": "3D FFT GFLOP/s (5 N log2 N per transform) + reshape GB/s",
        "value": round(W * flops_step / (ms_per_step * 1e-3) / 1e9, 2),
        "unit": "GFLOP/s",
        "n_gpus": W,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "arithmetic": "complex128 in native FP64 (the reference's arithmetic); the double-float form is reported "
                      "under double_float",
        "data": "synthetic: uniform[-1,1) complex128, seed 1, resident in HBM",
        "config": {"workload": workload_name(n), "virtual_ranks": P, "dat_pitch": dat_pitch,
                   "work_length_per_rank": wl, "l2": "inputs (2 GiB) larger than L2, no flush",
                   "parallelism": ("8x8 virtual grid on one GPU" if W == 1 else
                                   "8x8 virtual grid per GPU, %d independent replicas" % W)},
        "fft_gflops": round(flops_step / ((bd64["fft_forward"] + bd64["fft_inverse"]) * 1e-3) / 1e9, 2),
        "reshape_gbs": round(reshape_gbs, 1),
        "reshape_frac_of_hbm": round(reshape_gbs / peak, 4),
        "transform_roofline": transform_roof(w_N, bd64, bddf, peak),
        "ms_breakdown": {k: round(bd64[k], 3) for k in ("reshapes", "fft_forward", "fft_inverse")},
        "fft_pass_ms": [round(x, 3) for x in l64],
        "roundtrip_rel_l2": rt64,
        "roofline": {"bound": "hbm", "achieved": round(ach64, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach64 / peak, 4), "peak_kind": peak_kind,
                     "traffic": ncu_traffic("fft_pass_fp64_512c128"),
                     "kernel": "fft_pass_kernel<double> (one FP64 FFT pass over the array: 2*N*16 B algorithmic)",
                     "fp64_pipe": {"achieved_tflops": round(tf64, 3), "peak_tflops": FP64_PEAK_TFLOPS,
                                   "frac": round(tf64 / FP64_PEAK_TFLOPS, 4),
                                   "note": "conventional 5 N log2(n) flops per pass; the pass is bound by the "
                                           "FP64 pipe, whose nominal GB300 rate is the peak"}},
        "double_float": {
            "dtype": "df64", "value": round(W * flops_step / (df_ms_per_step * 1e-3) / 1e9, 2), "unit": "GFLOP/s",
            "ms_per_step": round(df_ms_per_step, 3), "steps": args.steps,
            "arithmetic": "complex128 data; each real an unevaluated sum of two floats (48-bit significand) on the "
                          "FP32 pipes, the input scaled by a power of two",
            "ms_breakdown": {k: round(bddf[k], 3) for k in ("reshapes", "fft_forward", "fft_inverse")},
            "fft_pass_ms": [round(x, 3) for x in ldf], "roundtrip_rel_l2": rtdf,
            "pass_roofline": {"achieved": round(achdf, 1), "peak": peak, "unit": "GB/s", "frac": round(achdf / peak, 4),
                              "traffic": ncu_traffic("fft_pass_512c128"),
                              "kernel": "fft_pass_kernel<df>"},
            "gpu_launches": df_launches * args.steps * W},
        "e2e": {"value": round(W * flops_step / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GFLOP/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_ms, 3), "steps": e2e_steps, "arithmetic": "fp64",
                "note": "pipelined: step k+1's upload and step k's download overlap the kernels of the steps "
                        "beside them",
                "serial_ms_per_step": round(serial_ms, 3),
                "serial_value": round(W * flops_step / (serial_ms * 1e-3) / 1e9, 2)},
        "gpu_launches": launches_per_step * args.steps * W,
        "clocks": clk,
        "cpu_baseline": cpu,
        "plans": plans,
    }
    line.update(extras)
    print(json.dumps(line))
    reps.close()


# ----------------------------------------------------------------------------- CPU arm (reference algorithm)

def _cpu_step_setup(n):
    import numpy as np

    from oracle import oracle as O

    blk, rotd, frv = specs(n)
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
    threads = os.cpu_count() or 1

    def one():
        pl1.run(a0, sp0, a1, p1, threads)
        pl2.run(a1, p1, a2, p2, threads)
        fft.run(a2, p2, work, -1, threads)
        fft.run(a2, p2, work, +1, threads)

    return one, threads


def cpu_baseline(args, reps=3, n=256):
    """The reference's algorithm on the host cores over a bounded sample of the workload: the same chain and
    split FFT at n^3 on the same 8x8 grid, restated in C (per-peer typemaps packed and unpacked for the
    reshapes; FFT stages on the oracle's FP64 FFT, standing in for FFTW).  Mean over `reps` steps after one
    untimed step."""
    one, threads = _cpu_step_setup(n)
    one()
    t = time.perf_counter()
    for _ in range(reps):
        one()
    dt = (time.perf_counter() - t) / reps
    flops = 2 * flops_per_transform(n ** 3)
    return {"value": round(flops / dt / 1e9, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
            "sample": "the same step at %d^3 complex128 on the 8x8 virtual grid (64 ranks on %d threads): "
                      "reshape chain with the reference's per-peer typemaps (pack + unpack) and the split FFT "
                      "with the oracle's FP64 FFT in place of FFTW; mean of %d steps" % (n, threads, reps),
            "ms_per_step": round(dt * 1e3, 2)}


def run_reference(args):
    """The reference arm: the reference's algorithm for the whole workload (same n, same grid, same chain and
    transforms) on the host cores, W untimed steps, then K timed steps; ms_per_step is their mean."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    n = args.n
    one, threads = _cpu_step_setup(n)
    for _ in range(args.warmup):
        one()
    t = time.perf_counter()
    for _ in range(args.steps):
        one()
    dt = (time.perf_counter() - t) / args.steps
    value = round(2 * flops_per_transform(n ** 3) / dt / 1e9, 3)
    cpu = {"value": value, "unit": "GFLOP/s", "cores": threads, "kind": "port",
           "sample": "the whole workload (%d^3 complex128, 8x8 virtual grid: 64 ranks on %d threads), every step: "
                     "the reshape chain with the reference's per-peer typemaps (pack + unpack) and the split FFT "
                     "forward and inverse with the oracle's FP64 FFT in place of FFTW; mean of %d steps"
                     % (n, threads, args.steps),
           "why_port": "the reference's own sources are compiled against the project's MPI/FFTW shims only where "
                       "its checkout is present; the GPU host has neither the checkout nor MPI or FFTW, so the "
                       "timed code is the oracle's step-for-step restatement"}
    line = {
        "metric": "3D FFT GFLOP/s (5 N log2 N per transform) + reshape GB/s",
        "value": value, "unit": "GFLOP/s", "n_gpus": int(args.gpus), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic: uniform[-1,1) complex128, seed 1",
        "config": {"workload": workload_name(n), "virtual_ranks": P},
        "impl": "reference", "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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


def sweep_cases(shapes, grids, dtypes):
    """Reshape bandwidth sweep: every transition both ways, GB/s = 2 * N * element size / time (mean of 5 runs
    after 3).  Each case checks placement (the destination holds every coordinate's global index in its slot,
    against the device index visitor's pattern of the destination) and the exact round trip."""
    import torch

    from decomp_mpi_gb300 import api

    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    peak, peak_kind = measured_peaks()
    out = []
    for shape in shapes:
        N = shape[0] * shape[1] * shape[2]
        for g in grids:
            blk, others = sweep_specs(shape, g)
            comm = api.Comm(g * g)
            B = api.decomp_from_spec(comm, blk)
            for kind, spec in others.items():
                D = api.decomp_from_spec(comm, spec)
                for name, (s, d) in (("block->" + kind, (B, D)), (kind + "->block", (D, B))):
                    pl = api.ReshapePlan(comm, 8, s, d)
                    back = api.ReshapePlan(comm, 8, d, s)
                    # these decompositions have no padding: every source slot moves and comes back
                    assert g * g * pl.src_pitch == N and pl.elements == N
                    src = torch.empty(g * g * pl.src_pitch, dtype=torch.int64, device=dev)
                    want = torch.empty(g * g * pl.dest_pitch, dtype=torch.int64, device=dev)
                    api.fill_index(s, 8, src.data_ptr(), sh)
                    api.fill_index(d, 8, want.data_ptr(), sh)
                    for dtype in dtypes:
                        tdt = torch.int64 if dtype == "int64" else torch.complex64
                        sv = src.view(tdt)
                        dst = torch.empty(g * g * pl.dest_pitch, dtype=tdt, device=dev)
                        rt = torch.empty_like(sv)
                        for _ in range(3):
                            pl.run(sv.data_ptr(), dst.data_ptr(), sh)
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        reps = 5
                        e0.record(stream)
                        for _ in range(reps):
                            pl.run(sv.data_ptr(), dst.data_ptr(), sh)
                        e1.record(stream)
                        back.run(dst.data_ptr(), rt.data_ptr(), sh)
                        torch.cuda.synchronize()
                        ms = e0.elapsed_time(e1) / reps
                        gbs = pl.bytes_moved / (ms * 1e-3) / 1e9
                        out.append({"sweep": "reshape", "shape": list(shape), "grid": "%dx%d" % (g, g),
                                    "transition": name, "dtype": dtype, "ms": round(ms, 4), "gbs": round(gbs, 1),
                                    "frac_of_hbm": round(gbs / peak, 4), "peak_kind": peak_kind, "elements": N,
                                    "placement_exact": bool(torch.equal(dst.view(torch.int64), want)),
                                    "roundtrip_exact": bool(torch.equal(rt, sv)), "plan": pl.describe()})
                        del dst, rt
                    del src, want
                    pl.free()
                    back.free()
    return out


def run_sweep(args):
    """The reshape sweep (one JSON line per case)."""
    shapes = [(256, 256, 256), (512, 512, 1024), (1024, 1024, 512)]
    if args.quick:
        shapes = shapes[:1]
    for c in sweep_cases(shapes, [4, 16, 32], ["int64", "complex64"]):
        print(json.dumps(c), flush=True)


SERVE_SIDES = [48, 64, 96, 120, 128, 160, 192, 240, 256, 320, 384, 480, 512]


def serve_study(args, njobs):
    """Served form: a Poisson stream (2000 req/s, seed 3) of block->rotate + split FFT forward + inverse jobs on
    a 4x4 virtual grid, sides from SERVE_SIDES, complex64 or complex128 with p = 1/2.  Runs the stream on the
    server (stream slots, admission by free HBM, same-shape batching), then the same jobs one at a time on a
    one-slot server without batching, in the same arithmetic ("alone") and with complex128 in native FP64, the
    plain form ("alone_plain_fp64"), and returns all three."""
    import numpy as np
    import torch

    from decomp_mpi_gb300 import api

    grid, P = 4, 16
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, njobs))
    side_set = ([int(x) for x in args.serve_sides.split(",")] if args.serve_sides else
                SERVE_SIDES if not args.quick else SERVE_SIDES[:7])
    sides = rng.choice(side_set, njobs)
    dtypes = np.where(rng.random(njobs) < 0.5, api.C128, api.C64)
    classes = sorted(set(zip(sides.tolist(), dtypes.tolist())))
    flops = float(sum(2 * flops_per_transform(int(sd) ** 3) for sd in sides))

    def make_server(slots, batch, mix=0):
        srv = api.Server(grid, args.arena_gb << 30, slots=slots, max_batch=batch)
        if mix:
            srv.set_mixing(mix)
        return srv

    srv = make_server(args.slots, args.batch, args.mix_side)
    # one input per class (uniform[-1,1)), pinned spectrum / output arrays per class: jobs of a class carry
    # the same values, so concurrent jobs of a class write identical results into them
    bufs = {}
    for side, dt in classes:
        blk, rot = api.cube_specs(side, grid)
        n_in, n_spec, n_out = srv.sizes(side, dt)
        tdt = torch.complex128 if dt == api.C128 else torch.complex64
        g = torch.Generator().manual_seed(side * 7 + dt)
        x = torch.empty(n_in, dtype=tdt)
        x.real.uniform_(-1, 1, generator=g)
        x.imag.uniform_(-1, 1, generator=g)
        bufs[(side, dt)] = (x.pin_memory(), torch.zeros(n_spec, dtype=tdt).pin_memory(),
                            torch.zeros(n_out, dtype=tdt).pin_memory())
    # warm-up: each class once (plans, device tables)
    for c in classes:
        hi, hs, ho = bufs[c]
        srv.submit(c[0], c[1], hi.data_ptr(), hs.data_ptr(), ho.data_ptr())
    srv.drain()
    srv.poll()

    def stream_run(server, paced):
        t0 = time.monotonic()
        ids = {}
        for i in range(njobs):
            if paced:
                wait = t0 + arrivals[i] - time.monotonic()
                if wait > 0:
                    time.sleep(wait)
            c = (int(sides[i]), int(dtypes[i]))
            hi, hs, ho = bufs[c]
            ids[server.submit(c[0], c[1], hi.data_ptr(), hs.data_ptr(), ho.data_ptr())] = i
            if not paced:
                server.drain()
        server.drain()
        t1 = time.monotonic()
        done = server.poll()
        assert len(done) == njobs and all(d["status"] == 0 for d in done), "failed jobs"
        return done, t1 - t0, ids

    done, span, ids = stream_run(srv, paced=True)
    srv.close()
    lat = np.array([d["t_done"] - d["t_submit"] for d in done])
    batches = np.array([d["batch"] for d in done])

    def alone_run(arith128):
        """One slot, no batching, each job run by itself (complex128 plans in `arith128`); per-job service times
        and the latencies the same arrivals would see queueing for that one slot."""
        alone = make_server(1, 1)
        if arith128 is not None:
            alone.set_arith(api.C128, arith128)
        for c in classes:
            hi, hs, ho = bufs[c]
            alone.submit(c[0], c[1], hi.data_ptr(), hs.data_ptr(), ho.data_ptr())
        alone.drain()
        alone.poll()
        adone, aspan, aids = stream_run(alone, paced=False)
        alone.close()
        service = np.zeros(njobs)
        for d in adone:
            service[aids[d["id"]]] = d["t_done"] - d["t_start"]
        finish, qlat = 0.0, np.zeros(njobs)
        for i in range(njobs):
            finish = max(arrivals[i], finish) + service[i]
            qlat[i] = finish - arrivals[i]
        return {"busy_s": round(float(service.sum()), 4), "jobs_per_s": round(njobs / float(service.sum()), 2),
                "gflops": round(flops / float(service.sum()) / 1e9, 2),
                "p50_ms_same_arrivals": round(1e3 * float(np.percentile(qlat, 50)), 3),
                "p99_ms_same_arrivals": round(1e3 * float(np.percentile(qlat, 99)), 3)}

    # the same arithmetic one job at a time, and the plain form (complex128 in native FP64) one job at a time
    alone_same = alone_run(None)
    alone_plain = alone_run(api.ARITH_FP64)
    served_rate = njobs / span

    # accuracy of the round trip per class (the inverse holds N times the rotated input)
    errs = {}
    for side, dt in classes:
        if side > 128:
            continue  # the host check gathers the cube: small classes only
        blk, rot = api.cube_specs(side, grid)
        comm = api.Comm(P)
        pb = api.decomp_from_spec(comm, blk).extent()
        pr = api.decomp_from_spec(comm, rot).extent()
        from oracle import oracle as O  # the parity check only
        hi, hs, ho = bufs[(side, dt)]
        gin = O.gather_global(P, blk, hi.numpy().astype(np.complex128), pb, (side,) * 3)
        gout = O.gather_global(P, rot, ho.numpy().astype(np.complex128), pr, (side,) * 3) / side ** 3
        errs["%d%s" % (side, "c128" if dt == api.C128 else "c64")] = float(
            np.linalg.norm(gout - gin) / np.linalg.norm(gin))
    line = {
        "metric": "served split 3D FFT jobs (forward + inverse): throughput and latency",
        "jobs": njobs, "offered_rate_per_s": args.rate, "arrival_span_s": round(float(arrivals[-1]), 4),
        "served": {"makespan_s": round(span, 4), "jobs_per_s": round(njobs / span, 2),
                   "gflops": round(flops / span / 1e9, 2), "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 3),
                   "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 3),
                   "mean_batch": round(float(batches.mean()), 2), "max_batch": int(batches.max()),
                   "slots": args.slots, "max_batch_limit": args.batch, "arena_gib": args.arena_gb,
                   "mixing_max_side": args.mix_side},
        "arithmetic": "served: complex128 in double-float, complex64 in FP32 (sides up to 512 have no 1024-point "
                      "lines for the tensor-core stages)",
        "alone": alone_same,
        "alone_plain_fp64": alone_plain,
        "served_over_alone": round(served_rate / alone_same["jobs_per_s"], 3),
        "served_over_plain": round(served_rate / alone_plain["jobs_per_s"], 3),
        "roundtrip_rel_l2": errs,
        "config": {"grid": "4x4 virtual", "sides": side_set,
                   "dtypes": "complex64 / complex128, p = 1/2", "seed": 3,
                   "chain": "H2D, block->rotate reshape, split FFT forward, spectrum D2H, inverse, output D2H"},
    }
    return line


def run_serve(args):
    print(json.dumps(serve_study(args, args.jobs)))


def precision_study(n):
    """Precision form: n^3 complex64 (n = 1024 in the benchmark), complex Gaussian N(0,1) (seed 2) plus 16
    unit-amplitude plane waves at random wavenumbers (seed 2), on an 8x8 grid in the block decomposition.
    Split 3D FFT forward in FP32 and in the tensor-core form (the 1024-point DFTs as FP16 hi + lo products
    with FP32 accumulation); the FP64-accuracy reference is the double-float complex128 transform of the same
    values on the GPU (the GPU tests pin the FP32 and tensor-core transforms against an FP64 oracle on the
    host); native FP64 is timed beside it."""
    import numpy as np
    import torch

    from decomp_mpi_gb300 import api

    g = 8
    Pp = g * g
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    comm = api.Comm(Pp)
    spec = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (n, g, n, g, n)
    D = api.decomp_from_spec(comm, spec)
    pitch = D.extent()
    N = n ** 3
    gen = torch.Generator(device=dev)
    gen.manual_seed(2)
    glob = torch.empty(N, dtype=torch.complex64, device=dev)
    glob.real.normal_(0, math.sqrt(0.5), generator=gen)
    glob.imag.normal_(0, math.sqrt(0.5), generator=gen)
    rng = np.random.default_rng(2)
    waves = rng.integers(0, n, size=(16, 3))
    idx = torch.arange(n, device=dev, dtype=torch.float64)
    g3 = glob.view(n, n, n)
    for k in waves:
        e = [torch.exp(2j * math.pi * float(k[d]) * idx / n) for d in range(3)]
        g3 += (e[0][:, None, None] * e[1][None, :, None] * e[2][None, None, :]).to(torch.complex64)
    x64 = torch.empty(Pp * pitch, dtype=torch.complex64, device=dev)
    api.io_scatter(D, 8, glob.data_ptr(), x64.data_ptr(), sh)
    del g3, glob
    x128 = x64.to(torch.complex128)
    probe = api.SplitPlan(D, 1 << 20, 1 << 40, 1 << 21, dtype=api.C64)
    ext = probe.extent64
    probe.free()
    length = 2 * ext
    w64 = torch.empty(Pp * length, dtype=torch.complex64, device=dev)
    sp64 = api.SplitPlan(D, x64.data_ptr(), length, w64.data_ptr(), dtype=api.C64)

    def timed(plan, reps=3):
        plan.run(api.FFTW_FORWARD, sh)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms = []
        for _ in range(reps):
            e0.record(stream)
            plan.run(api.FFTW_FORWARD, sh)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    ms32 = timed(sp64)
    sched64 = "lines" if sp64.schedule == api.SCHEDULE_LINES else "split"
    B = sp64.decomp_B()
    spec32 = w64.view(Pp, length)[:, :ext].contiguous()
    out32 = torch.empty(N, dtype=torch.complex64, device=dev)
    api.io_gather(B, 8, spec32.data_ptr(), out32.data_ptr(), sh)
    # the tensor-core form of the same plan on the same input
    sp64.set_arith(api.ARITH_TC16)
    ms_tc = timed(sp64)
    tc_status = sp64.device_status()
    sp64.set_timing(True)
    sp64.run(api.FFTW_FORWARD, sh)
    torch.cuda.synchronize()
    tc_passes = sp64.pass_times(api.FFTW_FORWARD)
    sp64.set_timing(False)
    spec32 = w64.view(Pp, length)[:, :ext].contiguous()
    outtc = torch.empty(N, dtype=torch.complex64, device=dev)
    api.io_gather(B, 8, spec32.data_ptr(), outtc.data_ptr(), sh)
    sp64.set_arith(api.ARITH_FP32)
    sp64.set_timing(True)
    sp64.run(api.FFTW_FORWARD, sh)
    torch.cuda.synchronize()
    f32_passes = sp64.pass_times(api.FFTW_FORWARD)
    sp64.set_timing(False)
    del spec32, w64
    sp64.free()
    del x64
    w128 = torch.empty(Pp * length, dtype=torch.complex128, device=dev)
    sp128 = api.SplitPlan(D, x128.data_ptr(), length, w128.data_ptr(), dtype=api.C128)
    ms_df = timed(sp128)
    spec128 = w128.view(Pp, length)[:, :ext].contiguous()
    ref = torch.empty(N, dtype=torch.complex128, device=dev)
    api.io_gather(sp128.decomp_B(), 16, spec128.data_ptr(), ref.data_ptr(), sh)
    del spec128
    sp128.set_arith(api.ARITH_FP64)
    ms_fp64 = timed(sp128, reps=2)
    torch.cuda.synchronize()
    diff = out32.to(torch.complex128) - ref
    rel_l2 = float((torch.linalg.vector_norm(diff) / torch.linalg.vector_norm(ref)).item())
    max_abs = float(diff.abs().max().item())
    max_ref = float(ref.abs().max().item())
    del diff
    dtc = outtc.to(torch.complex128) - ref
    tc_rel_l2 = float((torch.linalg.vector_norm(dtc) / torch.linalg.vector_norm(ref)).item())
    tc_max_abs = float(dtc.abs().max().item())
    del dtc
    # planted peaks: frequency k sits in slot s = k / B + A (k % B) of each dimension (the plan's factors)
    A, Bf = sp128.A_factors, [n // a for a in sp128.A_factors]
    peaks32, peaks64 = [], []
    for k in waves:
        s = [int(k[d]) // Bf[d] + A[d] * (int(k[d]) % Bf[d]) for d in range(3)]
        lin = (s[0] * n + s[1]) * n + s[2]
        peaks32.append(abs(complex(out32[lin].item()) - N) / N)
        peaks64.append(abs(complex(ref[lin].item()) - N) / N)
    flops = flops_per_transform(N)
    line = {
        "metric": "precision form: split 3D FFT of 1024^3 complex64, error against an FP64-accuracy transform",
        "config": {"n": n, "grid": "8x8 virtual", "input": "complex N(0,1), seed 2, + 16 unit plane waves (seed 2)",
                   "schedule_c64": sched64,
                   "schedule_c128": "lines" if sp128.schedule == api.SCHEDULE_LINES else "split"},
        "fp32": {"ms": round(ms32, 3), "gflops": round(flops / (ms32 * 1e-3) / 1e9, 1),
                 "hbm_gbs": round(6 * N * 8 / (ms32 * 1e-3) / 1e9, 1),
                 "hbm_note": "three passes, each reading and writing the array once (6 N * 8 bytes)"},
        "double_float_c128": {"ms": round(ms_df, 3), "gflops": round(flops / (ms_df * 1e-3) / 1e9, 1)},
        "native_fp64_c128": {"ms": round(ms_fp64, 3), "gflops": round(flops / (ms_fp64 * 1e-3) / 1e9, 1)},
        "fp32_error": {"rel_l2": rel_l2, "max_abs": max_abs, "max_abs_over_max": max_abs / max_ref,
                       "planted_peak_rel_dev_max": max(peaks32), "reference_peak_rel_dev_max": max(peaks64)},
        "fp32_pass_ms": [round(x, 3) for x in f32_passes],
        "tensor_core": {"ms": round(ms_tc, 3), "gflops": round(flops / (ms_tc * 1e-3) / 1e9, 1),
                        "pass_ms": [round(x, 3) for x in tc_passes],
                        "hbm_gbs": round(6 * N * 8 / (ms_tc * 1e-3) / 1e9, 1), "device_status": tc_status,
                        "error": {"rel_l2": tc_rel_l2, "max_abs": tc_max_abs, "max_abs_over_max": tc_max_abs / max_ref},
                        "arithmetic": "1024-point DFTs as two 32-point DFT products on the tensor cores: FP16 hi + lo "
                                      "operands, three products, FP32 accumulation, a power-of-two scale per row"},
    }
    return line


def run_precision(args):
    print(json.dumps(precision_study(args.n if args.n != N_SIDE else 1024)))


GROUP_SHAPES = [(32, 32, 32), (48, 40, 36), (64, 48, 32), (40, 40, 40), (24, 30, 36), (60, 48, 40), (72, 64, 48),
                (80, 60, 50), (96, 64, 32), (30, 30, 30), (36, 48, 60), (45, 40, 32), (64, 64, 64), (50, 40, 30),
                (96, 96, 48), (20, 24, 30)]


def group_study(steps=20, graphs=True):
    """Grouped form: the 16 uneven small arrays of GROUP_SHAPES (block decomposition on a 4x4 virtual grid,
    uniform[-1,1) values, seed 5), each transformed forward and back per step, (a) one plan at a time with the
    fixed radix schedules, (b) one plan at a time with the runtime radix schedule PLAN8, (c) all 16 in one
    dmg_split_run_group call (one launch per pass index, PLAN8), each eager and replayed from a CUDA graph;
    complex128 in native FP64 and complex64 in FP32.  CUDA events over `steps` steps after 3 warm-up steps."""
    import torch

    from decomp_mpi_gb300 import api

    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    gs, P = 4, 16
    comm = api.Comm(P)
    out = {"metric": "grouped small split 3D FFTs (forward + inverse): transforms per second",
           "shapes": [list(s) for s in GROUP_SHAPES], "grid": "4x4 virtual", "steps": steps}
    points = sum(math.prod(s) for s in GROUP_SHAPES)
    flops = 2 * sum(flops_per_transform(math.prod(s)) for s in GROUP_SHAPES)
    for dt, ar, name in ((api.C128, api.ARITH_FP64, "c128_fp64"), (api.C64, api.ARITH_FP32, "c64_fp32")):
        tdt = torch.complex128 if dt == api.C128 else torch.complex64
        gen = torch.Generator(device=dev)
        gen.manual_seed(5)
        keep, plans = [], []
        for L in GROUP_SHAPES:
            D = api.decomp_from_spec(comm, "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (L[0], gs, L[1], gs, L[2]))
            dat = torch.empty(P * D.extent(), dtype=tdt, device=dev)
            dat.real.uniform_(-1, 1, generator=gen)
            dat.imag.uniform_(-1, 1, generator=gen)
            wl = 2 * int(math.prod(L))
            work = torch.zeros(P * wl, dtype=tdt, device=dev)
            sp = api.SplitPlan(D, dat.data_ptr(), wl, work.data_ptr(), dtype=dt, arith=ar)
            keep.append((D, dat, work))
            plans.append(sp)

        def one_by_one(hs):
            for sp in plans:
                sp.run(api.FFTW_FORWARD, hs)
            for sp in plans:
                sp.run(api.FFTW_BACKWARD, hs)

        def grouped(hs):
            api.split_run_group(plans, api.FFTW_FORWARD, hs)
            api.split_run_group(plans, api.FFTW_BACKWARD, hs)

        def timed(fn):
            for _ in range(3):
                fn(sh)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn(sh)
            e1.record(stream)
            torch.cuda.synchronize()
            eager = e0.elapsed_time(e1) / steps
            if not graphs:
                return {"eager_ms": round(eager, 4),
                        "eager_transforms_per_s": round(2 * len(plans) / (eager * 1e-3), 1)}
            cap = torch.cuda.Stream(dev)
            cap.wait_stream(stream)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=cap):
                fn(torch.cuda.current_stream(dev).cuda_stream)
            for _ in range(3):
                g.replay()
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(steps):
                g.replay()
            e1.record(stream)
            torch.cuda.synchronize()
            graph = e0.elapsed_time(e1) / steps
            del g
            return {"eager_ms": round(eager, 4), "graph_ms": round(graph, 4),
                    "eager_transforms_per_s": round(2 * len(plans) / (eager * 1e-3), 1),
                    "graph_transforms_per_s": round(2 * len(plans) / (graph * 1e-3), 1),
                    "graph_gflops": round(flops / (graph * 1e-3) / 1e9, 1)}

        res = {}
        for sp in plans:
            sp.set_radix(api.RADIX_FIXED)
        res["one_by_one_fixed_radix"] = timed(one_by_one)
        res["one_by_one_fixed_radix"]["launches"] = sum(sp.launches(api.FFTW_FORWARD) + sp.launches(api.FFTW_BACKWARD)
                                                        for sp in plans)
        for sp in plans:
            sp.set_radix(api.RADIX_PLAN8)
        res["one_by_one_plan8"] = timed(one_by_one)
        res["grouped_plan8"] = timed(grouped)
        res["grouped_plan8"]["launches"] = (api.split_group_launches(plans, api.FFTW_FORWARD) +
                                            api.split_group_launches(plans, api.FFTW_BACKWARD))
        res["grouped_over_one_by_one_fixed"] = {
            k: round(res["one_by_one_fixed_radix"][k] / res["grouped_plan8"][k], 3)
            for k in (("eager_ms", "graph_ms") if graphs else ("eager_ms",))}
        out[name] = res
        for sp in plans:
            sp.free()
        del keep
        torch.cuda.empty_cache()
    out["points_per_step"] = 2 * points
    return out


def run_group(args):
    print(json.dumps(group_study(max(args.steps, 10), graphs=not args.no_graph)))


def compare_study(n=256, ranks=64, trials=10, repeat=10):
    """Slab plan against the autotuned plan, the comparison of plan_compare.c:319-358: an n^3 complex128 cube
    (uniform[-1,1), seed 4) in the block decomposition on makeProcessorGrid's grid for `ranks` virtual ranks;
    the slab plan is makeParallelPlan with B = [1, n, n], the other autotuneParallelPlan (workspace 2 x 4 x the
    start extent per rank, the reference's FUDGE).  Each plan: `trials` trials of `repeat` forward transforms
    (CUDA events), best and worst trial, in double-float (the arithmetic the autotuner times) and in native
    FP64."""
    import torch

    from decomp_mpi_gb300 import api

    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    comm = api.Comm(ranks)
    grid = api.processor_grid(comm, [n, n, n])
    start = api.decomp_from_spec(comm, "packed:block(%d,%d)|block(%d,%d)|block(%d,%d)" % (
        n, grid[0], n, grid[1], n, grid[2]))
    ext = start.extent()
    length = 2 * 4 * ext
    gen = torch.Generator(device=dev)
    gen.manual_seed(4)
    dat = torch.empty(ranks * ext, dtype=torch.complex128, device=dev)
    dat.real.uniform_(-1, 1, generator=gen)
    dat.imag.uniform_(-1, 1, generator=gen)
    keep = dat.clone()
    work = torch.zeros(ranks * length, dtype=torch.complex128, device=dev)
    slab = api.SplitPlan(start, dat.data_ptr(), length, work.data_ptr(), B=[1, n, n])
    t0 = time.monotonic()
    api.autotune_cache_clear()
    auto = api.SplitPlan(start, dat.data_ptr(), length, work.data_ptr(), autotune=True)
    tune_s = time.monotonic() - t0
    dat.copy_(keep)  # the autotuner ran transforms on the caller's arrays
    out = {"metric": "slab vs autotuned split plan: forward transform ms (best / worst of %d trials of %d)" % (
        trials, repeat), "n": n, "virtual_ranks": ranks, "start_grid": grid, "autotune_s": round(tune_s, 3),
        "autotune_timed_configs": api.autotune_last_timed()}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for ar, name in ((api.ARITH_DF, "double_float"), (api.ARITH_FP64, "fp64")):
        res = {}
        for label, sp in (("slab", slab), ("auto", auto)):
            sp.set_arith(ar)
            for _ in range(3):
                sp.run(api.FFTW_FORWARD, sh)
            torch.cuda.synchronize()
            per = []
            for _ in range(trials):
                e0.record(stream)
                for _ in range(repeat):
                    sp.run(api.FFTW_FORWARD, sh)
                e1.record(stream)
                torch.cuda.synchronize()
                per.append(e0.elapsed_time(e1) / repeat)
            res[label] = {"A": sp.A_factors, "schedule": "lines" if sp.schedule == api.SCHEDULE_LINES else "split",
                          "best_ms": round(min(per), 4), "worst_ms": round(max(per), 4),
                          "gflops_best": round(flops_per_transform(n ** 3) / (min(per) * 1e-3) / 1e9, 1)}
        res["slab_over_auto_best"] = round(res["slab"]["best_ms"] / res["auto"]["best_ms"], 3)
        out[name] = res
    slab.free()
    auto.free()
    return out


def run_compare(args):
    print(json.dumps(compare_study(args.n if args.n != N_SIDE else 256, args.grid * args.grid)))


def run_fft(args):
    """Split FFT alone: forward and inverse timings (CUDA events, median of 5 after 2 warm-up runs) and per-pass
    times at n^3 on a g x g grid (--grid, 8 by default) in the factor_reverse decomposition of the headline chain
    (or, with --shape L0,L1,L2, in the block decomposition of that shape), for the chosen element type and every
    arithmetic (or the one --arith names) and schedule that applies.  One JSON line."""
    import torch

    from decomp_mpi_gb300 import api

    n = args.n
    dt = api.C64 if args.dtype == "c64" else api.C128
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream
    gs = args.grid
    P = gs * gs
    if args.shape:
        L = [int(x) for x in args.shape.split(",")]
        frv = "packed:block(%d,%d)|block(%d,%d)|local(%d)" % (L[0], gs, L[1], gs, L[2])
    else:
        _, _, frv = specs(n, (gs, gs))
    comm = api.Comm(P)
    D = api.decomp_from_spec(comm, frv)
    tdt = torch.complex128 if dt == api.C128 else torch.complex64
    gen = torch.Generator(device=dev)
    gen.manual_seed(1)
    dat = torch.empty(P * D.extent(), dtype=tdt, device=dev)
    dat.real.uniform_(-1, 1, generator=gen)
    dat.imag.uniform_(-1, 1, generator=gen)
    probe = api.SplitPlan(D, 1 << 20, 1 << 40, 1 << 21, dtype=dt)
    length = 2 * probe.extent64
    probe.free()
    work = torch.empty(P * length, dtype=tdt, device=dev)
    sp = api.SplitPlan(D, dat.data_ptr(), length, work.data_ptr(), dtype=dt)
    if args.tile:
        sp.set_tile(args.tile)
    D_points = math.prod(int(x) for x in args.shape.split(",")) if args.shape else n ** 3
    scheds = {"lines": [api.SCHEDULE_LINES], "split": [api.SCHEDULE_SPLIT],
              "both": [api.SCHEDULE_LINES, api.SCHEDULE_SPLIT]}[args.schedule]
    ariths = [api.ARITH_DF, api.ARITH_FP64] if dt == api.C128 else [api.ARITH_FP32, api.ARITH_TC16]
    if args.arith:
        ariths = [{"fp64": api.ARITH_FP64, "df": api.ARITH_DF, "fp32": api.ARITH_FP32, "tc16": api.ARITH_TC16}[
            args.arith]]
    out = {}
    for sched in scheds:
        try:
            sp.set_schedule(sched)
        except Exception:
            continue
        for ar in ariths:
            sp.set_arith(ar)
            for _ in range(2):
                sp.run(api.FFTW_FORWARD, sh)
                sp.run(api.FFTW_BACKWARD, sh)
            torch.cuda.synchronize()
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            f, b = [], []
            for _ in range(5):
                e[0].record(stream)
                sp.run(api.FFTW_FORWARD, sh)
                e[1].record(stream)
                sp.run(api.FFTW_BACKWARD, sh)
                e[2].record(stream)
                torch.cuda.synchronize()
                f.append(e[0].elapsed_time(e[1]))
                b.append(e[1].elapsed_time(e[2]))
            sp.set_timing(True)
            sp.run(api.FFTW_FORWARD, sh)
            torch.cuda.synchronize()
            passes = sp.pass_times(api.FFTW_FORWARD)
            sp.set_timing(False)
            key = "%s/%s" % ("lines" if sched == api.SCHEDULE_LINES else "split",
                             {api.ARITH_FP64: "fp64", api.ARITH_FP32: "fp32", api.ARITH_DF: "double-float",
                              api.ARITH_TC16: "tensor-core"}[ar])
            out[key] = {"forward_ms": round(statistics.median(f), 3), "inverse_ms": round(statistics.median(b), 3),
                        "forward_pass_ms": [round(x, 3) for x in passes],
                        "forward_gflops": round(flops_per_transform(D_points) / (statistics.median(f) * 1e-3) / 1e9, 1)}
            if n <= 128:
                # small transforms are launch-bound: the same forward + inverse replayed from a CUDA graph
                # (the plan's tables are on the device after the runs above, so capture allocates nothing)
                try:
                    cap = torch.cuda.Stream(dev)
                    cap.wait_stream(stream)
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=cap):
                        hs = torch.cuda.current_stream(dev).cuda_stream
                        sp.run(api.FFTW_FORWARD, hs)
                        sp.run(api.FFTW_BACKWARD, hs)
                    for _ in range(3):
                        g.replay()
                    torch.cuda.synchronize()
                    gt = []
                    for _ in range(20):
                        e[0].record(stream)
                        g.replay()
                        e[1].record(stream)
                        torch.cuda.synchronize()
                        gt.append(e[0].elapsed_time(e[1]))
                    out[key]["graph_forward_inverse_ms"] = round(statistics.median(gt), 4)
                except RuntimeError as err:
                    out[key]["graph_forward_inverse_ms"] = None
                    out[key]["graph_error"] = str(err).splitlines()[0][:200]
                out[key]["eager_forward_inverse_ms"] = round(statistics.median(f) + statistics.median(b), 4)
    print(json.dumps({"mode": "fft", "n": n, "dtype": args.dtype, "grid": "%dx%d virtual" % (gs, gs),
                      "decomposition": frv, **out}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sweep", action="store_true", help="reshape bandwidth sweep (one JSON line per case)")
    ap.add_argument("--quick", action="store_true", help="with --sweep: the 256^3 shapes only")
    ap.add_argument("--gpus", type=int, default=1, help="replicas, one per GPU (under torch.distributed.run)")
    ap.add_argument("--steps", type=int, default=10, help="timed steps")
    ap.add_argument("--warmup", type=int, default=3, help="untimed steps before them (at least 3)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"],
                    help="reference: the reference's algorithm for the same workload on the host cores")
    ap.add_argument("--n", type=int, default=N_SIDE, help="cube side (the headline workload is 512)")
    ap.add_argument("--fft", action="store_true", help="split FFT alone at --n: per-arithmetic, per-schedule times")
    ap.add_argument("--dtype", default="c128", choices=["c128", "c64"], help="with --fft: element type")
    ap.add_argument("--grid", type=int, default=GRID[0], help="with --fft: virtual grid side (g x g ranks)")
    ap.add_argument("--schedule", default="both", choices=["lines", "split", "both"], help="with --fft")
    ap.add_argument("--shape", default="", help="with --fft: L0,L1,L2 in the block decomposition instead of n^3")
    ap.add_argument("--arith", default="", choices=["", "fp64", "df", "fp32", "tc16"],
                    help="with --fft: that arithmetic only")
    ap.add_argument("--tile", type=int, default=0, help="with --fft: values per pass tile (0: the default)")
    ap.add_argument("--serve", action="store_true", help="served form: Poisson stream of mixed-size jobs")
    ap.add_argument("--precision", action="store_true", help="precision form: 1024^3 complex64 with error")
    ap.add_argument("--group", action="store_true", help="grouped form: 16 uneven small transforms per launch")
    ap.add_argument("--no-graph", dest="no_graph", action="store_true",
                    help="with --group: eager runs only (no CUDA graph capture, e.g. under a profiler)")
    ap.add_argument("--compare", action="store_true",
                    help="slab plan vs autotuned plan at --n (256 by default) on --grid^2 virtual ranks")
    ap.add_argument("--jobs", type=int, default=200, help="with --serve: jobs in the stream")
    ap.add_argument("--rate", type=float, default=2000.0, help="with --serve: mean arrivals per second")
    ap.add_argument("--slots", type=int, default=4, help="with --serve: stream slots")
    ap.add_argument("--batch", type=int, default=8, help="with --serve: jobs that may share launches")
    ap.add_argument("--arena-gb", dest="arena_gb", type=int, default=96, help="with --serve: device arena")
    ap.add_argument("--serve-sides", dest="serve_sides", default="",
                    help="with --serve: comma-separated cube sides instead of the C5 set")
    ap.add_argument("--mix-side", dest="mix_side", type=int, default=0,
                    help="with --serve: jobs of sides up to this share launches with other sides (0: off)")
    ap.add_argument("--no-extras", dest="no_extras", action="store_true",
                    help="default run: leave out the reshape-sweep subset and the served stream")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return
    if not (args.sweep or args.fft or args.serve or args.precision or args.group or args.compare):
        run_gpu(args)  # every rank: one replica of the workload per GPU
        return
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 and int(os.environ.get("RANK", "0")) != 0:
        return  # the study modes run on one GPU: extra ranks do no work
    if args.sweep:
        run_sweep(args)
        return
    if args.fft:
        run_fft(args)
        return
    if args.serve:
        run_serve(args)
        return
    if args.precision:
        run_precision(args)
        return
    if args.group:
        run_group(args)
        return
    if args.compare:
        run_compare(args)
        return


if __name__ == "__main__":
    main()
