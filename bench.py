#!/usr/bin/env python
"""Benchmark of the GB300 muFFT FFT path.

Headline (default): one forward c2c FFT of N = 2^24 complex64 points per step
(the multi-pass configuration the metric "c2c GFLOP/s (5N log2 N) + % HBM
roofline" is quoted on), through libmufft_gb300's C ABI:

  value     GFLOP/s = 5 N log2 N / device time per step, inputs resident in HBM,
            rotating over 4 input/output buffer sets of 256 MiB (larger than L2)
  e2e       the same metric through the C ABI on page-locked host buffers,
            every step's host->device copy and device->host copy inside the
            timed region: mufft_gb_execute_plan_1d_host_pipeline (copies of
            neighbouring steps overlap the kernels; median of five runs), with
            mufft_execute_plan_1d() per step beside it
  roofline  the dominant kernel's algorithmic bytes per launch / its average
            CUDA-event duration, each launch timed in place inside whole steps,
            against the measured HBM copy bandwidth; the whole step's figure
            beside it; also a device copy of the same bytes over the same
            rotating buffers (the memory system's ceiling for one pass)
  cpu_baseline  the reference's scalar C path (the oracle port, or the
            reference itself where it was compiled) on all host cores, one
            independent 2^24 transform per thread

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --workload c2c_4096x65536   (other shapes, one JSON line each)

Multi-GPU (torchrun): every rank runs its own replica of the workload (the
transform does not shard without an all-to-all); value = all ranks' flops /
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import csv
import ctypes
import io
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "c2c GFLOP/s (5N·log2N) + % HBM roofline; split-TC vs FP32 at equal FP64 error"

# name -> (N, batch, description)
WORKLOADS = {
    "c2c_2^24": (1 << 24, 1, "c2c forward, N=2^24 complex64, one transform per step (multi-pass)"),
    "c2c_4096x65536": (4096, 65536, "c2c forward, batch 65536 x N=4096 complex64 (single pass)"),
    "c2c_1024x4096": (1024, 4096, "c2c forward, batch 4096 x N=1024 complex64 (single pass)"),
}


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def committed_traffic(workload: str, kernel: str) -> float | None:
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    try:
        return float(json.loads(p.read_text())[workload][kernel]["bytes_per_launch"])
    except (KeyError, ValueError, TypeError):
        return None


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.out = b""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self) -> dict | None:
        if not self.out:
            return None
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in csv.reader(io.StringIO(self.out.decode(errors="replace"))):
            if len(row) < 9:
                continue
            try:
                sm.append(float(row[1]))
                smax.append(float(row[2]))
            except ValueError:
                continue
            for name, v in zip(names, row[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        # samples "under load" = the upper half of the clock samples window
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- distributed

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ CPU baseline

def cpu_baseline(N: int, batch: int, threads: int, rounds: int = 1, prefer_reference: bool = True) -> dict:
    """Reference scalar path on host cores.  Each thread runs its own
    transforms (muFFT plans are single-threaded, fft.c:60)."""
    from mufft_gb300 import signals
    from oracle.oracle import load_oracle, load_reference
    ref = load_reference() if prefer_reference else None
    kind = "reference" if ref is not None else "port"
    x = signals.complex_uniform(2, N)
    per_thread = max(1, min(batch, 8) if batch > 1 else 1)
    flops = 5.0 * N * math.log2(N)
    if ref is not None:
        from mufft_gb300.capi import aligned_copy, aligned_zeros
        xin = aligned_copy(x, np.complex64)
        outs = [aligned_zeros(N, np.complex64) for _ in range(threads)]
        plans = [ref.create_plan_1d_c2c(N, -1, 0) for _ in range(threads)]

        def work(i):
            for _ in range(per_thread * rounds):
                ref.execute_plan_1d(plans[i], outs[i].ctypes.data, xin.ctypes.data)
        ths = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        el = time.perf_counter() - t0
        for p in plans:
            ref.free_plan_1d(p)
    else:
        ora = load_oracle()
        out = np.empty((threads, N), np.complex64)
        plan = ora.create_plan_1d_c2c(N, -1, 0)
        t0 = time.perf_counter()
        for _ in range(per_thread * rounds):
            # every thread transforms the same input into its own output row
            ora.lib.oracle_execute_plan_1d_many(plan, out.ctypes.data, x.ctypes.data, threads, N * 8, 0, threads)
        el = time.perf_counter() - t0
        ora.free_plan_1d(plan)
    total = flops * threads * per_thread * rounds
    return {"value": total / el / 1e9, "unit": "GFLOP/s", "cores": threads, "kind": kind,
            "sample": f"{threads} threads x {per_thread * rounds} c2c N={N} forward transforms "
                      f"({'reference muFFT, portable C tier' if kind == 'reference' and os.uname().machine != 'x86_64' else kind}), "
                      f"{el:.2f} s wall", "seconds": el}


# ------------------------------------------------------------------- ours

def run_ours(args, world, rank, local, pg) -> dict | None:
    import torch

    import mufft_gb300
    from mufft_gb300 import signals

    torch.cuda.set_device(local)
    lib = mufft_gb300.load()
    N, B, desc = WORKLOADS[args.workload]
    if args.batch:
        B = args.batch
        desc += f" [batch overridden to {B}]"
    flops_step = 5.0 * N * math.log2(N) * B
    algo_bytes_pass = 16.0 * N * B  # each pass reads and writes every point once (complex64)

    # schedule: measured choice (plan-time autotuning, outside the timed region)
    from mufft_gb300 import capi as K
    pflags = {"none": 0, "bf16x3": K.FLAG_SPLIT_BF16X3, "bf16x2": K.FLAG_SPLIT_BF16X2}[args.split]
    tuned = pflags == 0 and lib.gb_autotune_1d(0, N, -1, 0, B, None, 0) == 0
    plan = lib.gb_create_plan_1d_c2c_batched(N, -1, pflags, B, 0, 0)
    if not plan:
        raise RuntimeError(lib.gb_last_error_string().decode())
    launches = lib.gb_plan_1d_launches(plan)
    elems = N * B
    nsets = max(2, min(8, math.ceil(4 * 2 ** 30 / (16 * elems))))  # >= 4 GiB of rotating buffers
    nsets = 4 if elems * 16 >= 2 ** 28 else nsets
    x = signals.complex_uniform(2, elems)
    xt = torch.from_numpy(x).cuda()
    ins = [xt.clone() for _ in range(nsets)]
    outs = [torch.empty_like(xt) for _ in range(nsets)]
    del xt
    st = torch.cuda.current_stream()
    sp = st.cuda_stream

    def step(i):
        rc = lib.gb_execute_plan_1d_async(plan, outs[i % nsets].data_ptr(), ins[i % nsets].data_ptr(), sp)
        if rc:
            raise RuntimeError(lib.gb_last_error_string().decode())

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()

    # accuracy of one output against FP64 (outside the timed region)
    acc = None
    if rank == 0 and N * B <= (1 << 24):
        got = outs[(args.warmup - 1) % nsets].cpu().numpy().reshape(B, N)[: min(B, 64)]
        ref = np.fft.fft(x.reshape(B, N)[: min(B, 64)].astype(np.complex128), axis=-1)
        acc = {"rel_l2_vs_fp64": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
               "max_abs_vs_fp64": float(np.abs(got - ref).max())}

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        # the timed steps last milliseconds: run the same steps back to back
        # for about a second first (untimed), so that the clock samples taken
        # around the timed region see the GPU under this load
        t_soak = time.perf_counter()
        i = 0
        while time.perf_counter() - t_soak < 1.0:
            for _ in range(50):
                step(i)
                i += 1
            torch.cuda.synchronize()
        barrier(pg)
        torch.cuda.synchronize()
        torch.cuda.profiler.start()  # the capture range of `ncu --profile-from-start off`
        ev0.record(st)
        for i in range(args.steps):
            step(args.warmup + i)
        ev1.record(st)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        barrier(pg)
    ms = ev0.elapsed_time(ev1)
    ms_max = max_over_ranks(pg, ms)
    ms_step = ms_max / args.steps

    # per-kernel timing for the roofline (outside the headline region): each
    # launch timed in place, inside whole steps (CUDA events between the
    # launches of a step), so that it meets the cache state the launch before
    # it leaves -- the passes hand their intermediate over in L2
    per_kernel = [0.0] * launches
    reps = max(5, args.steps)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(launches + 1)] for _ in range(reps)]
    for i in range(reps):
        evs[i][0].record(st)
        for k in range(launches):
            rc = lib.gb_execute_plan_1d_launches_async(plan, outs[i % nsets].data_ptr(), ins[i % nsets].data_ptr(),
                                                       k, 1, sp)
            assert rc == 0
            evs[i][k + 1].record(st)
    torch.cuda.synchronize()
    for i in range(reps):
        for k in range(launches):
            per_kernel[k] += evs[i][k].elapsed_time(evs[i][k + 1]) / reps
    # the same bytes moved by a device copy over the same rotating sets: the
    # memory system's ceiling for one pass of this size
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i in range(2):
        outs[i % nsets].copy_(ins[i % nsets])
    e0.record(st)
    for i in range(reps):
        outs[i % nsets].copy_(ins[i % nsets])
    e1.record(st)
    torch.cuda.synchronize()
    copy_ms = e0.elapsed_time(e1) / reps
    dbuf = ctypes.create_string_buffer(4096)
    lib.gb_plan_1d_describe(plan, dbuf, 4096)
    kernels = dbuf.value.decode().split("; ")
    dom = int(np.argmax(per_kernel))
    peaks = load_peaks()
    achieved = algo_bytes_pass / (per_kernel[dom] * 1e-3) / 1e9
    traffic = committed_traffic(args.workload, f"launch{dom}")

    # end to end with pinned host buffers through the C ABI: the pipelined
    # execute (copies of neighbouring transforms overlap the kernels), and for
    # comparison the reference's synchronous mufft_execute_plan_1d per step
    e2e = None
    if rank == 0 or world > 1:
        nbytes = elems * 8
        if B == 1 and not pflags:
            hplan = lib.create_plan_1d_c2c(N, -1, 0)
        else:
            hplan = lib.gb_create_plan_1d_c2c_batched(N, -1, pflags, B, 0, 0)
        hin = [lib.alloc(nbytes) for _ in range(2)]
        hout = [lib.alloc(nbytes) for _ in range(2)]
        for h in hin:
            ctypes.memmove(h, x.ctypes.data, nbytes)
        e2e_steps = max(4, min(args.steps, 16))
        ins_l = (ctypes.c_void_p * e2e_steps)(*[hin[i % 2] for i in range(e2e_steps)])
        outs_l = (ctypes.c_void_p * e2e_steps)(*[hout[i % 2] for i in range(e2e_steps)])
        assert lib.gb_execute_plan_1d_host_pipeline(hplan, outs_l, ins_l, e2e_steps) == 0  # warm (device slots)
        lib.execute_plan_1d(hplan, hout[0], hin[0])  # warm (staging buffers)
        # the host link is shared with the other GPUs' jobs on the machine:
        # five timed runs of the steps, the median reported
        runs = []
        for _ in range(5):
            barrier(pg)
            t0 = time.perf_counter()
            rc = lib.gb_execute_plan_1d_host_pipeline(hplan, outs_l, ins_l, e2e_steps)
            el = time.perf_counter() - t0
            if rc:
                raise RuntimeError(lib.gb_last_error_string().decode())
            runs.append(max_over_ranks(pg, el))
        el = float(np.median(runs))
        last = (e2e_steps - 1) % 2
        piped = np.frombuffer((ctypes.c_char * nbytes).from_address(hout[last]), np.uint32).copy()
        t0 = time.perf_counter()
        for i in range(e2e_steps):
            lib.execute_plan_1d(hplan, hout[i % 2], hin[i % 2])
        el_sync = time.perf_counter() - t0
        lib.check("e2e execute")
        el_sync = max_over_ranks(pg, el_sync)
        synced = np.frombuffer((ctypes.c_char * nbytes).from_address(hout[last]), np.uint32)
        e2e_ok = bool(np.array_equal(piped, synced))
        for h in hin + hout:
            lib.free(h)
        lib.free_plan_1d(hplan)
        e2e = {"value": world * flops_step * e2e_steps / el / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "ms_per_step": 1e3 * el / e2e_steps, "steps": e2e_steps,
               "runs_ms_per_step": [round(1e3 * r / e2e_steps, 4) for r in runs],
               "api": "mufft_gb_execute_plan_1d_host_pipeline over the steps' page-locked host buffers (each "
                      "step's input copied in and output copied out inside the timed region, copies of neighbouring "
                      "steps overlapping); median of five timed runs",
               "output_bitwise_equal_to_sync_api": e2e_ok,
               "sync_fft_h": {"value": world * flops_step * e2e_steps / el_sync / 1e9,
                              "ms_per_step": 1e3 * el_sync / e2e_steps,
                              "api": "mufft_execute_plan_1d (fft.h) per step, copies and kernels in turn"}}

    lib.free_plan_1d(plan)
    if rank != 0:
        return None
    res = {
        "metric": METRIC,
        "value": world * flops_step / (ms_step * 1e-3) / 1e9,
        "unit": "GFLOP/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if not pflags else f"f32 via {args.split} tensor-core limbs",
        "data": "synthetic: complex64, re/im i.i.d. uniform [-1,1), SplitMix64 seed 2",
        "config": {"workload": desc + ("" if not pflags else f" [{args.split} split precision]"), "N": N, "batch": B,
                   "parallelism": f"replicas x{world}",
                   "l2": f"inputs larger than L2: {nsets} rotating input/output sets of {16 * elems / 2**20:.0f} MiB",
                   "schedule": kernels,
                   "schedule_choice": "autotuned at plan time (mufft_gb_autotune_1d)" if tuned else "default heuristic"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                     "kernel": kernels[dom], "kernel_ms": per_kernel[dom],
                     "algorithmic_bytes_per_launch": algo_bytes_pass,
                     "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)" if peaks["source"] == "measured"
                     else "fallback 6.8 TB/s",
                     "per_kernel_ms": per_kernel,
                     "per_kernel_timing": "each launch timed in place inside whole steps (CUDA events between "
                                          "the launches), so a pass pays the write-backs the pass before it left",
                     "step": {"algorithmic_bytes": algo_bytes_pass * launches,
                              "achieved": algo_bytes_pass * launches / (ms_step * 1e-3) / 1e9,
                              "frac": algo_bytes_pass * launches / (ms_step * 1e-3) / 1e9 / peaks["hbm_gbs"],
                              "frac_at_two_sweeps": 2 * 16 * elems / (ms_step * 1e-3) / 1e9 / peaks["hbm_gbs"]
                              if launches > 1 else None},
                     "frac_of_nominal_8tbs": achieved / 8000.0,
                     "same_bytes_device_copy_ms": copy_ms,
                     "frac_of_same_bytes_copy": copy_ms / per_kernel[dom]},
        "e2e": e2e,
        "gpu_launches": launches * args.steps,
        "clocks": clk.summary(),
        "accuracy": acc,
    }
    if world == 1 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(N, B, threads=os.cpu_count() or 1)
    if world == 1 and not args.no_companions:
        del ins, outs
        torch.cuda.empty_cache()
        wanted = set(COMPANIONS) if args.companions == "all" else set(args.companions.split(","))
        for name, fn in COMPANIONS.items():
            if name in wanted:
                res[name] = fn(lib, torch)
    return res


# ------------------------------------------------------- companion measurements
#
# Measured once per run next to the headline (rank 0, one GPU), each on its
# own workload: the split-precision tensor-core form against plain FP32, the
# ragged batched convolution against per-request launches, and one
# filter-fitting gradient step through the convolution adjoints.

def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_ms(torch, fn, reps: int, warm: int = 2) -> float:
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = _events(torch)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def companion_batched_1024(lib, torch) -> dict:
    """4096 x c2c N=1024 (32 MiB per set), rotating over 8 input/output sets so
    every transform reads HBM, not L2."""
    from mufft_gb300 import signals
    N, B, sets = 1024, 4096, 8
    sp = torch.cuda.current_stream().cuda_stream
    lib.gb_autotune_1d(0, N, -1, 0, B, None, 0)
    plan = lib.gb_create_plan_1d_c2c_batched(N, -1, 0, B, 0, 0)
    x = signals.complex_uniform(1, N * B)
    ins = [torch.from_numpy(x).cuda() for _ in range(sets)]
    outs = [torch.empty_like(ins[0]) for _ in range(sets)]
    it = [0]

    def run():
        i = it[0] % sets
        it[0] += 1
        lib.gb_execute_plan_1d_async(plan, outs[i].data_ptr(), ins[i].data_ptr(), sp)

    ms = _time_ms(torch, run, reps=64, warm=8)
    it[0] = 0

    def copy():
        i = it[0] % sets
        it[0] += 1
        outs[i].copy_(ins[i])

    # the same bytes moved by a device copy under the same rotation: the ceiling
    # for a kernel of this size (the measured peak is a large-buffer figure)
    ms_copy = _time_ms(torch, copy, reps=64, warm=8)
    lib.gb_execute_plan_1d_async(plan, outs[0].data_ptr(), ins[0].data_ptr(), sp)
    torch.cuda.synchronize()
    got = outs[0].cpu().numpy().reshape(B, N)[:64]
    ref = np.fft.fft(x.reshape(B, N)[:64].astype(np.complex128), axis=1)
    buf = ctypes.create_string_buffer(1024)
    lib.gb_plan_1d_describe(plan, buf, 1024)
    lib.free_plan_1d(plan)
    peaks = load_peaks()
    gbs = 16.0 * N * B / (ms * 1e-3) / 1e9
    return {"workload": "c2c forward, batch 4096 x N=1024 complex64, 8 rotating 32 MiB sets", "ms": ms,
            "GFLOP/s": 5.0 * N * 10 * B / (ms * 1e-3) / 1e9, "GB/s": gbs, "frac_of_measured_hbm": gbs / peaks["hbm_gbs"],
            "same_bytes_device_copy_ms": ms_copy, "frac_of_same_size_copy": ms_copy / ms,
            "schedule": buf.value.decode(),
            "rel_l2_vs_fp64": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            "max_abs_vs_fp64": float(np.abs(got - ref).max())}


def companion_2d(lib, torch) -> dict:
    """4096 x 4096 real grid: r2c then c2r (round trip), N(0,1) samples."""
    from mufft_gb300 import signals
    Nx = Ny = 4096
    sp = torch.cuda.current_stream().cuda_stream
    x = signals.normal(2, Nx * Ny).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    dX = torch.empty(Ny * Nx, dtype=torch.complex64, device="cuda")   # rows of Nx complex, Nx/2+1 valid
    dy = torch.empty(2 * Nx * Ny, dtype=torch.float32, device="cuda")  # the c2r output contract: 2 Nx Ny floats
    pf = lib.create_plan_2d_r2c(Nx, Ny, 0)
    pb = lib.create_plan_2d_c2r(Nx, Ny, 0)
    ms_f = _time_ms(torch, lambda: lib.gb_execute_plan_2d_async(pf, dX.data_ptr(), dx.data_ptr(), sp), reps=20)
    ms_b = _time_ms(torch, lambda: lib.gb_execute_plan_2d_async(pb, dy.data_ptr(), dX.data_ptr(), sp), reps=20)
    lib.gb_execute_plan_2d_async(pf, dX.data_ptr(), dx.data_ptr(), sp)
    torch.cuda.synchronize()
    spec = dX.cpu().numpy().reshape(Ny, Nx)[:, : Nx // 2 + 1]
    ref = np.fft.rfft2(x.reshape(Ny, Nx).astype(np.float64))
    fwd_rel = float(np.linalg.norm(spec - ref) / np.linalg.norm(ref))
    fwd_max = float(np.abs(spec - ref).max())
    del spec, ref
    lib.gb_execute_plan_2d_async(pb, dy.data_ptr(), dX.data_ptr(), sp)
    torch.cuda.synchronize()
    back = dy[: Nx * Ny].cpu().numpy() / (Nx * Ny)
    lf, lb = lib.gb_plan_2d_launches(pf), lib.gb_plan_2d_launches(pb)
    lib.free_plan_2d(pf)
    lib.free_plan_2d(pb)
    half = Ny * (Nx // 2 + 1) * 8.0   # complex half spectrum
    real = Nx * Ny * 4.0
    # algorithmic bytes: rows read the reals and write the half spectrum, columns read and write it
    bytes_f = (real + half) + 2 * half
    return {"workload": "2D r2c + c2r, 4096 x 4096 float32 N(0,1), output 4096 x 2049 complex64",
            "r2c_ms": ms_f, "c2r_ms": ms_b, "r2c_launches": lf, "c2r_launches": lb,
            "r2c_GB/s": bytes_f / (ms_f * 1e-3) / 1e9, "c2r_GB/s": bytes_f / (ms_b * 1e-3) / 1e9,
            "r2c_rel_l2_vs_fp64": fwd_rel, "r2c_max_abs_vs_fp64": fwd_max,
            "round_trip_rel_l2": float(np.linalg.norm(back - x) / np.linalg.norm(x)),
            "bytes_note": "algorithmic: row pass reads 64 MiB reals and writes the 4096 x 2049 half spectrum, "
                          "column pass reads and writes the half spectrum"}


def companion_stream_conv(lib, torch) -> dict:
    """Streaming partitioned convolution: stereo blocks of 1024 frames through
    a 2^20-tap filter (1024 partitions), one graph launch per block."""
    from mufft_gb300 import signals
    block, taps = 1024, 1 << 20
    t = np.arange(taps)
    h = (signals.normal(7, taps) * np.exp(-t / 8192.0)).astype(np.float32)
    sp = torch.cuda.current_stream().cuda_stream
    res = {}
    for fused in (1, 0):
        opts = lib.options(stream_conv_fused=fused)
        conv = lib.gb_create_stream_conv(block, 1, h.ctypes.data, taps, 0, ctypes.byref(opts))
        if not conv:
            raise RuntimeError(lib.gb_last_error_string().decode())
        res[fused] = (_time_ms(torch, lambda: lib.gb_stream_conv_process(conv, sp), reps=200, warm=20),
                      lib.gb_stream_conv_fused(conv), lib.gb_stream_conv_ranges(conv))
        if lib.gb_stream_conv_status(conv) != 0:
            raise RuntimeError(lib.gb_last_error_string().decode())
        lib.gb_free_stream_conv(conv)
    ms, fused, ranges = res[1]
    P = taps // block
    mac_bytes = 2.0 * P * (2 * block) * 8  # filter spectra + delay line, every block
    return {"workload": "stereo stream, 1024-frame blocks, 2^20-tap filter (1024 uniform partitions)",
            "ms_per_block": ms, "frames_per_s": block / (ms * 1e-3),
            "realtime_factor_48khz": (block / 48000.0) / (ms * 1e-3),
            "mac_GB/s": mac_bytes / (ms * 1e-3) / 1e9,
            "launch": "one fused launch per block" if fused else "graph of separate launches",
            "partition_ranges": ranges,
            "graph_of_launches_ms_per_block": res[0][0]}


def companion_split(lib, torch) -> dict:
    """65536 x c2c N=4096: plain FP32 vs BF16x3 / BF16x2 split tensor-core
    forms, time and error against FP64 on both input sets."""
    from mufft_gb300 import capi as K
    from mufft_gb300 import signals
    N, B, sub = 4096, 65536, 128
    sp = torch.cuda.current_stream().cuda_stream
    x = torch.empty((B, N), dtype=torch.complex64, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(3)
    x.real.uniform_(-1, 1, generator=g)
    x.imag.uniform_(-1, 1, generator=g)
    xa = signals.complex_uniform(3, sub * N).reshape(sub, N)
    xb = signals.complex_logmag(3, sub * N).reshape(sub, N)
    x[:sub] = torch.from_numpy(xa).cuda()
    y = torch.empty_like(x)
    refa = np.fft.fft(xa.astype(np.complex128), axis=1)
    refb = np.fft.fft(xb.astype(np.complex128), axis=1)
    dxb = torch.from_numpy(xb).cuda()
    dyb = torch.empty_like(dxb)
    out = {"workload": "c2c forward, batch 65536 x N=4096 complex64 (2 GiB in, 2 GiB out)",
           "engines": "bf16x3 / bf16x2: tcgen05.mma with TMEM accumulators; bf16x3_mma_sync: warp-level mma.sync",
           "sets": "A: re/im uniform [-1,1) (first 128 rows SplitMix64 seed 3, rest torch seed 3); "
                   "B: magnitude log-uniform 1e-3..1e3, uniform phase (128 rows)"}
    for name, flags, engine in (("fp32", 0, 0), ("bf16x3", K.FLAG_SPLIT_BF16X3, 0), ("bf16x2", K.FLAG_SPLIT_BF16X2, 0),
                                ("bf16x3_mma_sync", K.FLAG_SPLIT_BF16X3, 1)):
        opts = lib.options(split_engine=engine)
        p = lib.gb_create_plan_1d(0, N, -1, flags, B, 0, 0, ctypes.byref(opts))
        ps = lib.gb_create_plan_1d(0, N, -1, flags, sub, 0, 0, ctypes.byref(opts))
        if not p or not ps:
            raise RuntimeError(lib.gb_last_error_string().decode())
        ms = _time_ms(torch, lambda: lib.gb_execute_plan_1d_async(p, y.data_ptr(), x.data_ptr(), sp), reps=10)
        lib.gb_execute_plan_1d_async(ps, dyb.data_ptr(), dxb.data_ptr(), sp)
        torch.cuda.synchronize()
        ga, gb = y[:sub].cpu().numpy(), dyb.cpu().numpy()
        out[name] = {"ms": ms, "GFLOP/s": 5.0 * N * 12 * B / (ms * 1e-3) / 1e9,
                     "GB/s": 16.0 * N * B / (ms * 1e-3) / 1e9,
                     "rel_l2_set_a": float(np.linalg.norm(ga - refa) / np.linalg.norm(refa)),
                     "max_abs_set_a": float(np.abs(ga - refa).max()),
                     "rel_l2_set_b": float(np.linalg.norm(gb - refb) / np.linalg.norm(refb)),
                     "max_abs_set_b": float(np.abs(gb - refb).max())}
        lib.free_plan_1d(p)
        lib.free_plan_1d(ps)
    out["bf16x3_time_vs_fp32"] = out["bf16x3"]["ms"] / out["fp32"]["ms"]
    out["bf16x3_error_vs_fp32"] = out["bf16x3"]["rel_l2_set_a"] / out["fp32"]["rel_l2_set_a"]
    del x, y
    torch.cuda.empty_cache()
    return out


def companion_ragged(lib, torch) -> dict:
    from mufft_gb300 import capi as K
    from mufft_gb300 import signals
    PADS = K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST | K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND
    sp = torch.cuda.current_stream().cuda_stream
    reqs = signals.ragged_conv_requests(4, 512)
    creq = (K.ConvRequest * len(reqs))()
    plans, keep, seq, algo = {}, [], [], 0.0
    for i, (N, stereo, x, h) in enumerate(reqs):
        m = PADS | (1 if stereo else 0)
        if (N, m) not in plans:
            plans[(N, m)] = lib.create_plan_conv(N, 0, m)
        p = plans[(N, m)]
        nblk = lib.conv_get_transformed_block_size(p) // 8
        hp = np.zeros(N, np.float32)
        hp[: N // 2] = h
        dh_time = torch.from_numpy(hp).cuda()
        dH = torch.empty(nblk, dtype=torch.complex64, device="cuda")
        assert lib.gb_execute_conv_input_async(p, K.CONV_BLOCK_SECOND, dH.data_ptr(), dh_time.data_ptr(), sp) == 0
        din = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        dspec = torch.empty(nblk, dtype=torch.complex64, device="cuda")
        dout = torch.empty(N, dtype=torch.complex64 if stereo else torch.float32, device="cuda")
        dseq = torch.empty_like(dout)
        keep += [dh_time, dH, din, dspec, dout, dseq]
        creq[i] = K.ConvRequest(N, m, din.data_ptr(), dH.data_ptr(), dout.data_ptr())
        seq.append((p, din, dH, dspec, dseq))
        algo += (14 if stereo else 8) * N
    batch = lib.gb_create_conv_batch(creq, len(reqs), 0, None)
    if not batch:
        raise RuntimeError(lib.gb_last_error_string().decode())

    def run_seq():
        for p, din, dH, dspec, dseq in seq:
            lib.gb_execute_conv_input_async(p, K.CONV_BLOCK_FIRST, dspec.data_ptr(), din.data_ptr(), sp)
            lib.gb_execute_conv_output_async(p, dseq.data_ptr(), dspec.data_ptr(), dH.data_ptr(), sp)

    ms_batch = _time_ms(torch, lambda: lib.gb_execute_conv_batch(batch, sp), reps=20)
    ms_seq = _time_ms(torch, run_seq, reps=5)
    # accuracy: every request against an FP64 linear convolution (zero padding
    # makes the circular convolution of length N a linear one)
    worst = 0.0
    for i, (N, stereo, x, h) in enumerate(reqs):
        got = keep[6 * i + 4].cpu().numpy()
        ref = np.fft.ifft(np.fft.fft(np.asarray(x, np.complex128), N) * np.fft.fft(np.asarray(h, np.float64), N))
        ref = ref if stereo else ref.real
        worst = max(worst, float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    lib.gb_free_conv_batch(batch)
    for p in plans.values():
        lib.free_plan_conv(p)
    return {"workload": "512 conv requests, N = 2^e with e ~ U{8..16}, 256 STEREO_MONO, N/2-sample inputs, "
                        "N/2-tap filters (both zero-pad flags), seed 4",
            "batch_ms": ms_batch, "sequential_ms": ms_seq, "speedup_vs_sequential": ms_seq / ms_batch,
            "sequential": "per request mufft_gb_execute_conv_input_async(FIRST) + _conv_output_async on one stream",
            "algorithmic_GB/s": algo / (ms_batch * 1e-3) / 1e9,
            "worst_rel_l2_vs_fp64": worst}


def companion_ragged_fft(lib, torch) -> dict:
    """512 transform requests of mixed kinds and sizes as one batch (one
    persistent launch) against one plan execute per request."""
    from mufft_gb300 import capi as K
    from mufft_gb300 import signals
    sp = torch.cuda.current_stream().cuda_stream
    reqs = signals.ragged_fft_requests(6, 512)
    creq = (K.FftRequest * len(reqs))()
    plans, keep, seq, outs = {}, [], [], []
    for i, (N, kind, direction, flags, x) in enumerate(reqs):
        nout = N if kind == 0 or (kind == 1 and flags & K.FLAG_FULL_R2C) else (N // 2 + 1 if kind == 1 else N)
        din = torch.from_numpy(np.ascontiguousarray(x)).cuda()
        dt = torch.float32 if kind == 2 else torch.complex64
        dout = torch.empty(nout, dtype=dt, device="cuda")
        dseq = torch.empty_like(dout)
        creq[i] = K.FftRequest(N, kind, direction, flags, din.data_ptr(), dout.data_ptr())
        key = (N, kind, direction, flags)
        if key not in plans:
            plans[key] = lib.gb_create_plan_1d(kind, N, direction, flags, 1, 0, 0, None)
        keep += [din, dseq]
        outs.append(dout)
        seq.append((plans[key], dseq, din))
    batch = lib.gb_create_fft_batch(creq, len(reqs), 0, None)
    if not batch:
        raise RuntimeError(lib.gb_last_error_string().decode())
    buf = ctypes.create_string_buffer(256)
    lib.gb_fft_batch_describe(batch, buf, 256)
    desc = buf.value.decode()
    algo = float(desc.split("algorithmic_bytes=")[1])

    def run_seq():
        for p, dseq, din in seq:
            lib.gb_execute_plan_1d_async(p, dseq.data_ptr(), din.data_ptr(), sp)

    ms_batch = _time_ms(torch, lambda: lib.gb_execute_fft_batch(batch, sp), reps=50, warm=5)
    ms_seq = _time_ms(torch, run_seq, reps=5)
    if lib.gb_fft_batch_status(batch) != 0:
        raise RuntimeError(lib.gb_last_error_string().decode())
    # accuracy: every request against an FP64 numpy transform of the same kind
    worst = 0.0
    for (N, kind, direction, flags, x), dout in zip(reqs, outs):
        got = dout.cpu().numpy()
        xin = np.zeros(N, np.complex128 if kind == 0 else np.float64)
        if kind == 0:
            xin[: len(x)] = x
            ref = np.fft.fft(xin) if direction < 0 else np.fft.ifft(xin) * N
        elif kind == 1:
            xin[: len(x)] = x
            ref = np.fft.fft(xin)[: len(got)]
        else:
            # the c2r definition for any N/2 + 1 bins (kernel.c:36-45, fft.c:441-455): the
            # pre-pass Z[i] = (a + b) + (a - b) w_i, a = X[i], b = conj(X[M - i]),
            # w_i = i exp(i pi i / M), then an unnormalised inverse of M points
            X = x.astype(np.complex128)
            M = N // 2
            i = np.arange(M)
            a, b = X[:M], np.conj(X[M - i])
            Z = (a + b) + (a - b) * (1j * np.exp(1j * np.pi * i / M))
            z = np.fft.ifft(Z) * M
            ref = np.empty(N)
            ref[0::2], ref[1::2] = z.real, z.imag
        worst = max(worst, float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    lib.gb_free_fft_batch(batch)
    for p in plans.values():
        lib.free_plan_1d(p)
    return {"workload": "512 transform requests, N = 2^e with e ~ U{4..16}; c2c forward / c2c inverse / r2c / c2r "
                        "with equal odds, a quarter of c2c and r2c zero-padded, half of r2c FULL_R2C, seed 6",
            "batch_ms": ms_batch, "sequential_ms": ms_seq, "speedup_vs_sequential": ms_seq / ms_batch,
            "sequential": "per request mufft_gb_execute_plan_1d_async on one stream (one plan per shape)",
            "algorithmic_GB/s": algo / (ms_batch * 1e-3) / 1e9, "schedule": desc,
            "worst_rel_l2_vs_fp64": worst}


def companion_adjoint(lib, torch) -> dict:
    """One filter-fitting gradient step: 64 stereo signals of 2^20 frames,
    2^16 taps, N = 2^21 (zero-padded blocks make the convolution linear)."""
    from mufft_gb300 import capi as K
    B, L, T = 64, 1 << 20, 1 << 16
    N = 2 * L
    m = K.CONV_METHOD_FLAG_STEREO_MONO | K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST | \
        K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND
    sp = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    x[:, :L].real.uniform_(-1, 1, generator=g)
    x[:, :L].imag.uniform_(-1, 1, generator=g)
    t = torch.arange(T, device="cuda", dtype=torch.float32)
    h_hidden = torch.zeros(N, device="cuda")
    h_hidden[:T] = torch.randn(T, device="cuda", generator=g) * torch.exp(-t / 8192)
    h = torch.zeros(N, device="cuda")
    h[:T] = torch.randn(T, device="cuda", generator=g) * torch.exp(-t / 8192)
    plan = lib.create_plan_conv(N, 0, m)
    nblk = lib.conv_get_transformed_block_size(plan) // 8
    A = torch.empty((B, nblk), dtype=torch.complex64, device="cuda")
    for b in range(B):  # first-block spectra, cached across steps
        assert lib.gb_execute_conv_input_async(plan, K.CONV_BLOCK_FIRST, A[b].data_ptr(), x[b].data_ptr(), sp) == 0
    H = torch.empty(nblk, dtype=torch.complex64, device="cuda")
    ystar = torch.empty((B, N), dtype=torch.complex64, device="cuda")
    lib.gb_execute_conv_input_async(plan, K.CONV_BLOCK_SECOND, H.data_ptr(), h_hidden.data_ptr(), sp)
    for b in range(B):
        lib.gb_execute_conv_output_async(plan, ystar[b].data_ptr(), A[b].data_ptr(), H.data_ptr(), sp)
    y = torch.empty_like(ystar)
    gx = torch.empty_like(ystar)
    gh = torch.empty(N, device="cuda")
    lr = 1e-7

    def gd_step():
        assert lib.gb_execute_conv_input_async(plan, K.CONV_BLOCK_SECOND, H.data_ptr(), h.data_ptr(), sp) == 0
        assert lib.gb_execute_conv_output_batched(plan, y.data_ptr(), N, A.data_ptr(), nblk, H.data_ptr(), B, sp) == 0
        y.sub_(ystar)  # residual r = conv(x, h) - y*
        assert lib.gb_conv_adjoint(plan, gh.data_ptr(), gx.data_ptr(), N, y.data_ptr(), N, A.data_ptr(), nblk,
                                   H.data_ptr(), B, sp) == 0
        h[:T].sub_(lr * gh[:T])

    def gd_step_per_signal():  # the same step through the one-signal entry points
        assert lib.gb_execute_conv_input_async(plan, K.CONV_BLOCK_SECOND, H.data_ptr(), h.data_ptr(), sp) == 0
        for b in range(B):
            lib.gb_execute_conv_output_async(plan, y[b].data_ptr(), A[b].data_ptr(), H.data_ptr(), sp)
        y.sub_(ystar)
        assert lib.gb_conv_adjoint_filter(plan, gh.data_ptr(), y.data_ptr(), N, A.data_ptr(), nblk, B, sp) == 0
        for b in range(B):
            lib.gb_conv_adjoint_input(plan, gx[b].data_ptr(), y[b].data_ptr(), H.data_ptr(), sp)
        h[:T].sub_(lr * gh[:T])

    ms = _time_ms(torch, gd_step, reps=5)
    ms_per_signal = _time_ms(torch, gd_step_per_signal, reps=3)

    # accuracy: both gradients for two of the signals against FP64 (numpy)
    y2 = torch.empty((2, N), dtype=torch.complex64, device="cuda")
    gh2 = torch.empty(N, device="cuda")
    gx0 = torch.empty(N, dtype=torch.complex64, device="cuda")
    lib.gb_execute_conv_input_async(plan, K.CONV_BLOCK_SECOND, H.data_ptr(), h.data_ptr(), sp)
    for b in range(2):
        lib.gb_execute_conv_output_async(plan, y2[b].data_ptr(), A[b].data_ptr(), H.data_ptr(), sp)
    y2.sub_(ystar[:2])
    lib.gb_conv_adjoint_filter(plan, gh2.data_ptr(), y2.data_ptr(), N, A.data_ptr(), nblk, 2, sp)
    lib.gb_conv_adjoint_input(plan, gx0.data_ptr(), y2[0].data_ptr(), H.data_ptr(), sp)
    torch.cuda.synchronize()
    xs = x[:2].cpu().numpy().astype(np.complex128)
    hp = np.zeros(N)
    hp[: N // 2] = h[: N // 2].cpu().numpy()
    hs = np.zeros(N)
    hs[: N // 2] = h_hidden[: N // 2].cpu().numpy()
    Xf, Hf, Hs = np.fft.fft(xs, axis=1), np.fft.fft(hp), np.fft.fft(hs)
    r = np.fft.ifft(Xf * Hf, axis=1) - np.fft.ifft(Xf * Hs, axis=1).astype(np.complex64)
    R = np.fft.fft(r, axis=1)
    gh_ref = np.fft.ifft((R * np.conj(Xf)).sum(axis=0)).real
    gx_ref = np.fft.ifft(R[0] * np.conj(Hf))
    acc = {"grad_filter_rel_l2_vs_fp64": float(np.linalg.norm(gh2.cpu().numpy() - gh_ref) / np.linalg.norm(gh_ref)),
           "grad_input_rel_l2_vs_fp64": float(np.linalg.norm(gx0.cpu().numpy() - gx_ref) / np.linalg.norm(gx_ref)),
           "checked": "2 of the 64 signals, FP64 numpy gradients of the same residual"}
    # 200 steps of filter fitting from h = 0 (filter gradient only), step size
    # 1 / max_k sum_b |A_b[k]|^2; the loss of every step is reduced on the
    # device and read back once at the end
    lr_fit = 1.0 / float((A.real.square() + A.imag.square()).sum(dim=0).max())
    h.zero_()
    losses = torch.empty(200, dtype=torch.float64, device="cuda")

    def fit_step(i):
        assert lib.gb_execute_conv_input_async(plan, K.CONV_BLOCK_SECOND, H.data_ptr(), h.data_ptr(), sp) == 0
        assert lib.gb_execute_conv_output_batched(plan, y.data_ptr(), N, A.data_ptr(), nblk, H.data_ptr(), B, sp) == 0
        y.sub_(ystar)
        losses[i] = 0.5 * (y.real.square() + y.imag.square()).sum(dtype=torch.float64)
        assert lib.gb_conv_adjoint(plan, gh.data_ptr(), None, 0, y.data_ptr(), N, A.data_ptr(), nblk,
                                   H.data_ptr(), B, sp) == 0
        h[:T].sub_(lr_fit * gh[:T])

    torch.cuda.synchronize()
    f0, f1 = _events(torch)
    f0.record()
    for i in range(200):
        fit_step(i)
    f1.record()
    torch.cuda.synchronize()
    fit_ms = f0.elapsed_time(f1)
    lh = losses.cpu().numpy()
    descent = {"steps": 200, "wall_ms": fit_ms, "ms_per_step": fit_ms / 200, "first_loss": float(lh[0]),
               "last_loss": float(lh[-1]),
               "monotone_until_fp32_floor": bool(all(lh[i] < lh[i - 1] for i in range(1, 200)
                                                     if lh[i - 1] > 1e-9 * lh[0])),
               "step": "filter spectrum + batched conv output + residual + loss + filter adjoint + update, "
                       "from h = 0, step size 1 / max_k sum_b |A_b[k]|^2"}
    lib.free_plan_conv(plan)
    # transforms per step: B conv outputs, B output-gradient spectra (shared by
    # both adjoints), B input-gradient inverses, the filter spectrum and its c2r
    fft_flops = 5.0 * N * math.log2(N) * (3 * B + 2)
    del x, A, ystar, y, gx
    torch.cuda.empty_cache()
    return {"workload": "64 stereo signals x 2^20 frames, 2^16-tap filter, N = 2^21, loss 0.5||conv(x,h) - y*||^2",
            "step_ms": ms,
            "step": "filter spectrum + batched conv output (64 signals) + residual + both adjoints in one call "
                    "(one forward transform per output gradient) + update; first-block spectra cached",
            "per_signal_step_ms": ms_per_signal,
            "fft_GFLOP/s": fft_flops / (ms * 1e-3) / 1e9, "accuracy": acc, "descent_200": descent}


COMPANIONS = {
    "batched_1024": companion_batched_1024,
    "fft2d_4096": companion_2d,
    "split_tc": companion_split,
    "ragged_conv": companion_ragged,
    "ragged_fft": companion_ragged_fft,
    "adjoint": companion_adjoint,
    "stream_conv": companion_stream_conv,
}


# ------------------------------------------------------------ profiling cases
#
# `python bench.py --profile-case NAME`: one small workload, warmed up, then
# one iteration inside cudaProfilerStart/Stop, for `ncu --profile-from-start
# off` captures of the kernels that the headline line does not run.

def profile_case(name: str) -> None:
    import torch

    import mufft_gb300
    from mufft_gb300 import capi as K
    from mufft_gb300 import signals
    lib = mufft_gb300.load()
    sp = torch.cuda.current_stream().cuda_stream
    PADS = K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST | K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND
    keep = []

    def region(fn, warm=2):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        fn()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()

    if name == "c2c_1024x4096":  # batch 4096 x c2c N=1024 (32 MiB per buffer), the tuned schedule
        N, B = 1024, 4096
        lib.gb_autotune_1d(0, N, -1, 0, B, None, 0)
        p = lib.gb_create_plan_1d_c2c_batched(N, -1, 0, B, 0, 0)
        x = torch.from_numpy(signals.complex_uniform(1, N * B)).cuda()
        y = torch.empty_like(x)
        region(lambda: lib.gb_execute_plan_1d_async(p, y.data_ptr(), x.data_ptr(), sp))
    elif name == "fft2d_4096":  # 4096 x 4096 r2c then c2r
        Nx = Ny = 4096
        x = torch.randn(Nx * Ny, device="cuda")
        X = torch.empty(Nx * Ny, dtype=torch.complex64, device="cuda")
        y = torch.empty(2 * Nx * Ny, device="cuda")
        pf, pb = lib.create_plan_2d_r2c(Nx, Ny, 0), lib.create_plan_2d_c2r(Nx, Ny, 0)

        def f():
            lib.gb_execute_plan_2d_async(pf, X.data_ptr(), x.data_ptr(), sp)
            lib.gb_execute_plan_2d_async(pb, y.data_ptr(), X.data_ptr(), sp)
        region(f)
    elif name in ("conv_2e21", "adjoint_2e21x8"):
        N = 1 << 21
        p = lib.create_plan_conv(N, 0, K.CONV_METHOD_FLAG_STEREO_MONO | PADS)
        nb = lib.conv_get_transformed_block_size(p) // 8
        if name == "conv_2e21":  # one stereo convolution: input FIRST, SECOND, output
            x = torch.zeros(N, dtype=torch.complex64, device="cuda")
            x[: N // 2] = torch.from_numpy(signals.complex_uniform(3, N // 2)).cuda()
            h = torch.zeros(N, device="cuda")
            h[:65536] = torch.randn(65536, device="cuda")
            A, H = torch.empty(nb, dtype=torch.complex64, device="cuda"), torch.empty(nb, dtype=torch.complex64,
                                                                                     device="cuda")
            out = torch.empty(N, dtype=torch.complex64, device="cuda")

            def f():
                lib.gb_execute_conv_input_async(p, K.CONV_BLOCK_FIRST, A.data_ptr(), x.data_ptr(), sp)
                lib.gb_execute_conv_input_async(p, K.CONV_BLOCK_SECOND, H.data_ptr(), h.data_ptr(), sp)
                lib.gb_execute_conv_output_async(p, out.data_ptr(), A.data_ptr(), H.data_ptr(), sp)
        else:  # one gradient step's kernels for 8 stereo signals: batched outputs + both adjoints
            B = 8
            A = torch.randn((B, nb), dtype=torch.complex64, device="cuda")
            H = torch.randn(nb, dtype=torch.complex64, device="cuda")
            r = torch.randn((B, N), dtype=torch.complex64, device="cuda")
            y, gx, gh = torch.empty_like(r), torch.empty_like(r), torch.empty(N, device="cuda")

            def f():
                lib.gb_execute_conv_output_batched(p, y.data_ptr(), N, A.data_ptr(), nb, H.data_ptr(), B, sp)
                lib.gb_conv_adjoint(p, gh.data_ptr(), gx.data_ptr(), N, r.data_ptr(), N, A.data_ptr(), nb,
                                    H.data_ptr(), B, sp)
        region(f)
    elif name == "ragged_fft_512":  # the 512-request transform batch
        reqs = signals.ragged_fft_requests(6, 512)
        creq = (K.FftRequest * len(reqs))()
        for i, (N, kind, d, fl, x) in enumerate(reqs):
            din = torch.from_numpy(np.ascontiguousarray(x)).cuda()
            nout = N if kind == 0 or (kind == 1 and fl & K.FLAG_FULL_R2C) else (N // 2 + 1 if kind == 1 else N)
            dout = torch.empty(nout, dtype=torch.float32 if kind == 2 else torch.complex64, device="cuda")
            keep.extend([din, dout])
            creq[i] = K.FftRequest(N, kind, d, fl, din.data_ptr(), dout.data_ptr())
        b = lib.gb_create_fft_batch(creq, len(reqs), 0, None)
        region(lambda: lib.gb_execute_fft_batch(b, sp))
        assert lib.gb_fft_batch_status(b) == 0
    elif name == "ragged_conv_512":  # the 512-request convolution batch
        reqs = signals.ragged_conv_requests(4, 512)
        creq = (K.ConvRequest * len(reqs))()
        for i, (N, stereo, x, h) in enumerate(reqs):
            m = PADS | (1 if stereo else 0)
            nblk = N if stereo else N // 2 + 4
            din = torch.from_numpy(np.ascontiguousarray(x)).cuda()
            dH = torch.randn(nblk, dtype=torch.complex64, device="cuda")
            dout = torch.empty(N, dtype=torch.complex64 if stereo else torch.float32, device="cuda")
            keep.extend([din, dH, dout])
            creq[i] = K.ConvRequest(N, m, din.data_ptr(), dH.data_ptr(), dout.data_ptr())
        b = lib.gb_create_conv_batch(creq, len(reqs), 0, None)
        region(lambda: lib.gb_execute_conv_batch(b, sp))
        assert lib.gb_conv_batch_status(b) == 0
    else:
        raise SystemExit(f"unknown profile case {name}")
    print(json.dumps({"profile_case": name, "ok": True}))


PROFILE_CASES = ("c2c_1024x4096", "fft2d_4096", "conv_2e21", "adjoint_2e21x8", "ragged_fft_512", "ragged_conv_512")


def run_reference(args, world, rank, pg) -> dict | None:
    if rank != 0:
        return None
    N, B, desc = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(N, B, threads)
    samples = [cpu_baseline(N, B, threads) for _ in range(args.steps)]
    secs = sum(s["seconds"] for s in samples)
    value = statistics.mean(s["value"] for s in samples)
    base = samples[0]
    return {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "GFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: complex64, re/im i.i.d. uniform [-1,1), SplitMix64 seed 2",
        "config": {"workload": desc, "N": N, "batch": B, "parallelism": f"{threads} host threads"},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": threads, "kind": base["kind"],
                         "sample": base["sample"]},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c2c_2^24")
    ap.add_argument("--batch", type=int, default=0, help="override the workload's batch (profiling runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--split", choices=["none", "bf16x3", "bf16x2"], default="none",
                    help="run the workload's plan in split precision on the tensor cores (N = 256 or 4096)")
    ap.add_argument("--no-companions", action="store_true",
                    help="skip the split-precision, ragged-convolution and adjoint measurements")
    ap.add_argument("--companions", default="all",
                    help="comma-separated companion measurements to run (default all: " + ",".join(COMPANIONS) + ")")
    ap.add_argument("--profile-case", choices=PROFILE_CASES,
                    help="run one small workload inside a profiler range (for ncu) and exit")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    args.warmup = max(3, args.warmup)
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        res = run_reference(args, world, rank, pg)
    else:
        res = run_ours(args, world, rank, local, pg)
    if res is not None:
        print(json.dumps(res), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
