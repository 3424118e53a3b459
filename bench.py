#!/usr/bin/env python3
"""Benchmark of the corotational linear-tet FEM implicit-Euler step.

Metric: tet.CG-iter/s -- one tet taking part in one executed CG iteration,
summed over the timed steps, divided by the device time of those steps.
A "step" is one FixedStep of the workload (rotation, elastic force, right-hand
side, CG solve to tolerance, integration, energies), inputs resident in HBM.

  python bench.py [--steps K] [--warmup W] [--workload block60_fp64]
  python bench.py --impl reference ...   # the reference's CPU path, same metric

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tet·CG-iter/s & p99 step latency: batched/served vs plain GPU, ≤1e-5 rel err"
UNIT = "tet·CG-iter/s"
L2_BYTES = 129 * 1024 * 1024


def workload_scene(name: str):
    from risdsdgcfem_thesis_gb300 import scenes
    if name == "block60_fp64":
        return scenes.large_block(n=60)
    if name == "block20_fp64":
        return scenes.large_block(n=20)
    raise SystemExit(f"unknown workload {name}")


def workload_desc(name, sc):
    return (f"{sc.name}: {sc.num_tets} tets, {sc.num_nodes} nodes, h=0.01 m, jitter 0.1h, per-element E log-U"
            f"[5e4,5e5] nu U[0.25,0.45], bottom fixed, top v0=(1,0,0), dt=1/60, CG rel 1e-6 abs 0, "
            f"max {sc.max_iter}; plain FP64")


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    backend = "nccl"
    dist.init_process_group(backend=backend)
    return dist


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- CPU legs
class CpuSampler:
    """Times the CG iterations of the first FixedStep of a workload on the
    oracle restatement (bit-exact with the reference's FP64 translation units),
    single-threaded like the reference path. One sample = the step with the CG
    capped at `cap` iterations minus the same step capped at 0 iterations, so
    the figure is the CG loop's throughput alone (the per-step fixed work --
    rotations, elastic force, right-hand side -- is left out, which favours
    the CPU)."""

    def __init__(self, sc):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        pyoracle.build(reference=False)
        self.sc = sc
        self.solid = pyoracle.Solid(sc, "port")

    def _timed_step(self, cap):
        self.solid.reset()
        self.solid.set_solver(self.sc.rel_eps, self.sc.abs_eps, cap)
        t0 = time.perf_counter()
        st = self.solid.step()
        return st["iters"], time.perf_counter() - t0

    def sample(self, cap):
        _, t0 = self._timed_step(0)
        it, tc = self._timed_step(cap)
        return float(self.sc.num_tets) * it, max(tc - t0, 1e-9)


def run_reference(args):
    ws, rank = dist_info()
    if rank != 0:
        return 0
    sc = workload_scene(args.workload)
    sampler = CpuSampler(sc)
    cap = 8
    total_units, total_s = 0.0, 0.0
    for i in range(args.warmup + args.steps):
        u, s = sampler.sample(cap if i >= args.warmup else 1)
        if i >= args.warmup:
            total_units += u
            total_s += s
    value = total_units / total_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_desc(args.workload, sc)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"each step = the CG iterations of the first FixedStep of {sc.name} "
                                   f"(step capped at {cap} iterations minus the step capped at 0), one thread "
                                   "(the reference path is serial per mesh); oracle restatement, bit-exact with "
                                   "the reference's FP64 translation units"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU leg
def run_ours(args):
    import torch
    from risdsdgcfem_thesis_gb300 import capi
    ws, rank = dist_info()
    if ws > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist = dist_init(ws)
    capi.load()
    sc = workload_scene(args.workload)
    solid = capi.Solid(sc, compute_energy=True)
    stream = torch.cuda.ExternalStream(solid.stream())
    for _ in range(args.warmup):
        solid.step(1)

    # ---- device-resident timed region ----
    lib = capi.load()
    stats = capi.FemStepStats()
    capi.check(lib.fem_solid_synchronize(solid.h, C.byref(stats)))
    iters_before = stats.total_cg_iterations
    launches_before = capi.kernel_launches()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    capi.profile_enable(True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    evs[0].record(stream)
    for k in range(args.steps):
        capi.check(lib.fem_solid_step_async(solid.h, 1))
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    capi.profile_enable(False)
    clk = clocks.stop()
    capi.check(lib.fem_solid_synchronize(solid.h, C.byref(stats)))
    launches = capi.kernel_launches() - launches_before
    iters = stats.total_cg_iterations - iters_before
    elapsed_ms = sum(step_ms)
    elapsed_ms = reduce_max(dist, elapsed_ms)
    units = reduce_sum(dist, float(sc.num_tets) * iters)
    value = units / (elapsed_ms * 1e-3)

    # dominant kernel roofline (events around each launch on the lib stream)
    spmv_ms, spmv_n = capi.profile_read("elem_spmv_fp64")
    N, T = sc.num_nodes, sc.num_tets
    alg_bytes = T * (16 + 20 * 8) + N * 3 * 8
    avg_s = (spmv_ms / max(spmv_n, 1)) * 1e-3
    achieved = alg_bytes / avg_s / 1e9 if avg_s > 0 else 0.0
    peak, peak_kind = measured_peaks()
    traffic = profiled_traffic("elem_spmv_fp64", args.workload)

    # ---- end-to-end through the C ABI with host (pinned) buffers ----
    n3 = 3 * N
    hx = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    hv = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    capi.check(lib.fem_solid_get_state(solid.h, C.cast(hx.data_ptr(), C.POINTER(C.c_double)),
                                       C.cast(hv.data_ptr(), C.POINTER(C.c_double))))
    e2e_steps = max(1, min(args.steps, 10))
    capi.check(lib.fem_solid_synchronize(solid.h, C.byref(stats)))
    it0 = stats.total_cg_iterations
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        px = C.cast(hx.data_ptr(), C.POINTER(C.c_double))
        pv = C.cast(hv.data_ptr(), C.POINTER(C.c_double))
        capi.check(lib.fem_solid_step_host(solid.h, px, pv, 1, px, pv, C.byref(stats)))
    e2e_s = time.perf_counter() - t0
    e2e_iters = stats.total_cg_iterations - it0
    e2e_s = reduce_max(dist, e2e_s)
    e2e_value = reduce_sum(dist, float(T) * e2e_iters) / e2e_s

    # ---- CPU baseline (rank 0, N=1) ----
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cap = 30
        sampler = CpuSampler(sc)
        u, s = sampler.sample(cap)
        cpu = {"value": u / s, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"the CG iterations of the first FixedStep of {sc.name}: step capped at {cap} "
                         f"iterations minus the step capped at 0 ({s:.1f} s of CG), one thread, oracle "
                         "restatement (bit-exact with the reference's FP64 translation units)"}

    if rank == 0:
        elem_bytes = T * (16 + 20 * 8 + 96)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_desc(args.workload, sc), "precision": "fp64",
                       "parallelism": "replicas only" if ws > 1 else "1 GPU",
                       "l2": f"inputs larger than L2: {elem_bytes / 1e6:.0f} MB of element data per CG "
                             f"iteration vs {L2_BYTES / 1e6:.0f} MB L2",
                       "cg_iterations_timed": int(iters)},
            "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
            "clocks": clk,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * n3 * 8,
                    "d2h_bytes_per_step": 2 * n3 * 8 + 8 * 10, "steps": e2e_steps},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "elem_spmv_fp64", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_kind": peak_kind, "alg_bytes_per_launch": alg_bytes,
                         "avg_launch_us": avg_s * 1e6, "launches": int(spmv_n),
                         "note": "FP64 path: bound by FP64 issue on GB300, not HBM"},
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="block60_fp64")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
