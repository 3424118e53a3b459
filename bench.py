#!/usr/bin/env python3
"""Benchmark of the corotational linear-tet FEM implicit-Euler step on GB300.

Metric: tet.CG-iter/s -- one tet taking part in one executed CG iteration,
summed over the timed steps and divided by their time. A "step" is one
FixedStep of every solid of the workload (rotations, elastic force,
right-hand side, CG solve to each solid's own tolerance, integration,
energies), with the state resident in HBM.

Default workload: 1024 independent uneven meshes (a x b x c cubes x 5 tets,
a,b,c uniform in [4,30]) stepped together by the batched mixed-precision path
(FP32 products, FP64 dot products and residual refresh), one CUDA graph per
step. The plain FP64 drop-in path on the single 60^3 block (1.08M tets) is
timed beside it as the "plain GPU" comparator.

  python bench.py [--steps K] [--warmup W] [--workload batch1024|block60_mixed|block60_fp64]
  python bench.py --impl reference ...   # the reference's CPU path on the host cores

Prints one JSON line (rank 0). Under torchrun every rank steps its own batch
(seeded by rank): replicas only, no collective on the data path.
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
# algorithmic bytes of one element product (16 B of node ids + 20 element
# scalars R, Dm^-1, V lambda, V mu) and per node of the direction read once
# Algorithmic bytes of one element-product launch: per tet the ids (4 x
# int32) and R (9), Dm^-1 (9), V lambda, V mu in the element type (16 + 20
# s_e); per node d read and q written (6 s_v). One whole CG iteration touches
# the node vectors 11 times (33 s_v per node, ITER_NODE).
ALG_ELEM = {"mixed": 16 + 20 * 4, "fp64": 16 + 20 * 8}
ALG_NODE = {"mixed": 6 * 4, "fp64": 6 * 8}
ITER_NODE = {"mixed": 33 * 4, "fp64": 33 * 8}


# ---------------------------------------------------------------- workloads
def workload(name: str, rank: int = 0):
    from risdsdgcfem_thesis_gb300 import scenes
    if name == "batch1024":
        return scenes.batch_scenes(1024, seed=rank), "mixed"
    if name == "batch128":
        return scenes.batch_scenes(128, seed=rank), "mixed"
    if name == "block60_mixed":
        return [scenes.large_block(n=60, seed=rank)], "mixed"
    if name == "block60_fp64":
        return [scenes.large_block(n=60, seed=rank)], "fp64"
    raise SystemExit(f"unknown workload {name}")


def describe(name, scs, precision):
    T = sum(s.num_tets for s in scs)
    N = sum(s.num_nodes for s in scs)
    if name.startswith("batch"):
        return (f"{len(scs)} independent meshes, a x b x c cubes x 5 tets with a,b,c ~ U{{4..30}} (h=0.01 m, jitter "
                f"0.1h), per-mesh E log-U[1e4,1e6] nu U[0.2,0.45], one random face fixed, gravity -9.81 z, dt=1/60, "
                f"CG rel 1e-6 abs 0 max 500 per mesh; {T} tets, {N} nodes total; {precision}")
    return (f"{scs[0].name}: {T} tets, {N} nodes, h=0.01 m, jitter 0.1h, per-element E log-U[5e4,5e5] nu "
            f"U[0.25,0.45], bottom fixed, top v0=(1,0,0), dt=1/60, CG rel 1e-6 abs 0 max 500; {precision}")


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


def profiled_traffic(kernel: str, workload_name: str, tets_per_launch: float):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any:
    either a per-launch figure or a per-tet figure (a capture on a smaller
    batch) scaled by the tets a launch processes."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload_name}.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        for key, scale in (("traffic_bytes_per_launch:", 1.0), ("traffic_bytes_per_tet:", tets_per_launch)):
            if line.startswith(key):
                try:
                    return float(line.split(":", 1)[1].split()[0]) * scale
                except ValueError:
                    return None
    return None


def dist_info():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def aggregate(values, ws):
    """(value, "max"|"sum") pairs reduced over the ranks of the process group
    (NCCL under torchrun on GPUs, gloo on CPU)."""
    if ws <= 1:
        return [v for v, _ in values]
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    out = []
    for v, op in values:
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
        out.append(float(t.item()))
    return out


# ---------------------------------------------------------------- CPU legs
class CpuSampler:
    """The reference's CPU path (the oracle restatement, bit-exact with the
    reference's FP64 translation units) on the workload's meshes, one mesh per
    thread over `threads` host threads (the reference steps solids serially,
    one thread each). A sample is one whole FixedStep of every mesh --
    rotations, forces, right-hand side, the CG solve to each mesh's own
    tolerance, integration and energies -- continuing from the previous
    sample's state, as the GPU steps continue."""

    def __init__(self, scs, threads):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        pyoracle.build(reference=False)
        self.scs = scs
        self.threads = max(1, threads)
        self.solids = [pyoracle.Solid(sc, "port") for sc in scs]

    def sample(self):
        from concurrent.futures import ThreadPoolExecutor
        iters = [0] * len(self.solids)

        def run(i):
            iters[i] = self.solids[i].step()["iters"]

        t0 = time.perf_counter()
        with ThreadPoolExecutor(self.threads) as ex:
            list(ex.map(run, range(len(self.solids))))
        wall = time.perf_counter() - t0
        units = float(sum(sc.num_tets * it for sc, it in zip(self.scs, iters)))
        return units, max(wall, 1e-9)


def host_cpu():
    """The host's CPU model and logical core count."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.TimeoutExpired):
        pass
    if not model:
        import platform
        model = platform.processor() or platform.machine()
    return {"model": model, "nproc": os.cpu_count()}


def cpu_configs_leg():
    """The reference's CPU path on one thread (the reference steps one solid
    on one thread), whole FixedSteps: C1 (the 160-tet cantilever, 120 steps),
    C2 (the 60^3 block, its first step) and C5 (the 40^3 compressed cube, its
    first step); tet.CG-iter/s and per-step latency."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from risdsdgcfem_thesis_gb300 import scenes
    pyoracle.build(reference=False)
    out = {"host": host_cpu(), "threads": 1, "kind": "port"}
    for name, sc, steps in (("C1_cantilever", scenes.cantilever_160(), 120),
                            ("C2_block60", scenes.large_block(n=60), 1),
                            ("C5_compressed40", scenes.compressed_cube(40, 120, 0.4), 1)):
        o = pyoracle.Solid(sc, "port")
        ms, units = [], 0.0
        for _ in range(steps):
            t0 = time.perf_counter()
            st = o.step()
            ms.append(1e3 * (time.perf_counter() - t0))
            units += sc.num_tets * st["iters"]
        out[name] = {"tets": sc.num_tets, "steps": steps, "value": units / (1e-3 * sum(ms)), "unit": UNIT,
                     "p50_step_ms": float(np.percentile(ms, 50)), "p99_step_ms": float(np.percentile(ms, 99)),
                     "cg_iterations_per_step": units / sc.num_tets / steps}
    return out


def plain_fp64_c1_latency(steps=120):
    """The plain FP64 drop-in (fem_solid_step, synchronous) on the C1
    cantilever: per-step wall-clock latency. At 160 tets the CG solve is
    one thread-block-cluster kernel; the step's other kernels and the host
    round trip make up the rest."""
    from risdsdgcfem_thesis_gb300 import capi, scenes
    sc = scenes.cantilever_160()
    s = capi.Solid(sc, compute_energy=True)
    s.step(3)
    ms, units = [], 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        st = s.step(1)
        ms.append(1e3 * (time.perf_counter() - t0))
        units += sc.num_tets * st["cg_iterations"]
    s.close()
    return {"workload": f"{sc.name} ({sc.num_tets} tets), fem_solid_step, one step per call", "steps": steps,
            "value": units / (1e-3 * sum(ms)), "unit": UNIT, "p50_step_ms": float(np.percentile(ms, 50)),
            "p99_step_ms": float(np.percentile(ms, 99)), "cg_iterations_per_step": units / sc.num_tets / steps}


def cpu_sample_set(scs, max_tets):
    """A bounded subset of the workload's meshes for the CPU timings."""
    out, tot = [], 0
    for sc in scs:
        if tot + sc.num_tets > max_tets and out:
            break
        out.append(sc)
        tot += sc.num_tets
    return out


def run_reference(args):
    ws, rank = dist_info()
    if rank != 0:
        return 0
    scs, precision = workload(args.workload)
    sample = cpu_sample_set(scs, 1_500_000)
    threads = (os.cpu_count() or 1) if len(sample) > 1 else 1
    sampler = CpuSampler(sample, threads)
    total_units, step_s = 0.0, []
    for i in range(args.warmup + args.steps):
        u, t = sampler.sample()
        if i >= args.warmup:
            total_units += u
            step_s.append(t)
    total_s = sum(step_s)
    value = total_units / total_s
    cores = sampler.threads
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "p50_step_ms": float(1e3 * np.percentile(step_s, 50)), "p99_step_ms": float(1e3 * np.percentile(step_s, 99)),
        "config": {"workload": describe(args.workload, scs, "reference CPU path, FP64"), "host": host_cpu()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"each step = one whole FixedStep (rotations, forces, CG to each mesh's own "
                                   f"tolerance, integration, energies) of {len(sample)} of the workload's meshes "
                                   f"({sum(s.num_tets for s in sample)} tets), one mesh per thread on {cores} "
                                   "threads; oracle restatement, bit-exact with the reference's FP64 translation "
                                   "units"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- GPU legs
def time_batch(batch, steps, stream_ptr):
    """Device time of `steps` steps, per step, plus per-mesh CG iterations."""
    import torch
    from risdsdgcfem_thesis_gb300 import capi
    lib = batch.lib
    M = len(batch.scenes)
    before = [batch.stats(i)["total_cg_iterations"] for i in range(M)]
    stream = torch.cuda.ExternalStream(stream_ptr)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    torch.cuda.synchronize()
    evs[0].record(stream)
    for k in range(steps):
        capi.check(lib.fem_batch_step_async(batch.h, 1))
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    capi.check(lib.fem_batch_synchronize(batch.h))
    step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(steps)]
    iters = [batch.stats(i)["total_cg_iterations"] - before[i] for i in range(M)]
    return step_ms, iters


def plain_fp64_comparator(steps=3, ls_solver=0, material=0, assembled=False):
    """The FP64 drop-in path (fem_solid) on the 60^3 block, device time, with
    CG (ls_solver 0) or MINRES (1), material C_WRP (0) or C_LCM (1), with the
    matrix-free element product (the drop-in's default) or the assembled
    stiffness (fem_solid_set_assembled)."""
    import dataclasses
    import torch
    from risdsdgcfem_thesis_gb300 import capi, scenes
    sc = dataclasses.replace(scenes.large_block(n=60), ls_solver=ls_solver, material=material)
    s = capi.Solid(sc, compute_energy=True)
    s.set_assembled(assembled)
    s.step(1)
    lib = capi.load()
    st = capi.FemStepStats()
    capi.check(lib.fem_solid_synchronize(s.h, C.byref(st)))
    it0 = st.total_cg_iterations
    stream = torch.cuda.ExternalStream(s.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    capi.check(lib.fem_solid_step_async(s.h, steps))
    e1.record(stream)
    torch.cuda.synchronize()
    capi.check(lib.fem_solid_synchronize(s.h, C.byref(st)))
    ms = e0.elapsed_time(e1)
    units = float(sc.num_tets) * (st.total_cg_iterations - it0)
    s.close()
    return {"value": units / (ms * 1e-3), "unit": UNIT, "steps": steps,
            "workload": f"{sc.name} ({sc.num_tets} tets), plain FP64 drop-in path (fem_solid_step), "
                        f"{'MINRES' if ls_solver else 'CG'}, {'C_LCM' if material else 'C_WRP'}, "
                        f"{'assembled stiffness' if assembled else 'matrix-free element product'}",
            "ms_per_step": ms / steps, "iterations_per_step": (st.total_cg_iterations - it0) / steps}


def fie_leg(n=40, steps=2, cpu_n=16, assembled=False):
    """The fully-implicit Euler integrator (Newton on Delta x, 3 Newton
    iterations per step, Step_FullyImplicitEuler_dx) on the FP64 solid: the
    n^3 block, wall clock per step (the Newton loop reads |b_k| and |y_k| on
    the host), beside the oracle restatement's single-thread rate on the
    cpu_n^3 block (one step)."""
    import dataclasses
    import torch
    from risdsdgcfem_thesis_gb300 import capi, scenes
    sc = dataclasses.replace(scenes.large_block(n=n), integrator=capi.FEM_INTEGRATOR_FIE_DX)
    s = capi.Solid(sc, compute_energy=True)
    s.set_assembled(assembled)
    s.step(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = [s.step(1) for _ in range(steps)]
    wall = time.perf_counter() - t0
    s.close()
    cg = sum(x["cg_iterations"] for x in st)
    out = {"value": sc.num_tets * cg / wall, "unit": UNIT, "steps": steps, "ms_per_step": 1e3 * wall / steps,
           "workload": f"{sc.name} ({sc.num_tets} tets), FP64 solid, integrator FIE_DX, nr_max_iter 3"
                       + (", assembled stiffness" if assembled else ""),
           "newton_iterations_per_step": [x["nr_iterations"] for x in st],
           "cg_iterations_per_step": [x["cg_iterations"] for x in st]}
    if cpu_n:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        pyoracle.build()
        small = dataclasses.replace(scenes.large_block(n=cpu_n), integrator=1)
        o = pyoracle.Solid(small, "port")
        t0 = time.perf_counter()
        so = o.step()
        cs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": small.num_tets * so["iters"] / cs, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"one FIE step of {small.name} ({small.num_tets} tets, {so['nr_iters']} "
                                         f"Newton iterations, {so['iters']} CG iterations, {cs:.1f} s) on one "
                                         "thread; oracle restatement, bit-exact with the reference's "
                                         "translation units under the restated Leaf driver"}
    return out


def rotation_leg(n=60, reps=5):
    """BeginEvaluation (F, det F, rotation) on the FP64 solid, MSVD against
    DAPD, on the n^3 block crushed to 15 % of its height with lateral noise:
    DAPD takes the Newton polar rotation above det F = 0.1 and the
    time-of-collapse analysis at or below it. Kernel time from CUDA events
    around each launch on the solid's stream."""
    import dataclasses
    from risdsdgcfem_thesis_gb300 import capi, scenes
    sc = scenes.large_block(n=n)
    rng = np.random.default_rng(5)
    x1 = sc.rest.copy()
    x1[:, 2] *= 0.15
    x1 += 0.15 * sc.h * rng.standard_normal(x1.shape)
    out = {"workload": f"{sc.name} ({sc.num_tets} tets) crushed to 15 % of its height, lateral noise 0.15 h"}
    for name, rot, kname in (("msvd", capi.FEM_ROTATION_MSVD, "begin_eval_msvd_fp64"),
                             ("dapd", capi.FEM_ROTATION_DAPD, "begin_eval_dapd_fp64")):
        s = capi.Solid(dataclasses.replace(sc, rotation=rot), compute_energy=False)
        s.begin_eval(x1)  # warm-up (and, for DAPD, the directions of collapse from the rest state)
        capi.profile_enable(True)
        for _ in range(reps):
            s.begin_eval(x1)
        capi.profile_enable(False)
        ms, k = capi.profile_read(kname)
        _, detF = s.rotations()
        s.close()
        us = 1e3 * ms / max(k, 1)
        out[name] = {"us_per_launch": us, "tets_per_s": sc.num_tets / (us * 1e-6), "launches": k}
        out["degenerate_fraction"] = float(np.mean(detF <= float(np.float32(0.1))))
    out["dapd_over_msvd_time"] = out["dapd"]["us_per_launch"] / out["msvd"]["us_per_launch"]
    return out


def batch_variants_leg(meshes=128, steps=3, seed=7, names=None, use_graph=True):
    """The reference's alternatives on the batched mixed path, one batch of
    `meshes` meshes of the batched workload's generator per variant (every
    mesh with the variant): the step (QIE, CG, C_WRP, MSVD), MINRES, C_LCM,
    DAPD, FIE (Newton on Delta x, nr_max_iter 3) and the multi-solid Newton
    lock-step (fem_batch_multi_step, 3 NR iterations). Device time per step
    (CUDA events; the lock-step's phases read the loop flags on the host, so
    it is timed by the wall clock), after one warm-up step."""
    import dataclasses
    import torch
    from risdsdgcfem_thesis_gb300 import capi, scenes
    base = scenes.batch_scenes(meshes, seed=seed)
    variants = (("step", {}), ("minres", {"ls_solver": capi.FEM_LS_MINRES}),
                ("c_lcm", {"material": capi.FEM_MATERIAL_C_LCM}), ("dapd", {"rotation": capi.FEM_ROTATION_DAPD}),
                ("fie", {"integrator": capi.FEM_INTEGRATOR_FIE_DX, "nr_max_iter": 3}),
                ("lock_step", {"nr_max_iter": 3}))
    if names:
        variants = tuple(v for v in variants if v[0] in names)
    T = sum(sc.num_tets for sc in base)
    out = {"workload": f"{meshes} meshes of the batched workload's generator (seed {seed}), {T} tets, mixed",
           "steps": steps}
    for name, kw in variants:
        scs = [dataclasses.replace(sc, **kw) for sc in base]
        bt = capi.Batch(scs, precision=capi.FEM_PRECISION_MIXED, compute_energy=False, use_graph=use_graph)
        if name == "lock_step":
            dt = scs[0].dt
            bt.multi_step(dt, 1)
            torch.cuda.synchronize()
            it0 = [bt.stats(i)["total_cg_iterations"] for i in range(len(scs))]
            t0 = time.perf_counter()
            bt.multi_step(dt, steps)
            ms = [1e3 * (time.perf_counter() - t0) / steps] * steps
            tet_iters = float(sum(sc.num_tets * (bt.stats(i)["total_cg_iterations"] - it0[i])
                                  for i, sc in enumerate(scs)))
        else:
            bt.step(1)
            step_ms, iters = time_batch(bt, steps, bt.stream())
            ms = step_ms
            tet_iters = float(sum(sc.num_tets * it for sc, it in zip(scs, iters)))
        tot = sum(ms)
        out[name] = {"ms_per_step": tot / steps, "tet_cg_iter_per_s": tet_iters / (tot * 1e-3),
                     "status": max(bt.stats(i)["status"] for i in range(len(scs)))}
        if name in ("fie", "lock_step"):
            out[name]["nr_iterations_mean"] = float(np.mean([bt.stats(i)["nr_iterations"] for i in range(len(scs))]))
        bt.close()
        torch.cuda.synchronize()
    return out


def run_ours(args):
    import torch
    from risdsdgcfem_thesis_gb300 import capi
    ws, rank = dist_info()
    if ws > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        import torch.distributed as dist
        dist.init_process_group("nccl")
    capi.load()
    scs, precision = workload(args.workload, rank)
    prec = capi.FEM_PRECISION_MIXED if precision == "mixed" else capi.FEM_PRECISION_FP64
    tuned = None
    tile_elems, reorder, chunk_nodes = 256, True, 1024
    if not args.no_tune:
        from risdsdgcfem_thesis_gb300 import autotune
        t0 = time.perf_counter()
        tuned = autotune.tune(scs, prec, use_cache=False)
        tuned["tune_s"] = round(time.perf_counter() - t0, 1)
        tile_elems, reorder, chunk_nodes = tuned["tile_elems"], bool(tuned["reorder"]), tuned["chunk_nodes"]
    t0 = time.perf_counter()
    batch = capi.Batch(scs, precision=prec, tile_elems=tile_elems, reorder=reorder, chunk_nodes=chunk_nodes,
                       compute_energy=True, use_graph=not args.no_graph)
    setup_s = time.perf_counter() - t0
    info = batch.info()
    stream_ptr = batch.stream()
    batch.step(args.warmup)

    # ---- device-resident timed region ----
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    batch.reset_launch_count()
    if ws > 1:
        torch.distributed.barrier()
    step_ms, iters = time_batch(batch, args.steps, stream_ptr)
    clk = clocks.stop()
    launches = batch.kernel_launches(args.steps) if not args.no_graph else None
    units = float(sum(sc.num_tets * it for sc, it in zip(scs, iters)))
    elapsed_ms, units = aggregate([(sum(step_ms), "max"), (units, "sum")], ws)
    value = units / (elapsed_ms * 1e-3)

    # ---- dominant kernel: tile SpMV, CUDA events around each launch on its
    # stream, over one step run launch by launch (same kernels, host loop) ----
    kname = "tile_spmv_mixed" if precision == "mixed" else "tile_spmv_fp64"
    capi.check(batch.lib.fem_batch_use_graph(batch.h, 0))
    before = [batch.stats(i)["total_cg_iterations"] for i in range(len(scs))]
    capi.profile_enable(True)
    batch.step(1)
    capi.profile_enable(False)
    prof_iters = [batch.stats(i)["total_cg_iterations"] - before[i] for i in range(len(scs))]
    capi.check(batch.lib.fem_batch_use_graph(batch.h, 0 if args.no_graph else 1))
    k_ms, k_n = capi.profile_read(kname)
    alg = sum(it * (ALG_ELEM[precision] * sc.num_tets + ALG_NODE[precision] * sc.num_nodes)
              for sc, it in zip(scs, prof_iters))
    avg_launch_s = (k_ms * 1e-3) / max(k_n, 1)
    alg_per_launch = alg / max(k_n, 1)
    tets_per_launch = sum(it * sc.num_tets for sc, it in zip(scs, prof_iters)) / max(k_n, 1)
    # the whole CG iteration against the same peak: 11 vector touches per node
    iter_bytes_per_tet_iter = sum(ALG_ELEM[precision] * sc.num_tets + ITER_NODE[precision] * sc.num_nodes
                                  for sc in scs) / sum(sc.num_tets for sc in scs)
    achieved = alg_per_launch / avg_launch_s / 1e9 if avg_launch_s > 0 else 0.0
    peak, peak_kind = measured_peaks()

    # ---- end to end: host (pinned) buffers through the C ABI every step ----
    n3 = 3 * info["nodes"]
    hx = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    hv = torch.empty(n3, dtype=torch.float64, pin_memory=True)
    px = C.cast(hx.data_ptr(), C.POINTER(C.c_double))
    pv = C.cast(hv.data_ptr(), C.POINTER(C.c_double))
    capi.check(batch.lib.fem_batch_get_state_all(batch.h, px, pv))
    e2e_steps = max(1, min(args.steps, 5))
    capi.check(batch.lib.fem_batch_synchronize(batch.h))
    before = [batch.stats(i)["total_cg_iterations"] for i in range(len(scs))]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        capi.check(batch.lib.fem_batch_step_host(batch.h, px, pv, 1, px, pv))
    e2e_s = time.perf_counter() - t0
    e2e_iters = [batch.stats(i)["total_cg_iterations"] - before[i] for i in range(len(scs))]
    e2e_units = float(sum(sc.num_tets * it for sc, it in zip(scs, e2e_iters)))
    e2e_s, e2e_units = aggregate([(e2e_s, "max"), (e2e_units, "sum")], ws)
    batch.close()

    plain = plain_asm = None
    plain_c1 = None
    cpu_configs = None
    accuracy = None
    fie = None
    rotations = None
    minres = None
    lcm = None
    variants = None
    cpu = None
    served = None
    compression = None
    if rank == 0 and ws == 1:
        if not args.no_accuracy:
            from risdsdgcfem_thesis_gb300 import scenes as _sc
            acc_steps = args.accuracy_steps or (args.warmup + args.steps)
            accuracy = {"C3_batched": accuracy_leg(scs, acc_steps, tile_elems, reorder, chunk_nodes),
                        "C1_cantilever": single_mesh_error(_sc.cantilever_160(), 120),
                        "C2_block60": single_mesh_error(_sc.large_block(n=60), 60),
                        "C5": "see compression (the 40^3 compressed cube, 120 steps)"}
        if not args.no_compression:
            compression = compression_report()
        if not args.no_served:
            served = served_leg(args.served_rate, args.served_seconds, pool_count=args.served_pool)
        if not args.no_plain:
            plain = plain_fp64_comparator(3)
            plain_asm = plain_fp64_comparator(3, assembled=True)
            plain_c1 = plain_fp64_c1_latency()
        if not args.no_fie:
            fie = fie_leg()
            rotations = rotation_leg()
            minres = plain_fp64_comparator(3, ls_solver=1)
            lcm = plain_fp64_comparator(3, material=1)
            variants = batch_variants_leg()
        if not args.no_cpu:
            sample = cpu_sample_set(scs, 1_500_000)
            threads = (os.cpu_count() or 1) if len(sample) > 1 else 1
            sampler = CpuSampler(sample, threads)
            u, s, reps, step_s = 0.0, 0.0, 0, []
            while s < 12.0 and reps < 20:  # about 12 s of whole steps on the host cores
                du, ds = sampler.sample()
                u, s, reps = u + du, s + ds, reps + 1
                step_s.append(ds)
            cpu = {"value": u / s, "unit": UNIT, "cores": sampler.threads, "kind": "port",
                   "p50_step_ms": float(1e3 * np.percentile(step_s, 50)),
                   "p99_step_ms": float(1e3 * np.percentile(step_s, 99)), "host": host_cpu(),
                   "sample": f"{reps} whole FixedSteps (rotations, forces, CG to each mesh's own tolerance, "
                             f"integration, energies) of {len(sample)} of the workload's meshes "
                             f"({sum(x.num_tets for x in sample)} tets), one mesh per thread on {sampler.threads} "
                             f"threads ({s:.1f} s in total); oracle restatement, bit-exact with the reference's "
                             "FP64 translation units"}
            cpu_configs = cpu_configs_leg()

    if rank == 0:
        elem_bytes = info["tets"] * (88 if precision == "mixed" else 176)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64" if precision == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": describe(args.workload, scs, precision), "meshes": len(scs),
                       "tets": info["tets"], "nodes": info["nodes"], "tiles": info["tiles"],
                       "device_bytes": info["device_bytes"],
                       "parallelism": "replicas only" if ws > 1 else "1 GPU",
                       "l2": f"inputs larger than L2: {elem_bytes / 1e6:.0f} MB of element data streamed per CG "
                             f"iteration vs {L2_BYTES / 1e6:.0f} MB L2",
                       "cg_iterations_timed_max_mesh": int(max(iters)), "setup_s": round(setup_s, 2),
                       "tile_elems": tile_elems, "reorder": reorder, "chunk_nodes": chunk_nodes,
                       "autotune": tuned,
                       "graph": not args.no_graph},
            "p50_step_ms": float(np.percentile(step_ms, 50)), "p99_step_ms": float(np.percentile(step_ms, 99)),
            "clocks": clk,
            "e2e": {"value": e2e_units / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * n3 * 8,
                    "d2h_bytes_per_step": 2 * n3 * 8, "steps": e2e_steps,
                    "note": "fem_batch_step_host: all states up, one step, all states down, wall clock"},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": profiled_traffic(kname, args.workload, tets_per_launch),
                         "peak_kind": peak_kind, "alg_bytes_per_launch": alg_per_launch,
                         "avg_launch_us": avg_launch_s * 1e6, "launches": int(k_n)},
            "roofline_iteration": {"bound": "hbm", "bytes_per_tet_iter": iter_bytes_per_tet_iter,
                                   "achieved": value * iter_bytes_per_tet_iter / 1e9, "peak": peak,
                                   "unit": "GB/s", "frac": value * iter_bytes_per_tet_iter / 1e9 / peak,
                                   "note": "whole-job tet.CG-iter/s x algorithmic bytes of one CG "
                                           "iteration (16 + 20 s_e per tet + 33 s_v per node)"},
            "accuracy": accuracy,
            "plain_fp64_gpu": plain,
            "plain_fp64_gpu_assembled": plain_asm,
            "plain_fp64_gpu_c1": plain_c1,
            "cpu_single_thread": cpu_configs,
            "fie_fp64_gpu": fie,
            "rotations_fp64_gpu": rotations,
            "minres_fp64_gpu": minres,
            "lcm_fp64_gpu": lcm,
            "batch_variants_mixed": variants,
            "cpu_baseline": cpu,
            "served": served,
            "compression": compression,
        }
        if plain:
            line["speedup_vs_plain_fp64_gpu"] = value / plain["value"]
        if plain_asm:
            line["speedup_vs_plain_fp64_gpu_assembled"] = value / plain_asm["value"]
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------- accuracy
def _vstats(a):
    a = np.asarray(a, dtype=np.float64)
    if a.size == 0:
        return None
    return {"max": float(a.max()), "p99": float(np.percentile(a, 99)), "mean": float(a.mean())}


def accuracy_leg(scs, steps, tile_elems, reorder, chunk_nodes):
    """Error of the timed workload: the same meshes stepped `steps` times
    from their initial state by the mixed path (the timed configuration) and
    by the FP64 batch path (pinned to the FP64 oracle per mesh by the GPU
    tests). Per mesh: x rel-L2 and ||v - v64|| / max over the run of ||v64||
    (a body that comes to rest has v ~ 0, where a plain relative norm divides
    by ~0). Also every step that ended at the CG iteration cap, in either
    path, with its relative residual."""
    from risdsdgcfem_thesis_gb300 import capi
    M = len(scs)
    t0 = time.perf_counter()
    mix = capi.Batch(scs, precision=capi.FEM_PRECISION_MIXED, tile_elems=tile_elems, reorder=reorder,
                     chunk_nodes=chunk_nodes, compute_energy=False)
    f64 = capi.Batch(scs, precision=capi.FEM_PRECISION_FP64, tile_elems=tile_elems, reorder=reorder,
                     compute_energy=False)
    vpeak = np.zeros(M)
    it_m = np.zeros((steps, M), np.int64)
    it_f = np.zeros((steps, M), np.int64)
    res_m = np.zeros((steps, M))
    res_f = np.zeros((steps, M))
    for k in range(steps):
        mix.step(1)
        f64.step(1)
        for i in range(M):
            a, b = mix.stats(i), f64.stats(i)
            it_m[k, i], res_m[k, i] = a["cg_iterations"], a["rel_residual"]
            it_f[k, i], res_f[k, i] = b["cg_iterations"], b["rel_residual"]
            vpeak[i] = max(vpeak[i], float(np.linalg.norm(f64.state(i)[1])))
    ex, ev = np.zeros(M), np.zeros(M)
    for i in range(M):
        xm, vm = mix.state(i)
        xf, vf = f64.state(i)
        ex[i] = np.linalg.norm(xm - xf) / np.linalg.norm(xf)
        ev[i] = np.linalg.norm(vm - vf) / vpeak[i] if vpeak[i] > 0 else 0.0
    mix.close()
    f64.close()
    caps = np.array([sc.max_iter for sc in scs])
    capped_m = (it_m >= caps[None, :])
    capped_f = (it_f >= caps[None, :])
    capped_any = capped_m.any(axis=0) | capped_f.any(axis=0)
    conv = ~capped_any
    worst = np.argsort(-np.maximum(ex, ev))[:5]
    return {
        "workload": f"the timed workload's {M} meshes, {steps} steps from their initial state, mixed path against "
                    "the FP64 batch path",
        "steps": steps, "tolerance": 1e-5,
        "x_rel_err": _vstats(ex), "v_err_peak_normalised": _vstats(ev),
        "meshes_within_1e-5": int(np.sum((ex <= 1e-5) & (ev <= 1e-5))),
        "converged_every_step": {"meshes": int(conv.sum()), "x_rel_err": _vstats(ex[conv]),
                                 "v_err_peak_normalised": _vstats(ev[conv])},
        "at_cg_cap": {"meshes": int(capped_any.sum()), "x_rel_err": _vstats(ex[capped_any]),
                      "v_err_peak_normalised": _vstats(ev[capped_any]),
                      "steps_at_cap_mixed": int(capped_m.sum()), "steps_at_cap_fp64": int(capped_f.sum()),
                      "rel_residual_at_cap_mixed": _vstats(res_m[capped_m]),
                      "rel_residual_at_cap_fp64": _vstats(res_f[capped_f])},
        "cg_iterations_mean": {"mixed": float(it_m.mean()), "fp64": float(it_f.mean())},
        "worst_meshes": [{"mesh": int(i), "name": scs[i].name, "tets": scs[i].num_tets, "young": scs[i].young,
                          "x_rel_err": float(ex[i]), "v_err": float(ev[i]),
                          "steps_at_cap_mixed": int(capped_m[:, i].sum()),
                          "steps_at_cap_fp64": int(capped_f[:, i].sum())} for i in worst],
        "wall_s": round(time.perf_counter() - t0, 1),
    }


def single_mesh_error(sc, steps):
    """One mesh stepped by the mixed batch path and by the plain FP64 drop-in
    (fem_solid, parity-tested against the FP64 oracle): x rel-L2 and the
    peak-normalised v error after `steps` steps, CG iterations per step."""
    from risdsdgcfem_thesis_gb300 import capi
    mix = capi.Batch([sc], precision=capi.FEM_PRECISION_MIXED, compute_energy=False)
    f64 = capi.Solid(sc, compute_energy=False)
    vpeak, it_m, it_f = 0.0, [], []
    for _ in range(steps):
        mix.step(1)
        it_f.append(f64.step(1)["cg_iterations"])
        it_m.append(mix.stats(0)["cg_iterations"])
        vpeak = max(vpeak, float(np.linalg.norm(f64.state()[1])))
    xm, vm = mix.state(0)
    xf, vf = f64.state()
    mix.close()
    f64.close()
    return {"mesh": f"{sc.name} ({sc.num_tets} tets)", "steps": steps,
            "x_rel_err": float(np.linalg.norm(xm - xf) / np.linalg.norm(xf)),
            "v_err_peak_normalised": float(np.linalg.norm(vm - vf) / vpeak) if vpeak > 0 else 0.0,
            "cg_iterations_mean": {"mixed": float(np.mean(it_m)), "fp64": float(np.mean(it_f))},
            "steps_at_cap": {"mixed": int(sum(i >= sc.max_iter for i in it_m)),
                             "fp64": int(sum(i >= sc.max_iter for i in it_f))}}


# ---------------------------------------------------------------- compression
def compression_report(n=40, steps=120, ratio=0.4):
    """The large-deformation case: an n^3 x 5-tet cube (E 2e5, nu 0.45)
    compressed by its top face to `ratio` of its height over `steps` steps.
    The mixed path against the plain FP64 path (itself parity-tested against
    the FP64 oracle), step by step: share of rotations computed in FP64 and
    of inverted elements, CG iterations, and the final error -- with the
    default double-precision rotations (double-float, FP64 for degenerate
    elements), with FP32 rotations re-solved so where det F <= 1e-3 or the
    rotation is rounding-sensitive, and with the det F rule alone."""
    from risdsdgcfem_thesis_gb300 import capi, scenes
    sc = scenes.compressed_cube(n, steps, ratio)
    T = float(sc.num_tets)
    f64 = capi.Batch([sc], precision=capi.FEM_PRECISION_FP64, compute_energy=False)
    it64, xs64, vscale, t64 = [], None, 0.0, 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        f64.step(1)
        t64 += time.perf_counter() - t0
        it64.append(f64.stats(0)["cg_iterations"])
        vscale = max(vscale, float(np.linalg.norm(f64.state(0)[1])))
    x64, v64 = f64.state(0)
    f64.close()
    # the FP64 path's own sensitivity: the same run from an initial velocity
    # perturbed by 1e-15 (relative to the mesh size)
    pert = capi.Batch([sc], precision=capi.FEM_PRECISION_FP64, compute_energy=False)
    v0 = 1e-15 * float(np.abs(sc.rest).max()) * np.random.default_rng(1).standard_normal(sc.rest.shape)
    pert.set_state(0, v=v0)
    pert.step(steps)
    xp, vp = pert.state(0)
    pert.close()
    noise = {"x_rel": float(np.linalg.norm(xp - x64) / np.linalg.norm(x64)),
             "v": float(np.linalg.norm(vp - v64) / vscale) if vscale > 0 else None}

    # the FP64 path's response to FP32-sized changes of its input, the size
    # of what the mixed path changes: initial velocities perturbed by 6e-8 of
    # the mesh size (about one FP32 rounding of a position), and the rest
    # positions rounded to FP32 (so Dm^-1, volumes and stiffness move by FP32
    # roundings, as the mixed path's FP32 element data do)
    def fp64_variant(scene, v0=None):
        run = capi.Batch([scene], precision=capi.FEM_PRECISION_FP64, compute_energy=False)
        if v0 is not None:
            run.set_state(0, v=v0)
        run.step(steps)
        xq, vq = run.state(0)
        run.close()
        return {"x_rel": float(np.linalg.norm(xq - x64) / np.linalg.norm(x64)),
                "v": float(np.linalg.norm(vq - v64) / vscale) if vscale > 0 else None}

    import dataclasses
    v32 = 6e-8 * float(np.abs(sc.rest).max()) * np.random.default_rng(2).standard_normal(sc.rest.shape)
    rest32 = sc.rest.astype(np.float32).astype(np.float64)
    sc32 = dataclasses.replace(sc, rest=rest32, knc_targets=sc.knc_targets.astype(np.float32).astype(np.float64))
    fp32_sized = {"initial_velocity_6e-8": fp64_variant(sc, v32),
                  "rest_positions_rounded_to_fp32": fp64_variant(sc32)}

    def mixed(rot32, check):
        mix = capi.Batch([sc], precision=capi.FEM_PRECISION_MIXED, compute_energy=False, rotation_fp32=rot32,
                         rotation_check=check)
        res, inv, itm, tm = [], [], [], 0.0
        cause = {"det_F": [], "isotropic": [], "tie": [], "check": []}
        for _ in range(steps):
            t0 = time.perf_counter()
            mix.step(1)
            tm += time.perf_counter() - t0
            b = mix.stats(0)
            res.append(b["fp64_resolved"] / T)
            inv.append(b["inverted_elements"] / T)
            itm.append(b["cg_iterations"])
            for k in cause:
                cause[k].append(b["resolved_" + k] / T)
        xm, vm = mix.state(0)
        mix.close()
        return {"fp64_resolved_fraction_max": max(res), "fp64_resolved_fraction_mean": float(np.mean(res)),
                "resolved_by_cause_mean": {k: float(np.mean(v)) for k, v in cause.items()},
                "resolved_by_cause_max": {k: float(np.max(v)) for k, v in cause.items()},
                "inverted_fraction_max": max(inv),
                "x_rel_err_vs_fp64_path": float(np.linalg.norm(xm - x64) / np.linalg.norm(x64)),
                "v_err_vs_fp64_path": float(np.linalg.norm(vm - v64) / vscale) if vscale > 0 else None,
                "cg_iterations_mean": float(np.mean(itm)), "wall_s": tm}

    return {"case": f"{n}^3 x 5 tets ({int(T)}), top face to {ratio:.0%} height over {steps} steps, "
                    f"E 2e5, nu 0.45, dt 1/60, CG rel 1e-6",
            "mixed_default_double_precision_rotations": mixed(0, 1e-3),
            "mixed_fp32_rotations_checked": mixed(1, 1e-3),
            "mixed_fp32_rotations_det_F_rule_only": mixed(1, 0.0),
            "fp64_path_noise_floor": noise,
            "fp64_path_fp32_sized_input_change": fp32_sized,
            "cg_iterations_fp64_mean": float(np.mean(it64)), "wall_s_fp64": t64,
            "note": "v error normalised by the run's peak |v|; the FP64 path matches the FP64 oracle "
                    "(tests/test_gpu_fp64.py, tests/test_gpu_batch.py). fp64_resolved counts rotations "
                    "re-solved at double precision (every element under the default double-float "
                    "rotations); resolved_by_cause splits the FP64 MSVD re-solves (det_F: det F <= 1e-3, "
                    "isotropic: double-float unsafe) and, with FP32 rotations, why the FP32 one was "
                    "rejected (tie, check)"}


# ---------------------------------------------------------------- served leg
def served_leg(rate, seconds, pool_count=4096, seed=0, budget=120 << 30, deadline_ms=1000.0 / 60.0):
    """Step requests over a resident pool through the server (fem_server_*):
    `pool_count` scenes of log-uniform 200..200k tets admitted under a device
    budget, Poisson arrivals at `rate` requests/s for `seconds` on scenes
    drawn uniformly, continuous batching; then the same at 60 % and at 2 % of
    the completion rate the first run sustained (the light-load point, run
    twice as long for enough samples at its p99, shows the latency floor: one
    request's CG iterations on a nearly idle GPU).
    Latency is submit -> completion seen by the host loop."""
    from risdsdgcfem_thesis_gb300 import capi, scenes
    t0 = time.perf_counter()
    pool = scenes.served_pool(pool_count, seed)
    srv = capi.Server(precision=capi.FEM_PRECISION_MIXED, hbm_budget_bytes=budget)
    for sc in pool:
        srv.add(sc)
    admitted = srv.admit()
    setup_s = time.perf_counter() - t0
    st = srv.status()
    resident = np.array(srv.resident(), dtype=np.int64)
    tets = np.array([sc.num_tets for sc in pool], dtype=np.float64)
    # warm-up: every resident scene steps once
    for i in resident:
        srv.submit(int(i))
    srv.drain()

    def run(r, secs, rs):
        n = int(rs.poisson(r * secs))
        times = np.sort(rs.uniform(0.0, secs, n))
        which = resident[rs.integers(0, len(resident), n)]
        done, k = [], 0
        t_start = time.perf_counter()
        while k < n:
            now = time.perf_counter() - t_start
            while k < n and times[k] <= now:
                srv.submit(int(which[k]), k)
                k += 1
            done += srv.pump()
        done += srv.drain()
        wall = time.perf_counter() - t_start
        lat = np.array([c["latency_us"] for c in done]) / 1e3
        units = float(sum(tets[c["scene"]] * c["cg_iterations"] for c in done))
        return {"offered_per_s": r, "seconds": secs, "requests": n, "completed": len(done), "wall_s": wall,
                "completed_per_s": len(done) / wall, "tet_cg_iter_per_s": units / wall,
                "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
                "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
                "within_deadline": float(np.mean(lat <= deadline_ms)) if len(lat) else None,
                "mean_cg_iterations": float(np.mean([c["cg_iterations"] for c in done])) if done else None,
                "errors": int(sum(1 for c in done if c["status"] != 0))}

    rs = np.random.default_rng(seed + 1)
    offered = run(rate, seconds, rs)
    sustain_rate = 0.6 * offered["completed_per_s"]
    sustained = run(sustain_rate, seconds, rs)
    light = run(0.02 * offered["completed_per_s"], 2 * seconds, rs)
    st2 = srv.status()
    srv.close()
    return {"pool": f"{pool_count} scenes, 5*a*b*c blocks of log-uniform 200..200k tets "
                    f"({int(tets.sum())} tets), mixed precision, CG rel 1e-6, max 500",
            "budget_bytes": budget, "admitted": admitted, "device_bytes": st["device_bytes"],
            "shards": st["shards"], "max_busy_shards": st2["max_busy_shards"], "setup_s": round(setup_s, 1),
            "deadline_ms": deadline_ms, "at_offered_rate": offered, "at_60pct_of_capacity": sustained,
            "at_2pct_of_capacity": light}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch1024")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-fie", action="store_true",
                    help="skip the fully-implicit Euler, MSVD/DAPD rotation, MINRES and C_LCM legs")
    ap.add_argument("--no-graph", action="store_true", help="launch kernels one by one (for per-kernel profilers)")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-compression", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the error of the timed workload (mixed against the FP64 path) and per config")
    ap.add_argument("--accuracy-steps", type=int, default=0, help="steps of the accuracy leg (0: warmup + steps)")
    ap.add_argument("--no-tune", action="store_true", help="default tiles (256 tets, Morton order)")
    ap.add_argument("--served-rate", type=float, default=20000.0, help="offered step requests per second")
    ap.add_argument("--served-seconds", type=float, default=3.0)
    ap.add_argument("--served-pool", type=int, default=4096)
    ap.add_argument("--only-variants", action="store_true",
                    help="run only the batched variants leg and print its JSON (for per-kernel profiles)")
    ap.add_argument("--variants", default="step,minres,c_lcm,dapd,fie,lock_step",
                    help="comma-separated variants of the batched variants leg")
    ap.add_argument("--variants-meshes", type=int, default=128)
    ap.add_argument("--only-plain", action="store_true",
                    help="run only the plain FP64 solid legs: the FIE step of the 40^3 block with the assembled "
                         "stiffness, then matrix-free (host-driven solver loop, so per-kernel profilers see its "
                         "kernels), the 60^3 block (CG matrix-free and assembled, MINRES; C_WRP) and the "
                         "cantilever's latency, and print their JSON")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.only_plain:
        print(json.dumps({"fie_fp64_gpu_assembled": fie_leg(cpu_n=0, assembled=True),
                          "fie_fp64_gpu": fie_leg(cpu_n=0),
                          "plain_fp64_gpu": plain_fp64_comparator(args.steps),
                          "plain_fp64_gpu_assembled": plain_fp64_comparator(args.steps, assembled=True),
                          "minres_fp64_gpu": plain_fp64_comparator(args.steps, ls_solver=1),
                          "plain_fp64_gpu_c1": plain_fp64_c1_latency()}))
        return 0
    if args.only_variants:
        print(json.dumps(batch_variants_leg(meshes=args.variants_meshes, steps=args.steps,
                                            names=args.variants.split(","), use_graph=not args.no_graph)))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
