"""Tile-size and element-order autotuner for batches.

A batch cuts each mesh's elements (in Morton order of their centroids, or in
the mesh's own order) into tiles of at most `tile_elems` tets; the tile is
the unit of the element product's shared-memory staging and of its segmented
sum. The node pass walks each mesh's nodes in chunks of `chunk_nodes`, the
unit of its per-mesh reductions. Which sizes and order run fastest depends on
the meshes (their sizes and node sharing) and on the GPU, so `tune`
measures: it builds the batch of a sample of the workload for each candidate,
times launches of a fixed number of CG iterations (the batch's iteration
budget) and returns the fastest options. Results are cached per device and workload signature in a JSON file
(`$FEMGB_CACHE_DIR` or `~/.cache/risdsdgcfem_thesis_gb300/autotune.json`).

The choice changes speed only: every candidate computes the same step up to
the summation order inside tiles (each candidate is parity-tested like the
default)."""
import json
import math
import os
import time
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

from . import capi

# (tile_elems, reorder, chunk_nodes)
DEFAULT_CANDIDATES: Tuple[Tuple[int, int, int], ...] = ((256, 1, 1024), (256, 1, 512), (192, 1, 1024),
                                                         (128, 1, 1024), (256, 0, 1024), (256, 0, 512))


def _cache_path() -> str:
    d = os.environ.get("FEMGB_CACHE_DIR") or os.path.join(os.path.expanduser("~"), ".cache",
                                                          "risdsdgcfem_thesis_gb300")
    return os.path.join(d, "autotune.json")


def signature(scenes: Sequence, precision: int) -> str:
    """Device, precision and a coarse size profile of the workload."""
    dev = capi.device_info()
    T = sum(s.num_tets for s in scenes)
    sizes = sorted(s.num_tets for s in scenes)
    med = sizes[len(sizes) // 2] if sizes else 0
    return (f"sm{dev['cc'][0]}{dev['cc'][1]}x{dev['sm_count']}/p{precision}/"
            f"T2^{int(math.log2(max(T, 1)))}/med2^{int(math.log2(max(med, 1)))}/M{len(scenes)}")


def _time_candidate(scenes, precision, tile_elems, reorder, chunk_nodes, iters, reps) -> float:
    b = capi.Batch(scenes, precision=precision, tile_elems=tile_elems, reorder=bool(reorder), use_graph=True,
                   chunk_nodes=chunk_nodes, compute_energy=False)
    try:
        b.set_slice(iters)
        b.set_active(None)
        b.step(1)  # warm-up (graph upload, caches)
        best = float("inf")
        for _ in range(reps):
            b.set_active(None)  # every mesh starts its step again
            t0 = time.perf_counter()
            b.step(1)
            best = min(best, time.perf_counter() - t0)
        return best
    finally:
        b.close()


def tune(scenes: Sequence, precision: int = capi.FEM_PRECISION_MIXED,
         candidates: Iterable[Tuple[int, ...]] = DEFAULT_CANDIDATES, iters: int = 30, reps: int = 3,
         sample_tets: int = 4_000_000, use_cache: bool = True) -> Dict:
    """Returns {"tile_elems", "reorder", "chunk_nodes", "table", "signature",
    "cached"}. A candidate is (tile_elems, reorder) or (tile_elems, reorder,
    chunk_nodes).

    The timing runs on a prefix of `scenes` holding about `sample_tets` tets
    (the whole workload's tiles behave alike; the prefix keeps tuning to
    seconds)."""
    sample: List = []
    tot = 0
    for s in scenes:
        if sample and tot + s.num_tets > sample_tets:
            break
        sample.append(s)
        tot += s.num_tets
    sig = signature(scenes, precision)
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and sig in cache:
        out = dict(cache[sig])
        out["cached"] = True
        return out
    table = []
    for cand in candidates:
        tile_elems, reorder = cand[0], cand[1]
        chunk_nodes = cand[2] if len(cand) > 2 else 1024
        t = _time_candidate(sample, precision, tile_elems, reorder, chunk_nodes, iters, reps)
        table.append({"tile_elems": tile_elems, "reorder": reorder, "chunk_nodes": chunk_nodes,
                      "ms_per_launch": 1e3 * t, "tet_cg_iter_per_s": tot * iters / t})
    best = min(table, key=lambda r: r["ms_per_launch"])
    out = {"tile_elems": best["tile_elems"], "reorder": best["reorder"], "chunk_nodes": best["chunk_nodes"],
           "table": table, "signature": sig, "sample_tets": tot, "iters": iters}
    if use_cache:
        cache[sig] = out
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path + ".tmp", "w") as f:
                json.dump(cache, f, indent=1)
            os.replace(path + ".tmp", path)
        except OSError:
            pass
    out = dict(out)
    out["cached"] = False
    return out
