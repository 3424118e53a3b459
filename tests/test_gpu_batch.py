"""Tiled, batched step on the GPU (FP64 and mixed) through the C ABI.

Tolerances: FP64 as the single-solid path (rel-L2 <= max(1e-10, 10 x the
oracle's own 1e-15-perturbation noise floor), iterations within
max(1, 2 x spread + 1)); mixed precision rel-L2 <= 1e-5 against the FP64
oracle; a solid alone and inside a batch: bit-identical.
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes
from parity_util import bar_cap, check_bar, oracle_run, perturbed, rel

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _damped_driven():
    rng = np.random.default_rng(5)
    sc = scenes.random_block(rng, dims=(5, 3, 4))
    T = sc.num_tets
    sc.young_per_elem = np.exp(rng.uniform(np.log(5e4), np.log(5e5), T))
    sc.poisson_per_elem = rng.uniform(0.25, 0.45, T)
    sc.damping_ratio = 1.0
    sc.init_vel = rng.standard_normal(sc.rest.shape) * 0.1
    base = sc.knc_targets.copy()
    sc.knc_schedule = lambda k: base + np.array([0.0, 0.0, 0.001 * (k + 1)])
    return sc


def test_fp64_batch_of_one_matches_reference_cantilever(fem_lib):
    g = np.load(os.path.join(GOLDEN, "cantilever_160.npz"))
    sc = scenes.cantilever_160()
    b = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64)
    for k in range(sc.steps):
        b.step(1)
        st = b.stats(0)
        assert abs(st["cg_iterations"] - int(g["iters"][k])) <= 1, (k, st["cg_iterations"], g["iters"][k])
    x, v = b.state(0)
    assert rel(x, g["x"][-1]) <= 1e-10 and rel(v, g["v"][-1]) <= 1e-10, (rel(x, g["x"][-1]), rel(v, g["v"][-1]))
    assert abs(st["elastic_energy"] - g["elastic_energy"][-1]) <= 1e-8 * abs(g["elastic_energy"][-1])


def test_fp64_batch_matches_oracle_per_mesh(fem_lib, oracle):
    scs = [_damped_driven(), scenes.large_block(n=8), scenes.compressed_cube(n=5, steps=20, ratio=0.3),
           scenes.cantilever_160()]
    steps = 12
    b = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_FP64)
    its = [[] for _ in scs]
    for _ in range(steps):
        b.step(1)
        for i in range(len(scs)):
            its[i].append(b.stats(i)["cg_iterations"])
    for i, sc in enumerate(scs):
        ref = oracle_run(oracle, sc, steps)
        x, v = b.state(i)
        ex, ev = rel(x, ref["x"]), rel(v, ref["v"])
        check_bar(f"fp64 batch mesh {i} {sc.name}", "x", ex, 1e-10, ref["noise_x"], bar_cap(sc))
        check_bar(f"fp64 batch mesh {i} {sc.name}", "v", ev, 1e-10, ref["noise_v"], bar_cap(sc))
        worst = max(abs(a - c) for a, c in zip(its[i], ref["iters"]))
        assert worst <= max(1, 2 * ref["spread"] + 1), (i, worst, ref["spread"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_and_in_the_mix_are_identical(fem_lib, precision):
    p = fem_lib.FEM_PRECISION_FP64 if precision == "fp64" else fem_lib.FEM_PRECISION_MIXED
    rng = np.random.default_rng(21)
    target = scenes.random_block(rng, dims=(7, 5, 6), idx=0)
    others = [scenes.random_block(rng, idx=i) for i in range(1, 7)]
    alone = fem_lib.Batch([target], precision=p)
    mix = fem_lib.Batch(others[:3] + [target] + others[3:], precision=p)
    for _ in range(6):
        alone.step(1)
        mix.step(1)
        assert alone.stats(0)["cg_iterations"] == mix.stats(3)["cg_iterations"]
    xa, va = alone.state(0)
    xm, vm = mix.state(3)
    assert np.array_equal(xa, xm) and np.array_equal(va, vm)


def test_mixed_precision_error_vs_fp64_oracle(fem_lib, oracle):
    """Mixed path (FP32 products, FP64 reductions and refresh) against the
    FP64 oracle, tolerance 1e-5: positions by rel-L2; velocities by
    ||v - v_oracle|| / max over the run of ||v_oracle|| (an oscillating body
    passes through v ~ 0, where a plain relative norm divides by ~0)."""
    for sc, steps in ((scenes.cantilever_160(), 120), (scenes.large_block(n=10), 20), (_damped_driven(), 20)):
        b = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED)
        o = oracle.Solid(sc, "port")
        vscale = 0.0
        for _ in range(steps):
            b.step(1)
            o.step()
            vscale = max(vscale, float(np.linalg.norm(o.state()[1])))
        x, v = b.state(0)
        xo, vo = o.state()
        ex = rel(x, xo)
        ev = float(np.linalg.norm(v - vo)) / vscale
        assert ex <= 1e-5 and ev <= 1e-5, (sc.name, ex, ev)


def test_active_mask_leaves_inactive_meshes_untouched(fem_lib):
    rng = np.random.default_rng(3)
    scs = [scenes.random_block(rng, idx=i, dims=(4, 4, 4)) for i in range(4)]
    b = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED)
    b.step(1)
    before = [b.state(i) for i in range(4)]
    b.set_active(np.array([1, 0, 1, 0], np.uint8))
    b.step(2)
    after = [b.state(i) for i in range(4)]
    for i in (1, 3):
        assert np.array_equal(before[i][0], after[i][0]) and np.array_equal(before[i][1], after[i][1])
    for i in (0, 2):
        assert not np.array_equal(before[i][0], after[i][0])


def test_graph_and_host_loop_agree(fem_lib):
    rng = np.random.default_rng(8)
    scs = [scenes.random_block(rng, idx=i) for i in range(3)]
    a = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED, use_graph=True)
    b = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED, use_graph=False)
    a.step(3)
    b.step(3)
    for i in range(3):
        xa, va = a.state(i)
        xb, vb = b.state(i)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)
        assert a.stats(i)["cg_iterations"] == b.stats(i)["cg_iterations"]


@pytest.mark.parametrize("precision,graph", [("fp64", True), ("mixed", True), ("mixed", False)])
def test_sliced_launches_match_whole_steps(fem_lib, precision, graph):
    """An iteration budget per launch (steps continued with mask value 2)
    gives the same bits as whole steps."""
    p = fem_lib.FEM_PRECISION_FP64 if precision == "fp64" else fem_lib.FEM_PRECISION_MIXED
    rng = np.random.default_rng(12)
    scs = [scenes.random_block(rng, idx=i, dims=(4 + i, 3, 5)) for i in range(4)]
    whole = fem_lib.Batch(scs, precision=p, use_graph=graph)
    sliced = fem_lib.Batch(scs, precision=p, use_graph=graph)
    sliced.set_slice(7)
    for _ in range(3):
        whole.step(1)
        sliced.set_active(None)
        sliced.step(1)
        launches = 1
        while True:
            f = sliced.finished()
            if not (f == 2).any():
                break
            sliced.set_active(np.where(f == 2, 2, 0).astype(np.uint8))
            sliced.step(1)
            launches += 1
        assert launches > 1
        for i in range(len(scs)):
            assert whole.stats(i)["cg_iterations"] == sliced.stats(i)["cg_iterations"]
    for i in range(len(scs)):
        xa, va = whole.state(i)
        xb, vb = sliced.state(i)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), i


def test_compressed_cube_fp64_and_mixed_vs_oracle(fem_lib, oracle):
    """Large deformation at a size the oracle runs in seconds: the 8^3 x 5
    cube (E 2e5, nu 0.45) compressed by its top face to 40 % of its height
    over 120 steps. The case is close to unstable: a 1e-15 change of the
    input moves the oracle's final positions by ~1e-8 (an amplification of
    ~1e7 through the CG's discrete stopping points). The mixed path is judged
    against the oracle's own spread: what an FP32-sized change of the input
    (initial velocities perturbed by 6e-8 of the mesh size) does to it, and
    what stopping its CG at rel 1e-7 instead of 1e-6 does to it.
    FP64 path: rel-L2 <= max(1e-10, 10 x the 1e-15 noise floor).
    Mixed path (default double-precision rotations): positions rel-L2 and velocities
    (normalised by the run's peak |v|) <= max(1e-5, 2 x the larger of those
    spreads)."""
    sc = scenes.compressed_cube(n=8, steps=120, ratio=0.4)
    ref = oracle_run(oracle, sc, 120)
    f32_floor_x = f32_floor_v = 0.0
    for seed in (11, 12):
        p = oracle.Solid(perturbed(sc, seed, eps=6e-8), "port")
        for _ in range(120):
            p.step()
        xp, vp = p.state()
        f32_floor_x = max(f32_floor_x, rel(xp, ref["x"]))
        f32_floor_v = max(f32_floor_v, float(np.linalg.norm(vp - ref["v"])) / ref["vmax"])
    tight = oracle.Solid(sc, "port")
    tight.set_solver(sc.rel_eps / 10, sc.abs_eps, sc.max_iter)
    for _ in range(120):
        tight.step()
    xt, vt = tight.state()
    floor_x = max(f32_floor_x, rel(xt, ref["x"]))
    floor_v = max(f32_floor_v, float(np.linalg.norm(vt - ref["v"])) / ref["vmax"])
    f64 = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    mix = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False)
    resolved = 0
    for _ in range(120):
        f64.step(1)
        mix.step(1)
        resolved = max(resolved, mix.stats(0)["fp64_resolved"])
        assert mix.stats(0)["status"] == 0 and f64.stats(0)["status"] == 0
    x, v = f64.state(0)
    check_bar("compressed cube fp64 batch", "x", rel(x, ref["x"]), 1e-10, ref["noise_x"], bar_cap(sc))
    check_bar("compressed cube fp64 batch", "v", rel(v, ref["v"]), 1e-10, ref["noise_v"], bar_cap(sc))
    xm, vm = mix.state(0)
    ex = rel(xm, ref["x"])
    ev = float(np.linalg.norm(vm - ref["v"])) / ref["vmax"]
    check_bar("compressed cube mixed", "x", ex, 1e-5, floor_x, cap=1e-4, mult=2.0)
    check_bar("compressed cube mixed", "v", ev, 1e-5, floor_v, cap=1e-4, mult=2.0)
    assert resolved > 0


def test_mixed_converges_like_fp64_on_stiff_meshes(fem_lib):
    """Stiff meshes of the batched workload (E up to 1e6 Pa): the mixed CG
    reaches the same relative tolerance in about the iterations the FP64 CG
    needs (per mesh within 15 % or 20 iterations -- a CG's stopping point on
    a plateau moves with rounding -- and on average within 3 %: no stagnation
    at the iteration cap), and its states stay within
    max(1e-5, 10 x the FP64 path's own spread between CG tolerances 1e-6 and
    1e-7) of the FP64 path's."""
    rng = np.random.default_rng(77)
    scs = []
    for i in range(24):
        sc = scenes.random_block(rng, lo=6, hi=16, idx=i)
        sc.young = float(np.exp(rng.uniform(np.log(2e5), np.log(1e6))))
        scs.append(sc)
    f64 = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    mix = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False)
    tight = fem_lib.Batch([dataclasses.replace(sc, rel_eps=sc.rel_eps / 10) for sc in scs],
                          precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    tight.step(4)
    vmax = np.zeros(len(scs))
    n64 = nmix = 0
    for _ in range(4):
        f64.step(1)
        mix.step(1)
        for i in range(len(scs)):
            a, m = f64.stats(i), mix.stats(i)
            n64 += a["cg_iterations"]
            nmix += m["cg_iterations"]
            assert m["cg_iterations"] <= a["cg_iterations"] + max(20, 0.15 * a["cg_iterations"]), (i, a, m)
            assert m["rel_residual"] <= scs[i].rel_eps * 1.0001 or m["cg_iterations"] >= a["cg_iterations"], (i, m)
            vmax[i] = max(vmax[i], float(np.linalg.norm(f64.state(i)[1])))
    assert nmix <= 1.03 * n64, (nmix, n64)
    for i in range(len(scs)):
        xa, va = f64.state(i)
        xm, vm = mix.state(i)
        xt, vt = tight.state(i)
        bx = max(1e-5, 10 * rel(xt, xa))
        bv = max(1e-5, 10 * float(np.linalg.norm(vt - va)) / vmax[i])
        ex, ev = rel(xm, xa), float(np.linalg.norm(vm - va)) / vmax[i]
        assert ex <= bx and ev <= bv, (i, ex, ev, bx, bv)


def test_compression_counts_fp64_resolves(fem_lib):
    """FP32 rotations (rotation_fp32 = 1): under heavy compression some
    elements are re-solved at double precision (det F rule, branch ties, sensitivity),
    not all; with the default double-precision rotations every rotation is."""
    sc = scenes.compressed_cube(n=6, steps=20, ratio=0.2)
    b = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, rotation_fp32=1)
    d = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED)
    resolved = []
    for _ in range(20):
        b.step(1)
        d.step(1)
        st = b.stats(0)
        resolved.append(st["fp64_resolved"])
        assert st["status"] == 0 and d.stats(0)["status"] == 0
        assert d.stats(0)["fp64_resolved"] == sc.num_tets
    assert max(resolved[1:]) > 0 and min(resolved[1:]) < sc.num_tets, resolved
    # the FP32 option stays within the mixed bar of the default on this case
    xa, va = d.state(0)
    xb, vb = b.state(0)
    assert rel(xb, xa) <= 1e-4, rel(xb, xa)


@pytest.mark.parametrize("tile_elems,reorder", [(64, False), (128, True), (192, True)])
def test_tile_variants_match_reference_cantilever(fem_lib, tile_elems, reorder):
    """Every tile size and element order the autotuner may pick gives the
    FP64 cantilever within the FP64 bar (1e-10, +-1 iteration)."""
    g = np.load(os.path.join(GOLDEN, "cantilever_160.npz"))
    sc = scenes.cantilever_160()
    b = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64, tile_elems=tile_elems, reorder=reorder)
    for k in range(sc.steps):
        b.step(1)
        assert abs(b.stats(0)["cg_iterations"] - int(g["iters"][k])) <= 1
    x, v = b.state(0)
    assert rel(x, g["x"][-1]) <= 1e-10 and rel(v, g["v"][-1]) <= 1e-10


def test_autotuner_picks_a_measured_candidate(fem_lib, tmp_path, monkeypatch):
    from risdsdgcfem_thesis_gb300 import autotune
    monkeypatch.setenv("FEMGB_CACHE_DIR", str(tmp_path))
    rng = np.random.default_rng(4)
    scs = [scenes.random_block(rng, idx=i) for i in range(6)]
    cands = ((256, 1, 1024), (128, 1, 256))
    out = autotune.tune(scs, fem_lib.FEM_PRECISION_MIXED, candidates=cands, iters=10, reps=2)
    assert not out["cached"] and (out["tile_elems"], out["reorder"], out["chunk_nodes"]) in cands
    assert len(out["table"]) == 2 and all(r["ms_per_launch"] > 0 for r in out["table"])
    again = autotune.tune(scs, fem_lib.FEM_PRECISION_MIXED, candidates=cands, iters=10, reps=2)
    assert again["cached"] and again["tile_elems"] == out["tile_elems"]


def _edge_scenes():
    """A single tet falling free, a block whose every node is fixed, a
    free-floating block with an initial spin (no constraints at all), and a
    block with one fixed node."""
    rest = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0, 0, 0.1]], float)
    one = scenes.Scene(name="one_tet", rest=rest, tets=np.array([[0, 1, 2, 3]], np.uint32), young=2e5,
                       gravity=(0.0, 0.0, -9.81), steps=10)
    r2, t2, _ = scenes.grid_mesh(3, 2, 2, 0.05, 0.005, 3)
    fixed_all = scenes.Scene(name="all_fixed", rest=r2, tets=t2, young=1e5, gravity=(0.0, 0.0, -9.81),
                             knc_nodes=np.arange(r2.shape[0], dtype=np.uint32), knc_targets=r2.copy(), steps=10)
    r3, t3, _ = scenes.grid_mesh(3, 3, 2, 0.05, 0.005, 4)
    c = r3.mean(0)
    spin = np.cross(np.array([0.0, 0.0, 2.0]), r3 - c)
    free = scenes.Scene(name="free_spin", rest=r3, tets=t3, young=5e4, poisson=0.4, init_vel=spin, steps=10)
    r4, t4, _ = scenes.grid_mesh(2, 2, 3, 0.05, 0.005, 5)
    pinned = scenes.Scene(name="one_pin", rest=r4, tets=t4, young=3e5, gravity=(0.0, -9.81, 0.0),
                          knc_nodes=np.array([0], np.uint32), knc_targets=r4[:1].copy(), steps=10)
    return [one, fixed_all, free, pinned]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_edge_case_meshes_vs_oracle_alone_and_in_the_mix(fem_lib, oracle, precision):
    """Ragged batches: each edge-case mesh, in a batch with the others and
    with regular meshes, matches the oracle (FP64: 1e-10 or 10 x the noise
    floor; mixed: 1e-5 of the run's scale) and gives the same bits as when
    it is stepped alone; the fully fixed mesh does not move."""
    p = fem_lib.FEM_PRECISION_FP64 if precision == "fp64" else fem_lib.FEM_PRECISION_MIXED
    edge = _edge_scenes()
    rng = np.random.default_rng(9)
    mix = fem_lib.Batch(edge[:2] + [scenes.random_block(rng, idx=9)] + edge[2:], precision=p)
    index = [0, 1, 3, 4]
    steps = 10
    mix.step(steps)
    for k, sc in enumerate(edge):
        alone = fem_lib.Batch([sc], precision=p)
        alone.step(steps)
        xa, va = alone.state(0)
        xm, vm = mix.state(index[k])
        assert np.array_equal(xa, xm) and np.array_equal(va, vm), sc.name
        ref = oracle_run(oracle, sc, steps)
        scale_x = max(float(np.linalg.norm(ref["x"])), 1e-30)
        scale_v = max(ref["vmax"], 1e-30)
        ex = float(np.linalg.norm(xm - ref["x"])) / scale_x
        ev = float(np.linalg.norm(vm - ref["v"])) / scale_v
        if precision == "fp64":
            noise_v = ref["noise_v"] * float(np.linalg.norm(ref["v"])) / scale_v
            check_bar(f"edge case fp64 {sc.name}", "x", ex, 1e-10, ref["noise_x"], bar_cap(sc))
            check_bar(f"edge case fp64 {sc.name}", "v", ev, 1e-10, noise_v, bar_cap(sc))
        else:
            assert ex <= 1e-5 and ev <= 1e-5, (sc.name, ex, ev)
        alone.close()
    x1, v1 = mix.state(1)
    assert np.array_equal(x1, edge[1].rest) and not np.any(v1)


def test_fused_alpha_gives_the_same_bits(fem_lib):
    """fuse_alpha (each node-pass block forms its mesh's alpha, no separate
    kernel) runs the same fixed-order sum as the alpha kernel: states and
    iteration counts are bit-identical to the default."""
    rng = np.random.default_rng(21)
    scs = [scenes.random_block(rng, lo=3, hi=8, idx=i) for i in range(5)]
    a = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False)
    f = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, fuse_alpha=True)
    try:
        for _ in range(3):
            a.step(1)
            f.step(1)
            for i in range(len(scs)):
                assert a.stats(i)["cg_iterations"] == f.stats(i)["cg_iterations"], i
        for i in range(len(scs)):
            xa, va = a.state(i)
            xf, vf = f.state(i)
            assert np.array_equal(xa, xf) and np.array_equal(va, vf), i
    finally:
        a.close()
        f.close()
