"""Fully-implicit Euler (Newton on Delta x) on the FP64 solid, through the C
ABI, against the fixtures the reference's own element set and CG wrote
(tests/golden/fie_160.npz, fie_block.npz; the oracle restatement equals them
bit for bit).

Tolerances (FP64): positions and velocities rel-L2 <= 1e-10 after the run
(the quasi-static case: max(1e-10, 10 x the oracle's own sensitivity));
Newton iterations per step equal; CG iterations per step (summed over the
step's Newton solves) within max(1 per solve, 2 %): on the damped block the
residual plateaus near the threshold and the stopping iteration moves by a
few between orderings of the same sums; energies rel <= 1e-8; the last
Newton norm rel <= 1e-2 (it is |y_k| of the last correction, or |b_k| once
that fell below nr_abs_epsilon: a residual at the CG tolerance's level, which
moves by up to 1.5e-3 in the oracle itself under 1e-15 perturbations of the
initial velocity).
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _cg_slack(st):
    """CG iterations of a step may differ by one per Newton solve, or by 2 %
    where the residual sits on a plateau near the stopping threshold."""
    return max(st["nr_iterations"], int(np.ceil(0.02 * st["cg_iterations"])))


def _check_steps(stats, g, prefix=""):
    for k, st in enumerate(stats):
        assert st["status"] == 0
        assert st["nr_iterations"] == int(g[prefix + "nr_iters"][k]), k
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= _cg_slack(st), \
            (k, st["cg_iterations"], g[prefix + "iters"][k])
        assert abs(st["nr_abs_residual"] - g[prefix + "nr_abs"][k]) <= 1e-2 * g[prefix + "nr_abs"][k], k
    last = stats[-1]
    for key, gk in (("elastic_energy", "elastic_energy"), ("potential_energy", "potential_energy")):
        ref = float(g[prefix + gk][len(stats) - 1])
        assert abs(last[key] - ref) <= 1e-8 * abs(ref), key


def test_fie_cantilever_matches_reference(fem_lib):
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    sc = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    s = fem_lib.Solid(sc)
    stats = [s.step(1) for _ in range(g["x"].shape[0])]
    _check_steps(stats, g)
    x, v = s.state()
    ex, ev = rel(x, g["x"][-1]), rel(v, g["v"][-1])
    assert ex <= TOL and ev <= TOL, (ex, ev)


def test_fie_quasistatic_cantilever_matches_reference(fem_lib, oracle):
    """Quasi-static steps far from equilibrium (each step stops at the Newton
    cap with |b_k| near 5): the result is as sensitive to the last bits as
    the CG's stopping point, so the bar is max(1e-10, 10 x the oracle's own
    spread under 1e-15 perturbations of the initial positions), measured
    here (about 5e-9)."""
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    sc = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX_QUASISTATIC)
    steps = g["q_iters"].shape[0]
    floor, spread = 0.0, 0
    for seed in (1, 2, 3):
        o = oracle.Solid(sc, "port")
        x0 = sc.rest + 1e-15 * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
        o.set_state(x0, np.zeros_like(x0))
        its = [o.step()["iters"] for _ in range(steps)]
        spread = max(spread, max(abs(a - int(b)) for a, b in zip(its, g["q_iters"])))
        floor = max(floor, rel(o.state()[0], g["xq"]))
    s = fem_lib.Solid(sc)
    stats = [s.step(1) for _ in range(steps)]
    for k, st in enumerate(stats):
        assert st["status"] == 0 and st["nr_iterations"] == int(g["q_nr_iters"][k])
        assert abs(st["cg_iterations"] - int(g["q_iters"][k])) <= max(st["nr_iterations"], 2 * spread + 1), k
    x, v = s.state()
    assert rel(x, g["xq"]) <= max(TOL, 10 * floor), (rel(x, g["xq"]), floor)
    assert not np.any(v)


def test_fie_block_moving_constraint_matches_reference(fem_lib):
    """Per-element E and nu, damping, initial velocity and a constraint moved
    every step; some steps leave the Newton loop on |b_k| < nr_abs_epsilon."""
    g = np.load(os.path.join(GOLDEN, "fie_block.npz"))
    rng = np.random.default_rng(5)
    sc = scenes.random_block(rng, dims=(5, 3, 4))
    T = sc.num_tets
    sc.young_per_elem = np.exp(rng.uniform(np.log(5e4), np.log(5e5), T))
    sc.poisson_per_elem = rng.uniform(0.25, 0.45, T)
    sc.damping_ratio = 1.0
    sc.init_vel = rng.standard_normal(sc.rest.shape) * 0.1
    base = sc.knc_targets.copy()
    sc.knc_schedule = lambda k: base + np.array([0.0, 0.0, 0.002 * (k + 1)])
    sc.steps = 12
    sc.integrator = fem_lib.FEM_INTEGRATOR_FIE_DX
    sc.nr_max_iter = 4
    s = fem_lib.Solid(sc)
    stats = s.run()
    _check_steps(stats, g)
    assert min(st["nr_iterations"] for st in stats) < sc.nr_max_iter
    x, v = s.state()
    ex, ev = rel(x, g["x"]), rel(v, g["v"])
    assert ex <= TOL and ev <= TOL, (ex, ev)


def test_fie_matches_oracle_on_random_block(fem_lib, oracle):
    """A larger block than the fixtures (2,000+ tets), FIE dynamic, against the
    oracle restatement run here."""
    rng = np.random.default_rng(21)
    sc = scenes.random_block(rng, dims=(10, 6, 8))
    sc.integrator = fem_lib.FEM_INTEGRATOR_FIE_DX
    sc.gravity = (0.0, 0.0, -9.81)
    sc.rel_eps, sc.max_iter = 1e-8, 400
    a = fem_lib.Solid(sc)
    b = oracle.Solid(sc, "port")
    for _ in range(5):
        sa, sb = a.step(1), b.step()
        assert sa["nr_iterations"] == sb["nr_iters"]
        assert abs(sa["cg_iterations"] - sb["iters"]) <= _cg_slack(sa)
    xa, va = a.state()
    xb, vb = b.state()
    assert rel(xa, xb) <= TOL and rel(va, vb) <= 1e-8, (rel(xa, xb), rel(va, vb))


def _block_scene():
    from test_oracle_fie import _fie_block_scene
    return _fie_block_scene()


def test_fp64_batch_fie_matches_reference(fem_lib):
    """FIE meshes in an FP64 batch, each leaving the device-side Newton loop
    on its own test (the cantilever stops at the Newton cap, the block with
    a moving constraint partly on |b_k|), next to a QIE mesh: each against
    the fixture the reference's element set wrote, with the solid's bars
    (x, v 1e-10; Newton iterations equal; CG iterations within one per
    solve or 2 %; energies 1e-8). The QIE mesh's result is the same bits as
    in a batch of its own, and the host-driven loops give the graph's bits."""
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    gb = np.load(os.path.join(GOLDEN, "fie_block.npz"))
    cant = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    block = _block_scene()
    qie = scenes.cantilever_160()
    bt = fem_lib.Batch([cant, block, qie], precision=fem_lib.FEM_PRECISION_FP64)
    host = fem_lib.Batch([cant, block, qie], precision=fem_lib.FEM_PRECISION_FP64, use_graph=False)
    alone = fem_lib.Batch([qie], precision=fem_lib.FEM_PRECISION_FP64)
    stats0, stats1 = [], []
    for k in range(g["x"].shape[0]):
        bt.step(1)
        host.step(1)
        alone.step(1)
        stats0.append(bt.stats(0))
        if k < len(gb["iters"]):
            stats1.append(bt.stats(1))
        if k + 1 == len(gb["iters"]):
            xb, vb = bt.state(1)
            assert rel(xb, gb["x"]) <= TOL and rel(vb, gb["v"]) <= TOL, (rel(xb, gb["x"]), rel(vb, gb["v"]))
    _check_steps(stats0, g)
    _check_steps(stats1, gb)
    assert min(st["nr_iterations"] for st in stats1) < block.nr_max_iter
    x, v = bt.state(0)
    assert rel(x, g["x"][-1]) <= TOL and rel(v, g["v"][-1]) <= TOL, (rel(x, g["x"][-1]), rel(v, g["v"][-1]))
    xa, va = alone.state(0)
    xq, vq = bt.state(2)
    assert np.array_equal(xa, xq) and np.array_equal(va, vq)
    for i in range(3):
        xh, vh = host.state(i)
        xg, vg = bt.state(i)
        assert np.array_equal(xh, xg) and np.array_equal(vh, vg), i


def test_fp64_batch_fie_quasistatic_matches_reference(fem_lib, oracle):
    """The quasi-static cantilever (every step at the Newton cap) in a batch
    next to a dynamic FIE mesh, with the solid's bar: max(1e-10, 10 x the
    oracle's own spread under 1e-15 perturbations of the initial
    positions)."""
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    sc = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX_QUASISTATIC)
    steps = g["q_iters"].shape[0]
    floor, spread = 0.0, 0
    for seed in (1, 2, 3):
        o = oracle.Solid(sc, "port")
        x0 = sc.rest + 1e-15 * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
        o.set_state(x0, np.zeros_like(x0))
        its = [o.step()["iters"] for _ in range(steps)]
        spread = max(spread, max(abs(a - int(b)) for a, b in zip(its, g["q_iters"])))
        floor = max(floor, rel(o.state()[0], g["xq"]))
    other = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    bt = fem_lib.Batch([other, sc], precision=fem_lib.FEM_PRECISION_FP64)
    for k in range(steps):
        bt.step(1)
        st = bt.stats(1)
        assert st["status"] == 0 and st["nr_iterations"] == int(g["q_nr_iters"][k])
        assert abs(st["cg_iterations"] - int(g["q_iters"][k])) <= max(st["nr_iterations"], 2 * spread + 1), k
    x, v = bt.state(1)
    assert rel(x, g["xq"]) <= max(TOL, 10 * floor), (rel(x, g["xq"]), floor)
    assert not np.any(v)


def test_mixed_batch_fie_matches_reference(fem_lib):
    """FIE on the mixed path (FP32 products in the CG loops, FP64 Newton
    level: b_k, the update, the tests): the cantilever and the block with
    a moving constraint within 1e-5 (x) and 1e-4 (v) of the fixtures, every
    step's status 0; graph and host-driven loops give the same bits."""
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    gb = np.load(os.path.join(GOLDEN, "fie_block.npz"))
    cant = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    block = _block_scene()
    bt = fem_lib.Batch([cant, block], precision=fem_lib.FEM_PRECISION_MIXED, chunk_nodes=256)
    host = fem_lib.Batch([cant, block], precision=fem_lib.FEM_PRECISION_MIXED, chunk_nodes=256, use_graph=False)
    nb = len(gb["iters"])
    for k in range(g["x"].shape[0]):
        bt.step(1)
        host.step(1)
        assert bt.stats(0)["status"] == 0 and bt.stats(1)["status"] == 0, k
        assert bt.stats(0)["nr_iterations"] == int(g["nr_iters"][k]), k
        if k + 1 == nb:
            xb, vb = bt.state(1)
            assert rel(xb, gb["x"]) <= 1e-5 and rel(vb, gb["v"]) <= 1e-4, (rel(xb, gb["x"]), rel(vb, gb["v"]))
    x, v = bt.state(0)
    assert rel(x, g["x"][-1]) <= 1e-5 and rel(v, g["v"][-1]) <= 1e-4, (rel(x, g["x"][-1]), rel(v, g["v"][-1]))
    for i in range(2):
        xh, vh = host.state(i)
        xg, vg = bt.state(i)
        assert np.array_equal(xh, xg) and np.array_equal(vh, vg), i


def test_fie_batch_runs_newton_steps_whole(fem_lib):
    """A batch with an FIE mesh takes no iteration budget (a Newton step runs
    whole); the persistent loop takes QIE meshes only."""
    sc = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64)
    with pytest.raises(fem_lib.FemError) as e:
        bt.set_slice(10)
    assert e.value.code == fem_lib.FEM_E_ARG
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, persistent_loop=1)
    assert e.value.code == fem_lib.FEM_E_ARG


def test_server_steps_fie_scenes_in_whole_step_shards(fem_lib):
    """The server takes FIE scenes into shards of their own (whole Newton
    steps, no iteration budget) beside sliced QIE shards: each scene's
    result is the bits of a mixed batch of its own, the FIE cantilever
    within 1e-5 of the fixture."""
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    cant = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    quasi = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX_QUASISTATIC)
    qie = scenes.cantilever_160()
    steps = 10
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED)
    ids = [srv.add(sc) for sc in (cant, qie, quasi)]
    srv.admit()
    for k in range(steps):
        for i in ids:
            srv.submit(i, k)
    done = srv.drain()
    assert len(done) == 3 * steps and all(c["status"] == 0 for c in done)
    for i, sc in zip(ids, (cant, qie, quasi)):
        one = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
        one.step(steps)
        xs, vs = srv.state(i)
        xo, vo = one.state(0)
        assert np.array_equal(xs, xo) and np.array_equal(vs, vo), sc.integrator
    x, v = srv.state(ids[0])
    assert rel(x, g["x"][steps - 1]) <= 1e-5 and rel(v, g["v"][steps - 1]) <= 1e-4


def test_fp64_batch_fie_with_every_alternative_matches_oracle(fem_lib, oracle):
    """One FP64 batch holding the crushed cube with FIE, DAPD, C_LCM and
    MINRES together, next to a QIE cantilever: the cube against the oracle
    restatement over 8 steps within max(1e-10, 10 x the oracle's movement
    under a 1e-13 change of the initial velocities), capped per scene; the
    Newton iteration counts equal the oracle's."""
    from parity_util import bar_cap, check_bar, perturbed
    sc = dataclasses.replace(scenes.compressed_cube(n=4, steps=10, ratio=0.4), rotation=1, material=1,
                             ls_solver=1, integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    steps = 8
    o = oracle.Solid(sc, "port")
    noisy = [oracle.Solid(perturbed(sc, s, eps=1e-13), "port") for s in (1, 2, 3)]
    bt = fem_lib.Batch([scenes.cantilever_160(), sc], precision=fem_lib.FEM_PRECISION_FP64)
    for k in range(steps):
        so = o.step()
        for n in noisy:
            n.step()
        bt.step(1)
        st = bt.stats(1)
        assert st["status"] == 0 and st["nr_iterations"] == so["nr_iters"], (k, st, so)
    xo, vo = o.state()
    xg, vg = bt.state(1)
    fx = max(rel(n.state()[0], xo) for n in noisy)
    fv = max(rel(n.state()[1], vo) for n in noisy)
    check_bar("fp64 batch FIE+DAPD+C_LCM+MINRES", "x", rel(xg, xo), TOL, fx, bar_cap(sc))
    check_bar("fp64 batch FIE+DAPD+C_LCM+MINRES", "v", rel(vg, vo), TOL, fv, bar_cap(sc))


def test_fie_batch_with_a_mesh_left_out(fem_lib):
    """fem_batch_set_active over an FIE batch: the mesh left out keeps its
    state, the other steps as in a batch of its own (same bits)."""
    cant = dataclasses.replace(scenes.cantilever_160(), integrator=fem_lib.FEM_INTEGRATOR_FIE_DX)
    block = _block_scene()
    bt = fem_lib.Batch([cant, block], precision=fem_lib.FEM_PRECISION_FP64)
    x1, v1 = bt.state(1)
    bt.set_active(np.array([1, 0], np.uint8))
    bt.step(3)
    xb, vb = bt.state(1)
    assert np.array_equal(xb, x1) and np.array_equal(vb, v1)
    alone = fem_lib.Batch([cant], precision=fem_lib.FEM_PRECISION_FP64)
    alone.step(3)
    xa, va = alone.state(0)
    x0, v0 = bt.state(0)
    assert np.array_equal(xa, x0) and np.array_equal(va, v0)
    assert bt.stats(0)["nr_iterations"] == alone.stats(0)["nr_iterations"]
