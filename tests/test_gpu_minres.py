"""MINRES on the FP64 solid, through the C ABI, against the fixture the
reference's own ILSS_MINRES wrote (tests/golden/minres.npz).

Tolerances (FP64): on the cantilever (QIE 60 steps, FIE 20 steps) x and v
rel-L2 <= 1e-10 and iterations within 1 per solve per step; the driven block
stops at rel 1e-6 after few iterations and is as sensitive as the oracle
itself (5e-8 in x, 8e-7 in v under 1e-15 perturbations of the initial
positions), so its bar is max(1e-10, 10 x that spread) measured here, and
iterations within max(1, 2 x spread + 1).
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _cases():
    from test_oracle_minres import minres_cases
    return minres_cases()


@pytest.mark.parametrize("case", [0, 1])
def test_minres_cantilever_matches_reference(fem_lib, case):
    g = np.load(os.path.join(GOLDEN, "minres.npz"))
    prefix, sc, steps = _cases()[case]
    s = fem_lib.Solid(sc)
    for k in range(steps):
        st = s.step(1)
        assert st["status"] == 0
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= max(1, st["nr_iterations"]), k
        assert st["nr_iterations"] == int(g[prefix + "nr_iters"][k])
    x, v = s.state()
    assert rel(x, g[prefix + "x"]) <= 1e-10 and rel(v, g[prefix + "v"]) <= 1e-10, \
        (rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    # MINRES's residual estimate at the stop (|r| carried by the Givens
    # sines) lands anywhere just below the target: below rel_eps and within
    # 50 % of the reference's
    ref_rel = float(g[prefix + "rel_res"][-1])
    assert st["rel_residual"] <= sc.rel_eps and abs(st["rel_residual"] - ref_rel) <= 0.5 * ref_rel


def test_minres_driven_block_matches_reference(fem_lib, oracle):
    g = np.load(os.path.join(GOLDEN, "minres.npz"))
    prefix, sc, steps = _cases()[2]
    fx, fv, spread = 0.0, 0.0, 0
    for seed in (1, 2, 3):
        o = oracle.Solid(sc, "port")
        x0 = sc.rest + 1e-15 * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
        o.set_state(x0, sc.init_vel)
        its = [o.step()["iters"] for _ in range(steps)]
        spread = max(spread, max(abs(a - int(b)) for a, b in zip(its, g[prefix + "iters"])))
        x, v = o.state()
        fx, fv = max(fx, rel(x, g[prefix + "x"])), max(fv, rel(v, g[prefix + "v"]))
    s = fem_lib.Solid(sc)
    for k in range(steps):
        st = s.step(1)
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= max(1, 2 * spread + 1), k
    x, v = s.state()
    assert rel(x, g[prefix + "x"]) <= max(1e-10, 10 * fx), (rel(x, g[prefix + "x"]), fx)
    assert rel(v, g[prefix + "v"]) <= max(1e-10, 10 * fv), (rel(v, g[prefix + "v"]), fv)


@pytest.mark.parametrize("assembled", [False, True])
def test_minres_matches_oracle_on_random_block(fem_lib, oracle, assembled):
    """2,400 tets under gravity, MINRES with FIE, against the oracle run here;
    with the element products and with the assembled stiffness."""
    rng = np.random.default_rng(21)
    sc = scenes.random_block(rng, dims=(10, 6, 8))
    sc.integrator = fem_lib.FEM_INTEGRATOR_FIE_DX
    sc.ls_solver = fem_lib.FEM_LS_MINRES
    sc.gravity = (0.0, 0.0, -9.81)
    sc.rel_eps, sc.max_iter = 1e-8, 400
    a = fem_lib.Solid(sc)
    a.set_assembled(assembled)
    b = oracle.Solid(sc, "port")
    for _ in range(4):
        sa, sb = a.step(1), b.step()
        assert sa["nr_iterations"] == sb["nr_iters"]
        assert abs(sa["cg_iterations"] - sb["iters"]) <= max(sa["nr_iterations"], int(np.ceil(0.02 * sb["iters"])))
    xa, va = a.state()
    xb, vb = b.state()
    assert rel(xa, xb) <= 1e-10 and rel(va, vb) <= 1e-8, (rel(xa, xb), rel(va, vb))


@pytest.mark.parametrize("case", [0, 2])
def test_fp64_batch_minres_matches_reference(fem_lib, oracle, case):
    """MINRES meshes in an FP64 batch (the reference's recurrence per mesh:
    v1 = A v - beta v0, alpha = v1.v, Givens, the iterate update), next to a
    CG mesh: the QIE cases of the fixture, with the solid's bars (the
    cantilever 1e-10 and iterations within 1; the driven block within 10 x
    the oracle's own spread under 1e-13 perturbations of the initial
    positions -- the batch sums in another order than the solid, which moves
    the block's iteration counts as much as such a perturbation does in the
    oracle: 6 to 10 iterations at step 10). The CG mesh's result is the
    same bits as in a batch of its own."""
    g = np.load(os.path.join(GOLDEN, "minres.npz"))
    prefix, sc, steps = _cases()[case]
    fx, fv, spread = 0.0, 0.0, 0
    if case == 2:
        for seed in (1, 2, 3, 4, 5, 6):
            o = oracle.Solid(sc, "port")
            x0 = sc.rest + 1e-13 * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
            o.set_state(x0, sc.init_vel)
            its = [o.step()["iters"] for _ in range(steps)]
            spread = max(spread, max(abs(a - int(b)) for a, b in zip(its, g[prefix + "iters"])))
            x, v = o.state()
            fx, fv = max(fx, rel(x, g[prefix + "x"])), max(fv, rel(v, g[prefix + "v"]))
    cg = scenes.cantilever_160()
    bt = fem_lib.Batch([cg, sc], precision=fem_lib.FEM_PRECISION_FP64)
    alone = fem_lib.Batch([cg], precision=fem_lib.FEM_PRECISION_FP64)
    for k in range(steps):
        bt.step(1)
        alone.step(1)
        st = bt.stats(1)
        assert st["status"] == 0
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= max(1, 2 * spread + 1), k
    x, v = bt.state(1)
    assert rel(x, g[prefix + "x"]) <= max(1e-10, 10 * fx), (rel(x, g[prefix + "x"]), fx)
    assert rel(v, g[prefix + "v"]) <= max(1e-10, 10 * fv), (rel(v, g[prefix + "v"]), fv)
    if case == 0:
        ref_rel = float(g[prefix + "rel_res"][-1])
        assert st["rel_residual"] <= sc.rel_eps and abs(st["rel_residual"] - ref_rel) <= 0.5 * ref_rel
    xa, va = alone.state(0)
    xc, vc = bt.state(0)
    assert np.array_equal(xa, xc) and np.array_equal(va, vc)


def test_mixed_batch_and_server_minres_match_reference(fem_lib):
    """MINRES on the mixed path (FP32 Lanczos vectors and products, FP64
    iterate; when the Givens estimate passes, the FP64 residual of the
    iterate decides, restarting MINRES from it if needed): within 1e-5 of
    the reference's fixture after the 60 cantilever steps, every step's
    FP64 relative residual at or below rel_eps, in a batch and, the same
    bits alone, next to a CG mesh and through the server."""
    g = np.load(os.path.join(GOLDEN, "minres.npz"))
    prefix, sc, steps = _cases()[0]
    bt = fem_lib.Batch([scenes.cantilever_160(), sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False,
                       chunk_nodes=256)
    for k in range(steps):
        bt.step(1)
        st = bt.stats(1)
        assert st["status"] == 0 and st["rel_residual"] <= sc.rel_eps, (k, st)
        assert st["cg_iterations"] >= int(g[prefix + "iters"][k]) - 2, k
    x, v = bt.state(1)
    assert rel(x, g[prefix + "x"]) <= 1e-5 and rel(v, g[prefix + "v"]) <= 1e-4, \
        (rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED)
    sid = srv.add(sc)
    srv.admit()
    for k in range(steps):
        srv.submit(sid, k)
    done = srv.drain()
    assert len(done) == steps and all(c["status"] == 0 for c in done)
    one = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
    one.step(steps)
    xs, vs = srv.state(sid)
    xo, vo = one.state(0)
    assert np.array_equal(xo, x) and np.array_equal(vo, v)
    assert np.array_equal(xs, x) and np.array_equal(vs, v)


def test_persistent_loop_rejects_minres(fem_lib):
    sc = dataclasses.replace(scenes.cantilever_160(), ls_solver=1)
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, persistent_loop=1)
    assert e.value.code == fem_lib.FEM_E_ARG
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.Batch([dataclasses.replace(sc, ls_solver=7)], precision=fem_lib.FEM_PRECISION_FP64)
    assert e.value.code == fem_lib.FEM_E_ARG
