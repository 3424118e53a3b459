"""The C_LCM material on the FP64 solid, through the C ABI, against the
fixture the reference's element set built with eMM_C_LCM wrote
(tests/golden/lcm.npz) and the oracle restatement.

Tolerances (FP64): x and v rel-L2 <= 1e-10 after the runs (the oracle moves
by at most 2e-14 under 1e-15 perturbations here), iterations within 1 per
solve per step; element force, differential and energy within 1e-12 of the
oracle's at a deformed state.
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


@pytest.mark.parametrize("case", [0, 1, 2])
def test_lcm_matches_reference(fem_lib, case):
    from test_oracle_lcm import lcm_cases
    g = np.load(os.path.join(GOLDEN, "lcm.npz"))
    prefix, sc, steps = lcm_cases()[case]
    s = fem_lib.Solid(sc)
    for k in range(steps):
        st = s.step(1)
        assert st["status"] == 0
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= max(1, st["nr_iterations"]), k
    x, v = s.state()
    assert rel(x, g[prefix + "x"]) <= 1e-10 and rel(v, g[prefix + "v"]) <= 1e-10, \
        (rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    ref_e = float(g[prefix + "elastic_energy"][-1])
    assert abs(st["elastic_energy"] - ref_e) <= 1e-8 * abs(ref_e)


def test_lcm_element_hooks_match_oracle(fem_lib, oracle):
    rng = np.random.default_rng(9)
    sc = dataclasses.replace(scenes.random_block(rng, dims=(4, 3, 3)), material=1)
    x = sc.rest + 0.05 * sc.h * rng.standard_normal(sc.rest.shape)
    dx = rng.standard_normal(sc.rest.shape)
    g = fem_lib.Solid(sc)
    o = oracle.Solid(sc, "port")
    g.begin_eval(x)
    o.begin_eval(x)
    assert rel(g.f_e(), o.f_e()) <= 1e-12
    assert rel(g.df_x(dx), o.df_x(dx)) <= 1e-12
    assert abs(g.V() - o.V()) <= 1e-12 * abs(o.V())


@pytest.mark.parametrize("case", [0, 2])
def test_fp64_batch_lcm_matches_reference(fem_lib, case):
    """C_LCM meshes in an FP64 batch (the FP64 solid's element arithmetic,
    V, mu and lambda apart), next to a C_WRP mesh: the QIE cases of the
    fixture the reference's element set wrote, rel-L2 <= 1e-10, iterations
    within 1 per step, elastic energy 1e-8."""
    from test_oracle_lcm import lcm_cases
    g = np.load(os.path.join(GOLDEN, "lcm.npz"))
    prefix, sc, steps = lcm_cases()[case]
    bt = fem_lib.Batch([scenes.cantilever_160(), sc], precision=fem_lib.FEM_PRECISION_FP64)
    for k in range(steps):
        bt.step(1)
        st = bt.stats(1)
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= 1, k
    x, v = bt.state(1)
    assert rel(x, g[prefix + "x"]) <= 1e-10 and rel(v, g[prefix + "v"]) <= 1e-10, \
        (rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    ref_e = float(g[prefix + "elastic_energy"][-1])
    assert abs(st["elastic_energy"] - ref_e) <= 1e-8 * abs(ref_e)


def test_mixed_batch_and_server_lcm_match_reference(fem_lib):
    """C_LCM on the mixed path (FP32 products on the element's V lambda and V
    mu, FP64 force and refresh): within 1e-5 of the reference's fixture after
    the 60 cantilever steps, in a batch and through the server (the mixed
    batch's bits)."""
    from test_oracle_lcm import lcm_cases
    g = np.load(os.path.join(GOLDEN, "lcm.npz"))
    prefix, sc, steps = lcm_cases()[0]
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
    bt.step(steps)
    x, v = bt.state(0)
    assert rel(x, g[prefix + "x"]) <= 1e-5 and rel(v, g[prefix + "v"]) <= 1e-4, \
        (rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED)
    sid = srv.add(sc)
    srv.admit()
    for k in range(steps):
        srv.submit(sid, k)
    done = srv.drain()
    assert len(done) == steps and all(c["status"] == 0 for c in done)
    xs, vs = srv.state(sid)
    assert np.array_equal(xs, x) and np.array_equal(vs, v)


@pytest.mark.parametrize("case", [0, 1, 3])
def test_fp64_batch_lcmh_matches_reference(fem_lib, case):
    """C_LCMH meshes in an FP64 batch (the solid's pk_dforce on the F and
    det F of the last evaluation), next to a C_WRP mesh: the fixture's cases
    (blend radius 1 and 0.05) with the solid's bars."""
    from test_oracle_materials import material_cases
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    prefix, sc, steps = material_cases()[case]
    bt = fem_lib.Batch([scenes.cantilever_160(), sc], precision=fem_lib.FEM_PRECISION_FP64)
    for k in range(steps):
        bt.step(1)
        st = bt.stats(1)
        assert st["status"] == 0
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= 1, k
    x, v = bt.state(1)
    assert rel(x, g[prefix + "x"]) <= 1e-10 and rel(v, g[prefix + "v"]) <= 1e-10, \
        (prefix, rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    ref_e = float(g[prefix + "elastic_energy"][-1])
    assert abs(st["elastic_energy"] - ref_e) <= 1e-8 * abs(ref_e)


def test_mixed_batch_and_server_lcmh_match_reference(fem_lib):
    """C_LCMH on the mixed path (the blend weight of each element from the
    last evaluation, FP32 products): the cantilever within 1e-5 (x) and 1e-4
    (v) of the fixture, in a batch and, the same bits, through the server."""
    from test_oracle_materials import material_cases
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    prefix, sc, steps = material_cases()[0]
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
    bt.step(steps)
    x, v = bt.state(0)
    assert rel(x, g[prefix + "x"]) <= 1e-5 and rel(v, g[prefix + "v"]) <= 1e-4, \
        (rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED)
    sid = srv.add(sc)
    srv.admit()
    for k in range(steps):
        srv.submit(sid, k)
    done = srv.drain()
    assert len(done) == steps and all(c["status"] == 0 for c in done)
    xs, vs = srv.state(sid)
    assert np.array_equal(xs, x) and np.array_equal(vs, v)


def test_fp64_batch_ccm_runs_away_as_in_the_reference(fem_lib):
    """C_CCM in an FP64 batch: the first step's CG diverges as the fixture's
    (iteration cap, relative residual > 1), the run ends in FEM_E_NAN; the
    mixed path refuses C_CCM."""
    from test_oracle_materials import material_cases
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    prefix, sc, steps = material_cases()[2]
    assert prefix == "ccm_"
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64)
    bt.step(1)
    st = bt.stats(0)
    assert st["cg_iterations"] == int(g["ccm_iters"][0]) == sc.max_iter
    assert st["rel_residual"] > 1.0
    with pytest.raises(fem_lib.FemError) as e:
        for _ in range(steps):
            bt.step(1)
    assert e.value.code == fem_lib.FEM_E_NAN
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED)
    assert e.value.code == fem_lib.FEM_E_ARG


@pytest.mark.parametrize("case", [0, 1, 3])
def test_lcmh_matches_reference(fem_lib, case):
    """C_LCMH (blend radius 1, and 0.05 where it is C_LCM's differential) on
    the cantilever and the moving-constraint block, against the fixture the
    reference's element set built with eMM_C_LCMH wrote (materials.npz):
    rel-L2 <= 1e-10, iterations within 1 per step, energy 1e-8."""
    from test_oracle_materials import material_cases
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    prefix, sc, steps = material_cases()[case]
    s = fem_lib.Solid(sc)
    for k in range(steps):
        st = s.step(1)
        assert st["status"] == 0
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= 1, k
    x, v = s.state()
    assert rel(x, g[prefix + "x"]) <= 1e-10 and rel(v, g[prefix + "v"]) <= 1e-10, \
        (prefix, rel(x, g[prefix + "x"]), rel(v, g[prefix + "v"]))
    ref_e = float(g[prefix + "elastic_energy"][-1])
    assert abs(st["elastic_energy"] - ref_e) <= 1e-8 * abs(ref_e)


@pytest.mark.parametrize("material,k", [(2, 1.0), (3, 1.0)])
def test_lcmh_and_ccm_element_hooks_match_oracle(fem_lib, oracle, material, k):
    rng = np.random.default_rng(9)
    sc = dataclasses.replace(scenes.random_block(rng, dims=(4, 3, 3)), material=material, ecie_k_factor=k)
    x = sc.rest + 0.05 * sc.h * rng.standard_normal(sc.rest.shape)
    dx = rng.standard_normal(sc.rest.shape)
    g = fem_lib.Solid(sc)
    o = oracle.Solid(sc, "port")
    g.begin_eval(x)
    o.begin_eval(x)
    assert rel(g.f_e(), o.f_e()) <= 1e-12
    assert rel(g.df_x(dx), o.df_x(dx)) <= 1e-12
    assert abs(g.V() - o.V()) <= 1e-12 * max(abs(o.V()), 1e-300)


def test_ccm_runs_away_as_in_the_reference(fem_lib):
    """C_CCM's CG diverges from the first step (its A is not symmetric, see
    the oracle tests); the reference's state then runs to Inf/NaN within 10
    steps (materials.npz). Here the first step matches the fixture's
    diverging CG in iteration count, and the run ends in FEM_E_NAN."""
    from test_oracle_materials import material_cases
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    prefix, sc, steps = material_cases()[2]
    assert prefix == "ccm_"
    s = fem_lib.Solid(sc)
    st = s.step(1)
    assert st["cg_iterations"] == int(g["ccm_iters"][0]) == sc.max_iter
    assert st["rel_residual"] > 1.0 and g["ccm_rel_res"][0] > 1.0
    with pytest.raises(fem_lib.FemError) as e:
        for _ in range(steps):
            s.step(1)
    assert e.value.code == fem_lib.FEM_E_NAN
