"""Oracle pinning for the fully-implicit Euler integrator (CPU).

Step_FullyImplicitEuler_dx (LeafDSH_Solid3D_FEM.cpp:1357-1552): Newton on
Delta x with the rotations and the elastic force re-evaluated at every Newton
iterate. The restatement (oracle/fem_oracle.c, step_fie) is checked against
  * the restated Leaf driver around the reference's own element set and CG
    (oracle/ref_harness.cpp, step_fie), bit for bit, where the reference
    sources are present;
  * the fixtures that driver wrote (tests/golden/fie_160.npz, fie_block.npz);
  * equilibrium: the quasi-static variant, iterated to convergence, balances
    gravity against the elastic force on every free node.
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAT_KEYS = ("iters", "rel_res", "abs_res", "elastic_energy", "potential_energy", "nr_iters", "nr_rel", "nr_abs")


def _have_ref(oracle):
    return os.path.exists(oracle.REF_DBL_SO)


def _fie_block_scene():
    """The moving-constraint block of tests/golden/make_golden.py (fie_block_scene)."""
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
    sc.integrator = 1
    sc.nr_max_iter = 4
    return sc


def _cantilever(integrator):
    sc = scenes.cantilever_160()
    sc.integrator = integrator
    return sc


@pytest.mark.parametrize("integrator", [1, 2])
def test_fie_port_equals_reference_bitwise_cantilever(oracle, integrator):
    if not _have_ref(oracle):
        pytest.skip("reference sources not present in this container")
    sc = _cantilever(integrator)
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for step in range(8):
        assert a.step() == b.step(), step
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_fie_port_equals_reference_bitwise_block(oracle):
    if not _have_ref(oracle):
        pytest.skip("reference sources not present in this container")
    sc = _fie_block_scene()
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for _ in range(sc.steps):
        assert a.step() == b.step()
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_fie_port_matches_golden(oracle):
    g = np.load(os.path.join(GOLDEN, "fie_160.npz"))
    sc = _cantilever(1)
    a = oracle.Solid(sc, "port")
    for k in range(g["x"].shape[0]):
        s = a.step()
        for key in STAT_KEYS:
            assert s[key] == g[key][k], (k, key)
        x, v = a.state()
        np.testing.assert_array_equal(x, g["x"][k])
        np.testing.assert_array_equal(v, g["v"][k])
    q = oracle.Solid(_cantilever(2), "port")
    for k in range(g["q_iters"].shape[0]):
        s = q.step()
        for key in STAT_KEYS:
            assert s[key] == g["q_" + key][k], (k, key)
    xq, vq = q.state()
    np.testing.assert_array_equal(xq, g["xq"])
    np.testing.assert_array_equal(vq, g["vq"])
    assert not np.any(vq)  # quasi-static: v = (1/h)(x_k - x^n) with 1/h = 0


def test_fie_port_matches_golden_block(oracle):
    g = np.load(os.path.join(GOLDEN, "fie_block.npz"))
    sc = _fie_block_scene()
    a = oracle.Solid(sc, "port")
    stats = a.run()
    for key in STAT_KEYS:
        assert [s[key] for s in stats] == list(g[key]), key
    # both Newton exits occur: the iteration cap and |b_k| < nr_abs_eps
    assert min(s["nr_iters"] for s in stats) < sc.nr_max_iter
    x, v = a.state()
    np.testing.assert_array_equal(x, g["x"])
    np.testing.assert_array_equal(v, g["v"])


def test_quasistatic_fie_reaches_equilibrium(oracle):
    """Iterated to convergence, the quasi-static Newton loop stops with
    |m g + f_e(x)| < nr_abs_eps over the free nodes, i.e. at equilibrium.
    E = 1e6 keeps the sag near 0.1 of the beam's length: the truncated
    differentials drop the derivative of R, so the Newton loop converges
    only linearly, and for the softer default beam (sag 0.6) it does not."""
    sc = dataclasses.replace(scenes.cantilever_160(), young=1e6, integrator=2, nr_max_iter=40, nr_abs_eps=1e-7,
                             rel_eps=1e-12, max_iter=4000)
    a = oracle.Solid(sc, "port")
    s = a.step()
    assert s["nr_iters"] < sc.nr_max_iter
    x, _ = a.state()
    a.begin_eval(x)
    f = a.f_e() + a.node_mass() * np.asarray(sc.gravity)
    free = np.ones(sc.num_nodes, bool)
    free[np.asarray(sc.knc_nodes, int)] = False
    assert np.linalg.norm(f[free]) < 1e-7
    assert np.abs(x - sc.rest).max() > 1e-3  # it did sag under gravity
