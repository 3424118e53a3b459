"""Oracle pinning for the MINRES linear solver (CPU).

ILSS_MINRES::Solve (src/Saphyre2/ns/ILSS_MINRES.h:51-168) selected by the
Leaf's LS_Solve (LeafDSH_Solid3D_FEM.cpp:1136-1154). The restatement
(oracle/fem_oracle.c, minres_solve) is checked against the reference's own
header-only solver driven by the restated Leaf (oracle/ref_harness.cpp,
ls_solve), bit for bit, where the reference sources are present; against the
fixture that build wrote (tests/golden/minres.npz); and against the
mathematics: with tight tolerances MINRES and CG reach the same solution of
the same SPD system.
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAT_KEYS = ("iters", "rel_res", "abs_res", "elastic_energy", "potential_energy", "nr_iters", "nr_rel", "nr_abs")


def minres_cases():
    """The cases of tests/golden/make_golden.py (minres_cases)."""
    from test_oracle_fie import _fie_block_scene
    cant = scenes.cantilever_160()
    return (("qie_", dataclasses.replace(cant, ls_solver=1), 60),
            ("fie_", dataclasses.replace(cant, ls_solver=1, integrator=1), 20),
            ("block_", dataclasses.replace(_fie_block_scene(), ls_solver=1, integrator=0), 12))


@pytest.mark.parametrize("case", [0, 1, 2])
def test_minres_port_equals_reference_bitwise(oracle, case):
    if not os.path.exists(oracle.REF_DBL_SO):
        pytest.skip("reference sources not present in this container")
    _, sc, steps = minres_cases()[case]
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for k in range(steps):
        assert a.step() == b.step(), k
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_minres_port_matches_golden(oracle):
    g = np.load(os.path.join(GOLDEN, "minres.npz"))
    for prefix, sc, steps in minres_cases():
        a = oracle.Solid(sc, "port")
        stats = [a.step() for _ in range(steps)]
        for key in STAT_KEYS:
            assert [s[key] for s in stats] == list(g[prefix + key]), (prefix, key)
        x, v = a.state()
        np.testing.assert_array_equal(x, g[prefix + "x"])
        np.testing.assert_array_equal(v, g[prefix + "v"])


def test_minres_and_cg_agree_at_tight_tolerance(oracle):
    sc = dataclasses.replace(scenes.cantilever_160(), rel_eps=1e-13, max_iter=2000)
    states = []
    for ls in (0, 1):
        a = oracle.Solid(dataclasses.replace(sc, ls_solver=ls), "port")
        for _ in range(5):
            s = a.step()
            assert s["iters"] < sc.max_iter
        states.append(a.state())
    (xc, vc), (xm, vm) = states
    assert np.linalg.norm(xm - xc) / np.linalg.norm(xc) < 1e-11
    assert np.linalg.norm(vm - vc) / np.linalg.norm(vc) < 1e-9
