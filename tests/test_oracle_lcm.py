"""Oracle pinning for the C_LCM material (CPU): the restatement
(oracle/fem_oracle.c, lcm_f_e_acc / lcm_df_x_acc / lcm_V) against the
reference's element set built with m_MM = eMM_C_LCM (oracle/ref_harness.cpp,
PerElementTES::SetMaterial), bit for bit, where the reference sources are
present, and against the fixture that build wrote (tests/golden/lcm.npz).
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAT_KEYS = ("iters", "rel_res", "abs_res", "elastic_energy", "potential_energy", "nr_iters", "nr_rel", "nr_abs")


def lcm_cases():
    """The cases of tests/golden/make_golden.py (lcm_cases)."""
    from test_oracle_fie import _fie_block_scene
    cant = scenes.cantilever_160()
    return (("qie_", dataclasses.replace(cant, material=1), 60),
            ("fie_", dataclasses.replace(cant, material=1, integrator=1), 20),
            ("block_", dataclasses.replace(_fie_block_scene(), material=1, integrator=0), 12))


@pytest.mark.parametrize("case", [0, 1, 2])
def test_lcm_port_equals_reference_bitwise(oracle, case):
    if not os.path.exists(oracle.REF_DBL_SO):
        pytest.skip("reference sources not present in this container")
    _, sc, steps = lcm_cases()[case]
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for k in range(steps):
        assert a.step() == b.step(), k
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_lcm_port_matches_golden(oracle):
    g = np.load(os.path.join(GOLDEN, "lcm.npz"))
    for prefix, sc, steps in lcm_cases():
        a = oracle.Solid(sc, "port")
        stats = [a.step() for _ in range(steps)]
        for key in STAT_KEYS:
            assert [s[key] for s in stats] == list(g[prefix + key]), (prefix, key)
        x, v = a.state()
        np.testing.assert_array_equal(x, g[prefix + "x"])
        np.testing.assert_array_equal(v, g[prefix + "v"])


def test_lcm_force_is_zero_at_rest_and_rigid(oracle):
    """P(S = I) = 0: no force at rest or under a rigid rotation."""
    sc = dataclasses.replace(scenes.cantilever_160(), material=1)
    a = oracle.Solid(sc, "port")
    a.begin_eval(sc.rest)
    assert np.abs(a.f_e()).max() < 1e-9 and abs(a.V()) < 1e-12
    c, s_ = np.cos(0.7), np.sin(0.7)
    Q = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]])
    a.begin_eval(sc.rest @ Q.T)
    assert np.abs(a.f_e()).max() < 1e-6 * sc.young * sc.h ** 2


def test_all_widened_options_together_bitwise(oracle):
    """C_LCM with the DAPD rotation, the FIE integrator and MINRES on the
    crushed cube: the restatement equals the reference build bit for bit."""
    if not os.path.exists(oracle.REF_DBL_SO):
        pytest.skip("reference sources not present in this container")
    sc = dataclasses.replace(scenes.compressed_cube(n=5, steps=20, ratio=0.2), material=1, rotation=1,
                             integrator=1, ls_solver=1)
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for k in range(20):
        assert a.step() == b.step(), k
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    doc = a.doc()
    assert (doc[:, 0] <= doc[:, 1]).sum() > 0  # the DAPD degenerate branch ran
