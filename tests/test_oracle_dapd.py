"""Oracle pinning for the DAPD rotation (CPU).

ComputeRotations_DAPD (TetrahedronElementSet3.cpp:860-892) with
UpdateDegeneration / ComputeDoC (:477-533, :589-743) and
Compute_R_DAPD_Degenerate (Rotation.cpp:364-495). The restatement
(oracle/fem_oracle.c) is checked against
  * the reference's own element set built with m_RM = eRM_DAPD
    (oracle/ref_harness.cpp, PerElementTES::SetRotation), bit for bit, where
    the reference sources are present, under both integrators;
  * the fixture that build wrote (tests/golden/dapd_cube.npz);
  * the polar rotation of a rotated stretch (a known answer).
The time-of-collapse cubic goes through GSL's gsl_poly_solve_cubic in the
reference; GSL is not part of the reference tree, and both builds here link
the same restatement of its published method (oracle/gsl_poly_cubic.c).
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAT_KEYS = ("iters", "rel_res", "abs_res", "elastic_energy", "potential_energy", "nr_iters", "nr_rel", "nr_abs")


def crushed_cube(integrator):
    """A 6^3-cube block (1,080 tets) crushed to 15 % of its height over 30
    steps: hundreds of elements fall below det F = 0.1 and many invert."""
    return dataclasses.replace(scenes.compressed_cube(n=6, steps=30, ratio=0.15), rotation=1,
                               integrator=integrator)


@pytest.mark.parametrize("integrator", [0, 1])
def test_dapd_port_equals_reference_bitwise(oracle, integrator):
    if not os.path.exists(oracle.REF_DBL_SO):
        pytest.skip("reference sources not present in this container")
    sc = crushed_cube(integrator)
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for step in range(30):
        assert a.step() == b.step(), step
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


@pytest.mark.parametrize("prefix,integrator", [("qie_", 0), ("fie_", 1)])
def test_dapd_port_matches_golden(oracle, prefix, integrator):
    g = np.load(os.path.join(GOLDEN, "dapd_cube.npz"))
    a = oracle.Solid(crushed_cube(integrator), "port")
    stats = [a.step() for _ in range(30)]
    for key in STAT_KEYS:
        assert [s[key] for s in stats] == list(g[prefix + key]), key
    x, v = a.state()
    np.testing.assert_array_equal(x, g[prefix + "x"])
    np.testing.assert_array_equal(v, g[prefix + "v"])
    doc = a.doc()
    np.testing.assert_array_equal(doc, g[prefix + "doc"])
    valid = doc[:, 0] <= doc[:, 1]
    assert valid.sum() > 200                        # collapse directions were found
    assert np.any(doc[valid, 0] == doc[valid, 1])   # vertex-face collapses
    assert a.detF().min() < 0 or integrator == 1    # and inverted elements (QIE run)


def test_dapd_rotation_of_rotated_stretch(oracle):
    """Above the threshold DAPD takes the Newton polar rotation: for
    x = Q S X (Q a rotation, S a symmetric stretch) every element's R is Q
    to within the loose stopping test (|H1 - H0|_F^2 <= 0.01)."""
    rng = np.random.default_rng(3)
    sc = dataclasses.replace(scenes.random_block(rng, dims=(3, 3, 3)), rotation=1)
    q = rng.standard_normal(4)
    w, x, y, z = q / np.linalg.norm(q)
    Q = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    S = np.diag([1.3, 0.9, 1.1])
    a = oracle.Solid(sc, "port")
    a.begin_eval(sc.rest @ (Q @ S).T)
    R = a.rotations()
    assert np.abs(R - Q).max() < 2e-2
    assert np.abs(np.linalg.det(R) - 1).max() < 2e-2
    # the MSVD rotation of the same F is exact to rounding
    m = oracle.Solid(dataclasses.replace(sc, rotation=0), "port")
    m.begin_eval(sc.rest @ (Q @ S).T)
    assert np.abs(m.rotations() - Q).max() < 1e-9


@pytest.mark.parametrize("integrator", [0, 1])
def test_dapd_offset_branch_port_equals_reference_bitwise(oracle, integrator):
    """The sheared crush of 10 cm cubes: large enough elements that DAPD's
    collapse axis passes the reference's absolute area test
    (len^2 > 1e-6f, Rotation.cpp:364-495), so the degenerate elements take
    the offset polar rotation (on the 1 cm cubes of the other cases that
    test fails and R = I). The restatement equals the reference build bit
    for bit over 30 steps, and the offset branch ran."""
    import dataclasses
    from risdsdgcfem_thesis_gb300 import scenes
    if not os.path.exists(oracle.REF_DBL_SO):
        pytest.skip("reference sources not present in this container")
    sc = dataclasses.replace(scenes.sheared_crush(), integrator=integrator)
    a = oracle.Solid(sc, "port")
    b = oracle.Solid(sc, "ref_dbl")
    for k in range(30):
        assert a.step() == b.step(), k
    xa, va = a.state()
    xb, vb = b.state()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    doc, R, detF = a.doc(), a.rotations(), a.detF()
    held = (doc[:, 0] <= doc[:, 1]) & (detF <= np.float32(0.1))
    assert held.sum() > 40
    assert (np.abs(R[held] - np.eye(3)).reshape(-1, 9).max(axis=1) > 1e-6).sum() > 0.9 * held.sum()
