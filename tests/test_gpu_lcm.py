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


def test_batch_rejects_lcm(fem_lib):
    sc = dataclasses.replace(scenes.cantilever_160(), material=1)
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64)
    assert e.value.code == fem_lib.FEM_E_ARG
