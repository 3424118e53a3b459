"""Run-time parameter changes (fem_solid_set_params, the Solid3D::
SetParamsExtra seam) and checkpoint/resume of the DAPD state, on the FP64
solid through the C ABI.

A solid whose parameters change between steps must step exactly as a solid
created with the new parameters and given the same state (bit-identical:
both are the same FP64 kernels on the same data), and a DAPD run resumed
from a checkpoint of (x, v, previous positions, directions of collapse) must
continue bit for bit as the uninterrupted run.
"""
import dataclasses

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu


def _same(a, b):
    xa, va = a.state()
    xb, vb = b.state()
    return np.array_equal(xa, xb) and np.array_equal(va, vb)


def _restart_like(fem_lib, sc, src):
    """A fresh solid of scene `sc` given the state of solid `src`."""
    x, v = src.state()
    fresh = fem_lib.Solid(sc)
    fresh.set_state(x, v)
    return fresh


def test_tolerances_gravity_damping_and_dt_change_between_steps(fem_lib):
    sc = scenes.large_block(n=6)
    s = fem_lib.Solid(sc)
    s.step(3)
    sc2 = dataclasses.replace(sc, rel_eps=1e-9, max_iter=300, gravity=(0.5, 0.0, -9.81), damping_ratio=0.3,
                              dt=1.0 / 120.0)
    s.set_params(fem_lib.params_for(sc2))
    ref = _restart_like(fem_lib, sc2, s)
    for _ in range(4):
        a, b = s.step(1), ref.step(1)
        assert a["cg_iterations"] == b["cg_iterations"]
    assert _same(s, ref)
    got = s.get_params()
    assert got.ls_rel_epsilon == 1e-9 and got.ls_max_iter == 300 and got.gravity[0] == 0.5


def test_young_modulus_change_rebakes_every_element_from_the_scalar(fem_lib):
    sc = scenes.large_block(n=6)  # per-element E and nu at creation
    s = fem_lib.Solid(sc)
    s.step(2)
    sc2 = dataclasses.replace(sc, young=3e5, poisson=0.33, young_per_elem=None, poisson_per_elem=None)
    s.set_params(fem_lib.params_for(sc2))
    ref = _restart_like(fem_lib, sc2, s)
    s.step(3)
    ref.step(3)
    assert _same(s, ref)


@pytest.mark.parametrize("change", ["material", "rotation", "solver", "integrator"])
def test_method_switches_between_steps(fem_lib, change):
    sc = scenes.compressed_cube(n=5, steps=20, ratio=0.5)
    kw = {"material": {"material": 1}, "rotation": {"rotation": 1}, "solver": {"ls_solver": 1},
          "integrator": {"integrator": 1}}[change]
    s = fem_lib.Solid(sc)
    s.step(4)
    sc2 = dataclasses.replace(sc, **kw)
    s.set_params(fem_lib.params_for(sc2))
    ref = _restart_like(fem_lib, sc2, s)
    ref.step_index = s.step_index
    s.step(4)
    ref.step(4)
    assert _same(s, ref)


def test_set_params_rejects_bad_values(fem_lib):
    sc = scenes.cantilever_160()
    s = fem_lib.Solid(sc)
    p = fem_lib.params_for(sc)
    p.precision = fem_lib.FEM_PRECISION_MIXED
    with pytest.raises(fem_lib.FemError) as e:
        s.set_params(p)
    assert e.value.code == fem_lib.FEM_E_ARG
    p = fem_lib.params_for(sc)
    p.fixed_dt = 0.0
    with pytest.raises(fem_lib.FemError):
        s.set_params(p)
    assert s.get_params().fixed_dt == sc.dt  # unchanged


def test_dapd_run_resumes_bit_for_bit_from_a_checkpoint(fem_lib):
    # the sheared crush of 10 cm cubes: its elements start to collapse at
    # step 23 and take DAPD's offset rotation, which needs each element's
    # direction of collapse (on 1 cm cubes that rotation is I either way)
    sc = scenes.sheared_crush()
    whole = fem_lib.Solid(sc)
    whole.step(28)
    first = fem_lib.Solid(sc)
    first.step(24)
    x, v = first.state()
    prev_x, doc = first.dapd_state()
    assert (doc[:, 0] <= doc[:, 1]).sum() >= 5  # elements hold a direction of collapse
    resumed = fem_lib.Solid(sc)
    resumed.set_state(x, v)
    resumed.set_dapd_state(prev_x, doc)
    resumed.step_index = 24  # the driven face's schedule continues
    resumed.step(4)
    assert _same(whole, resumed)
    # without the DAPD state the resumed run differs (the previous positions
    # reset to x and the directions of collapse are lost)
    naive = fem_lib.Solid(sc)
    naive.set_state(x, v)
    naive.step_index = 24
    naive.step(4)
    assert not _same(whole, naive)


def test_dapd_state_rejects_malformed_directions(fem_lib):
    sc = dataclasses.replace(scenes.compressed_cube(n=3, steps=5, ratio=0.5), rotation=1)
    s = fem_lib.Solid(sc)
    doc = np.zeros((sc.num_tets, 2), np.uint8)
    doc[0] = (2, 1)
    with pytest.raises(fem_lib.FemError) as e:
        s.set_dapd_state(doc=doc)
    assert e.value.code == fem_lib.FEM_E_ARG
    plain = fem_lib.Solid(scenes.compressed_cube(n=3, steps=5, ratio=0.5))
    with pytest.raises(fem_lib.FemError):
        plain.dapd_state()


# ---- fem_batch_set_params: one solid of an aggregate changes its parameters

def _batch_fresh_like(fem_lib, scs, src, precision):
    """A fresh batch of scenes `scs` given the states of batch `src`."""
    fresh = fem_lib.Batch(scs, precision=precision, chunk_nodes=256)
    for i in range(len(scs)):
        x, v = src.state(i)
        fresh.set_state(i, x, v)
    fresh.step_index = src.step_index
    return fresh


def _batch_same(a, b, i):
    xa, va = a.state(i)
    xb, vb = b.state(i)
    return np.array_equal(xa, xb) and np.array_equal(va, vb)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("change", ["scalars", "young", "material", "rotation", "solver", "integrator"])
def test_batch_set_params_equals_a_batch_built_with_them(fem_lib, precision, change):
    """A mesh of a batch whose parameters change between steps steps as in a
    batch built with the new parameters and given the same states (the same
    bits), in either precision; the other mesh is untouched by the change."""
    other = scenes.cantilever_160()
    sc = scenes.large_block(n=5)  # per-element E and nu at creation
    kw = {"scalars": dict(rel_eps=1e-8, max_iter=300, gravity=(0.5, 0.0, -9.81), damping_ratio=0.3, dt=1.0 / 120.0,
                          density=1500.0),
          "young": dict(young=3e5, poisson=0.33, young_per_elem=None, poisson_per_elem=None),
          "material": dict(material=1),
          "rotation": dict(rotation=1),
          "solver": dict(ls_solver=1),
          "integrator": dict(integrator=1)}[change]
    sc2 = dataclasses.replace(sc, **kw)
    bt = fem_lib.Batch([other, sc], precision=precision, chunk_nodes=256)
    bt.step(3)
    bt.set_params(1, fem_lib.params_for(sc2, precision))
    ref = _batch_fresh_like(fem_lib, [other, sc2], bt, precision)
    bt.step(3)
    ref.step(3)
    assert _batch_same(bt, ref, 1) and _batch_same(bt, ref, 0)
    assert bt.stats(1)["status"] == 0
    got = bt.get_params(1)
    want = fem_lib.params_for(sc2, precision)
    assert (got.material, got.rotation, got.ls_solver, got.integrator) == \
        (want.material, want.rotation, want.ls_solver, want.integrator)
    assert got.fixed_dt == want.fixed_dt and got.young_modulus == want.young_modulus


def test_mixed_batch_refuses_a_return_to_per_element_data(fem_lib):
    """On the mixed path a mesh built with per-element E, nu whose data were
    re-baked for a P-K material cannot go back to C_WRP without new scalar
    values; with them it can."""
    sc = scenes.large_block(n=4)
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, chunk_nodes=256)
    bt.set_params(0, fem_lib.params_for(dataclasses.replace(sc, material=1), fem_lib.FEM_PRECISION_MIXED))
    bt.step(1)
    with pytest.raises(fem_lib.FemError) as e:
        bt.set_params(0, fem_lib.params_for(sc, fem_lib.FEM_PRECISION_MIXED))
    assert e.value.code == fem_lib.FEM_E_ARG
    bt.set_params(0, fem_lib.params_for(dataclasses.replace(sc, young=2e5), fem_lib.FEM_PRECISION_MIXED))
    bt.step(1)
    assert bt.stats(0)["status"] == 0
