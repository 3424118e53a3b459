"""The DAPD rotation on the FP64 solid, through the C ABI, against the
fixture the reference's own element set wrote (tests/golden/dapd_cube.npz)
and the oracle restatement.

The crushed cube is sensitive: the oracle itself moves by up to 8e-9 in x and
7e-8 in v, and one element's direction of collapse can change, under 1e-15
perturbations of the initial positions. The bars are therefore measured in
the test: x within max(1e-10, 10 x the oracle's own spread), v within
max(1e-8, 10 x its spread), directions of collapse equal on all but 1 % of
the elements, CG iterations within max(1 per solve, 2 %) per step.
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


def crushed_cube(integrator):
    return dataclasses.replace(scenes.compressed_cube(n=6, steps=30, ratio=0.15), rotation=1,
                               integrator=integrator)


def _floor(oracle, sc, g, prefix, steps=30):
    fx, fv = 0.0, 0.0
    for seed in (1, 2, 3):
        o = oracle.Solid(sc, "port")
        x0 = sc.rest + 1e-15 * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
        o.set_state(x0, np.zeros_like(x0))
        for _ in range(steps):
            o.step()
        x, v = o.state()
        fx, fv = max(fx, rel(x, g[prefix + "x"])), max(fv, rel(v, g[prefix + "v"]))
    return fx, fv


@pytest.mark.parametrize("prefix,integrator", [("qie_", 0), ("fie_", 1)])
def test_dapd_crushed_cube_matches_reference(fem_lib, oracle, prefix, integrator):
    g = np.load(os.path.join(GOLDEN, "dapd_cube.npz"))
    sc = crushed_cube(integrator)
    fx, fv = _floor(oracle, sc, g, prefix)
    s = fem_lib.Solid(sc)
    for k in range(30):
        st = s.step(1)
        assert st["status"] == 0
        solves = max(1, st["nr_iterations"])
        assert abs(st["cg_iterations"] - int(g[prefix + "iters"][k])) <= max(solves, int(np.ceil(0.02 * st["cg_iterations"]))), k
    x, v = s.state()
    assert rel(x, g[prefix + "x"]) <= max(1e-10, 10 * fx), (rel(x, g[prefix + "x"]), fx)
    assert rel(v, g[prefix + "v"]) <= max(1e-8, 10 * fv), (rel(v, g[prefix + "v"]), fv)
    doc = s.doc()
    assert np.mean(np.any(doc != g[prefix + "doc"], axis=1)) <= 0.01
    assert (doc[:, 0] <= doc[:, 1]).sum() > 200


def test_dapd_rotations_match_oracle(fem_lib, oracle):
    """BeginEvaluation under DAPD on the same previous and current positions
    (elements above and below the threshold, newly degenerate ones taking the
    time-of-collapse path): R within 1e-12 and the same directions of
    collapse, det F equal."""
    rng = np.random.default_rng(8)
    sc = dataclasses.replace(scenes.random_block(rng, dims=(5, 4, 4)), rotation=1)
    x1 = sc.rest.copy()
    zmax = x1[:, 2].max()
    x1[:, 2] *= 0.12 + 0.05 * rng.standard_normal(x1.shape[0]) * (x1[:, 2] / zmax)  # crush, some invert
    # lateral motion too: with a purely vertical path the cubic's leading
    # coefficients vanish and, at this element size (1 cm), the reference's
    # absolute IsZero epsilon (1e-4) rejects the linear fallback as well
    x1 += 0.15 * sc.h * rng.standard_normal(x1.shape)
    g = fem_lib.Solid(sc)
    o = oracle.Solid(sc, "port")
    g.begin_eval(x1)
    o.begin_eval(x1)
    Rg, dg = g.rotations()
    assert np.array_equal(dg, o.detF())
    assert np.abs(Rg - o.rotations()).max() < 1e-12
    assert np.array_equal(g.doc(), o.doc())
    assert (g.doc()[:, 0] <= g.doc()[:, 1]).sum() > 10


def _sheared_crush_evaluation(oracle, sc):
    """The oracle after 26 steps of sc: (x25, x26, v26, the directions of
    collapse before the 27th BeginEvaluation, and the oracle evaluated at
    x26 against x25)."""
    o25, o26 = oracle.Solid(sc, "port"), oracle.Solid(sc, "port")
    for k in range(26):
        if k < 25:
            o25.step()
        o26.step()
    x25, _ = o25.state()
    x26, v26 = o26.state()
    doc_before = o26.doc()
    o26.begin_eval(x26)
    return x25, x26, v26, doc_before, o26


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_dapd_offset_rotations_match_oracle(fem_lib, oracle, precision):
    """DAPD in a batch (FP64 rotations in either precision): the sheared
    crush restored to the oracle's state after 26 steps (positions, the
    previous step's positions, the directions of collapse, through
    fem_batch_set_state / set_dapd_state), next to an MSVD mesh; the step's
    BeginEvaluation gives the oracle's rotations (1e-12; the mixed batch
    stores them in FP32) and directions of collapse, the offset rotation on
    the collapsing elements."""
    sc = scenes.sheared_crush()
    x25, x26, v26, doc_before, o26 = _sheared_crush_evaluation(oracle, sc)
    other = scenes.cantilever_160()
    bt = fem_lib.Batch([other, sc], precision=precision, compute_energy=False)
    bt.set_state(1, x26, v26)
    bt.set_dapd_state(1, x25, doc_before)
    bt.step_index = 26
    bt.step(1)
    R, detF = bt.rotations(1)
    Ro = o26.rotations()
    tol = 1e-12 if precision == 0 else 1e-6
    assert np.abs(R - Ro).max() < tol
    assert np.abs(detF - o26.detF()).max() < 1e-12
    _, doc = bt.dapd_state(1)
    assert np.array_equal(doc, o26.doc())
    held = (doc[:, 0] <= doc[:, 1]) & (o26.detF() <= np.float32(0.1))
    assert held.sum() > 40
    assert (np.abs(Ro[held] - np.eye(3)).reshape(-1, 9).max(axis=1) > 1e-6).sum() > 0.9 * held.sum()


def test_batched_dapd_steps_like_the_solid_and_resumes(fem_lib):
    """A DAPD mesh in an FP64 batch steps as the FP64 solid does before its
    elements collapse (the crushed cube's first 20 steps, 1e-10), and a
    batch run resumed from a checkpoint of (x, v, previous positions,
    directions of collapse) continues bit for bit, through the collapse."""
    sc = crushed_cube(0)
    s = fem_lib.Solid(sc)
    bt = fem_lib.Batch([sc, scenes.cantilever_160()], precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    s.step(20)
    bt.step(20)
    xs, vs = s.state()
    xb, vb = bt.state(0)
    assert rel(xb, xs) < 1e-10 and rel(vb, vs) < 1e-8
    whole = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    whole.step(28)
    first = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    first.step(24)
    x, v = first.state(0)
    px, doc = first.dapd_state(0)
    resumed = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_FP64, compute_energy=False)
    resumed.set_state(0, x, v)
    resumed.set_dapd_state(0, px, doc)
    resumed.step_index = 24
    resumed.step(4)
    xa, va = whole.state(0)
    xr, vr = resumed.state(0)
    assert np.array_equal(xa, xr) and np.array_equal(va, vr)
    assert (whole.dapd_state(0)[1][:, 0] <= whole.dapd_state(0)[1][:, 1]).sum() > 0


def test_mixed_batch_and_server_with_dapd_match_oracle(fem_lib, oracle):
    """The mixed path with a DAPD mesh: within 1e-5 of the FP64 oracle after
    10 steps of a hanging cantilever, in a batch and through the server
    (whose result is the mixed batch's, bit for bit)."""
    sc = dataclasses.replace(scenes.cantilever_160(), rotation=1)
    o = oracle.Solid(sc, "port")
    for _ in range(10):
        o.step()
    xo, vo = o.state()
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
    bt.step(10)
    xb, vb = bt.state(0)
    assert rel(xb, xo) < 1e-5 and rel(vb, vo) < 1e-4
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED)
    sid = srv.add(sc)
    srv.admit()
    for k in range(10):
        srv.submit(sid, k)
    done = srv.drain()
    assert len(done) == 10 and all(c["status"] == 0 for c in done)
    xs, vs = srv.state(sid)
    assert np.array_equal(xs, xb) and np.array_equal(vs, vb)


def test_batch_dapd_state_calls_check_the_mesh(fem_lib):
    bt = fem_lib.Batch([scenes.cantilever_160()], precision=fem_lib.FEM_PRECISION_FP64)
    with pytest.raises(fem_lib.FemError) as e:
        bt.dapd_state(0)
    assert e.value.code == fem_lib.FEM_E_ARG


def test_dapd_offset_rotations_match_oracle(fem_lib, oracle):
    """DAPD's offset branch at the element level: the sheared crush of 10 cm
    cubes (elements large enough for the reference's absolute area test on
    the collapse axis), evaluated at the oracle's positions after 26 steps
    against the previous step's positions and the directions of collapse the
    run had reached, restored through fem_solid_set_dapd_state. Rotations
    within 1e-12 of the oracle's, the same directions of collapse, and the
    offset rotation (not I) on the collapsing elements. (Whole runs of this
    scene are chaotic: the oracle itself moves by ~1e-2 under a 1e-15 input
    change once elements collapse, so they are compared on the CPU only,
    restatement against the reference build, bit for bit.)"""
    sc = scenes.sheared_crush()
    o25, o26 = oracle.Solid(sc, "port"), oracle.Solid(sc, "port")
    for k in range(26):
        if k < 25:
            o25.step()
        o26.step()
    x25, _ = o25.state()
    x26, v26 = o26.state()
    doc_before = o26.doc()
    o26.begin_eval(x26)  # BeginEvaluation(x25, x26), as the next step opens
    g = fem_lib.Solid(sc)
    g.set_state(x26, v26)
    g.set_dapd_state(x25, doc_before)
    g.begin_eval(x26)
    Rg, dg = g.rotations()
    Ro = o26.rotations()
    assert np.array_equal(dg, o26.detF())
    assert np.array_equal(g.doc(), o26.doc())
    assert np.abs(Rg - Ro).max() < 1e-12
    doc = o26.doc()
    held = (doc[:, 0] <= doc[:, 1]) & (o26.detF() <= np.float32(0.1))
    assert held.sum() > 40
    assert (np.abs(Ro[held] - np.eye(3)).reshape(-1, 9).max(axis=1) > 1e-6).sum() > 0.9 * held.sum()
