"""Failure paths on the GPU, made on the host: no GPU fault, trap or hang.

* A bounded device wait that gives up: the tile product's waits for a tile
  copy get a poll limit of 0 (fem_batch_set_wait_limit), so every wait gives
  up at once while the copy itself completes; the blocks drain their copies
  and fem_batch_synchronize reports FEM_E_TIMEOUT once. The batch then steps
  normally again, and as a fresh batch does.
* NaN injected through the state setters (a NaN initial velocity): the CG
  residual turns NaN and the solid, the batch and the server report
  FEM_E_NAN (ILSS_CG.h:42-46 -- the reference has no such check; its loop
  test is false for NaN and it returns silently).
"""
import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu


def _meshes():
    rng = np.random.default_rng(11)
    return [scenes.random_block(rng, idx=i, dims=d) for i, d in enumerate([(6, 5, 4), (9, 4, 5), (5, 5, 5)])]


def test_tile_copy_wait_gives_up_and_reports_timeout(fem_lib):
    sc = _meshes()
    b = fem_lib.Batch(sc, fem_lib.FEM_PRECISION_MIXED, reorder=False)
    fresh = fem_lib.Batch(sc, fem_lib.FEM_PRECISION_MIXED, reorder=False)
    x0 = [b.state(i) for i in range(len(sc))]
    b.set_wait_limit(0)
    with pytest.raises(fem_lib.FemError) as e:
        b.step(1)
    assert e.value.code == fem_lib.FEM_E_TIMEOUT and "gave up" in str(e.value)
    # reported once (the word is cleared); the aborted step's own statistics
    # are left as they were (its CG loop stopped half way)
    assert fem_lib.load().fem_batch_synchronize(b.h) != fem_lib.FEM_E_TIMEOUT
    # back to the default limit, from the initial states: the same step as a
    # batch that never timed out
    b.set_wait_limit(None)
    for i, (x, v) in enumerate(x0):
        b.set_state(i, x, v)
    b.step(2)
    fresh.step(2)
    for i in range(len(sc)):
        xa, va = b.state(i)
        xb, vb = fresh.state(i)
        assert np.isfinite(xa).all() and np.isfinite(va).all()
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), i
        assert b.stats(i)["cg_iterations"] == fresh.stats(i)["cg_iterations"]


def _nan_velocity(sc):
    """NaN on every node (a single node could sit on the fixed face, whose
    rows the constraint projection zeroes)."""
    return np.full_like(sc.rest, np.nan)


def test_nan_velocity_is_reported_by_the_solid(fem_lib):
    sc = scenes.cantilever_160()
    s = fem_lib.Solid(sc)
    s.set_state(v=_nan_velocity(sc))
    with pytest.raises(fem_lib.FemError) as e:
        s.step(1)
    assert e.value.code == fem_lib.FEM_E_NAN


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_velocity_is_reported_by_the_batch(fem_lib, precision):
    prec = fem_lib.FEM_PRECISION_FP64 if precision == "fp64" else fem_lib.FEM_PRECISION_MIXED
    sc = _meshes()
    b = fem_lib.Batch(sc, prec, reorder=False)
    b.set_state(1, v=_nan_velocity(sc[1]))
    with pytest.raises(fem_lib.FemError) as e:
        b.step(1)
    assert e.value.code == fem_lib.FEM_E_NAN and "mesh 1" in str(e.value)
    # the other meshes stepped as they do alone
    alone = fem_lib.Batch([sc[0]], prec, reorder=False)
    alone.step(1)
    assert np.array_equal(b.state(0)[0], alone.state(0)[0])


def test_nan_velocity_is_reported_by_the_server(fem_lib):
    sc = _meshes()
    srv = fem_lib.Server(fem_lib.FEM_PRECISION_MIXED)
    ids = [srv.add(s) for s in sc]
    assert srv.admit() == len(sc)
    srv.set_state(ids[2], v=_nan_velocity(sc[2]))
    for i in ids:
        srv.submit(i, tag=100 + i)
    done = {c["scene"]: c for c in srv.drain()}
    assert done[ids[2]]["status"] == fem_lib.FEM_E_NAN
    assert done[ids[0]]["status"] == fem_lib.FEM_OK and done[ids[1]]["status"] == fem_lib.FEM_OK
