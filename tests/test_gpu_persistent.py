"""The persistent CG loop of the mixed path (fem_batch_options.persistent_loop:
one cooperative kernel per launch, the phases of an iteration separated by
bounded grid barriers) against the four-kernel CUDA-graph loop: the same
device code in the same order per value, so the same bits -- for whole
steps, for steps split into slices over launches with masks, through the
server, and with refreshes of the residual -- and a grid barrier that gives
up is reported as FEM_E_TIMEOUT (made on the host: no barrier is broken)."""
import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu


def _meshes(n=5, seed=17):
    rng = np.random.default_rng(seed)
    return [scenes.random_block(rng, lo=3, hi=12, idx=i) for i in range(n)]


def _same(a, b, n):
    for i in range(n):
        xa, va = a.state(i)
        xb, vb = b.state(i)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), i
        assert a.stats(i)["cg_iterations"] == b.stats(i)["cg_iterations"], i


@pytest.mark.parametrize("refresh_every", [None, 7])
def test_persistent_loop_gives_the_graph_loop_bits(fem_lib, refresh_every):
    scs = _meshes()
    g = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, refresh_every=refresh_every)
    p = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, refresh_every=refresh_every, persistent_loop=True)
    for _ in range(4):
        g.step(1)
        p.step(1)
        _same(g, p, len(scs))
    assert all(p.stats(i)["cg_iterations"] > 10 for i in range(len(scs)))


def test_persistent_loop_slices_and_masks(fem_lib):
    scs = _meshes(4, seed=23)
    whole = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED)
    sliced = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, persistent_loop=True)
    sliced.set_slice(7)
    for k in range(3):
        # mesh k % 4 sits the step out in both
        mask = np.ones(len(scs), np.uint8)
        mask[k % len(scs)] = 0
        whole.set_active(mask)
        whole.step(1)
        sliced.set_active(mask)
        sliced.step(1)
        launches = 1
        while True:
            f = sliced.finished()
            if not (f == 2).any():
                break
            sliced.set_active(np.where(f == 2, 2, 0).astype(np.uint8))
            sliced.step(1)
            launches += 1
        assert launches > 1
    _same(whole, sliced, len(scs))


def test_persistent_loop_through_the_server(fem_lib):
    pool = _meshes(6, seed=29)
    a = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED, shard_max_scenes=3)
    b = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED, shard_max_scenes=3, persistent_loop=True)
    for srv in (a, b):
        ids = [srv.add(sc) for sc in pool]
        srv.admit()
        for wave, chosen in enumerate((ids, ids[0::2], ids[1::2])):
            for i in chosen:
                srv.submit(i, tag=10 * wave + i)
            srv.pump()
        srv.drain()
    for i in range(len(pool)):
        xa, va = a.state(i)
        xb, vb = b.state(i)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), i


def test_persistent_loop_reports_a_copy_wait_that_gives_up(fem_lib):
    scs = _meshes(3, seed=37)
    p = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, persistent_loop=True)
    fresh = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, persistent_loop=True)
    x0 = [p.state(i) for i in range(len(scs))]
    p.set_wait_limit(0)
    with pytest.raises(fem_lib.FemError) as e:
        p.step(1)
    assert e.value.code == fem_lib.FEM_E_TIMEOUT
    p.set_wait_limit(None)
    for i, (x, v) in enumerate(x0):
        p.set_state(i, x, v)
    p.step(2)
    fresh.step(2)
    _same(p, fresh, len(scs))


def test_persistent_loop_options_are_checked(fem_lib):
    sc = _meshes(1)
    for kw in ({"precision": fem_lib.FEM_PRECISION_FP64}, {"tile_elems": 128}):
        with pytest.raises(fem_lib.FemError) as e:
            fem_lib.Batch(sc, persistent_loop=True, **kw)
        assert e.value.code == fem_lib.FEM_E_ARG


def test_persistent_loop_streams_tiles_beyond_the_resident_capacity(fem_lib):
    """Running tiles beyond what the blocks can keep resident (two per block)
    go through the streaming form of the persistent kernel (a bulk copy per
    tile and iteration): the same bits as the graph loop."""
    rng = np.random.default_rng(41)
    scs = [scenes.random_block(rng, idx=i, dims=(40, 30, 30)) for i in range(2)]  # 2 x 180,000 tets
    g = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, compute_energy=False)
    p = fem_lib.Batch(scs, fem_lib.FEM_PRECISION_MIXED, compute_energy=False, persistent_loop=True)
    assert g.info()["tiles"] > 1000
    g.step(1)
    p.step(1)
    _same(g, p, len(scs))
