"""The step-request server (fem_server_*) on the GPU: a scene's result is the
same alone and in the mix under continuous batching (bit-identical to the
scene stepped alone in its own batch with the server's node chunk), admission respects the device-memory
budget, and shards overlap on the device."""
import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu


def _pool(n, seed=31):
    rng = np.random.default_rng(seed)
    return [scenes.random_block(rng, lo=3, hi=9, idx=i) for i in range(n)]


def test_server_results_alone_and_in_the_mix_are_identical(fem_lib):
    pool = _pool(7)
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED, shard_max_scenes=3)
    ids = [srv.add(sc) for sc in pool]
    assert srv.admit() == len(pool)
    st = srv.status()
    assert st["shards"] == 3 and st["resident_scenes"] == len(pool)
    # an uneven, interleaved request stream: requests arrive while shards are busy
    rng = np.random.default_rng(5)
    steps = [0] * len(pool)
    done = []
    for wave in range(6):
        for i in rng.permutation(len(pool))[: rng.integers(2, len(pool) + 1)]:
            srv.submit(ids[i], tag=1000 * wave + int(i))
            steps[i] += 1
        for _ in range(int(rng.integers(0, 3))):
            done += srv.pump()
    done += srv.drain()
    assert len(done) == sum(steps)
    assert all(c["status"] == 0 for c in done)
    assert all(c["latency_us"] > 0 and c["device_us"] > 0 for c in done)
    # requests of one scene complete in submission order
    for i in range(len(pool)):
        tags = [c["tag"] for c in done if c["scene"] == ids[i]]
        assert tags == sorted(tags)
    # the scene alone in a batch with the server's node chunk (256): the
    # chunk size fixes the order of the |r|^2 partial sums
    for i, sc in enumerate(pool):
        alone = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
        its = []
        for _ in range(steps[i]):
            alone.step(1)
            its.append(alone.stats(0)["cg_iterations"])
        xa, va = alone.state(0)
        xs, vs = srv.state(ids[i])
        assert np.array_equal(xa, xs) and np.array_equal(va, vs), i
        served = [c["cg_iterations"] for c in sorted(done, key=lambda c: c["tag"]) if c["scene"] == ids[i]]
        assert served == its, (i, served, its)
        alone.close()
    srv.close()


def test_server_short_slices_give_the_same_results(fem_lib):
    pool = _pool(4, seed=44)
    srv = fem_lib.Server(shard_max_scenes=2, slice_iterations=3)
    ids = [srv.add(sc) for sc in pool]
    srv.admit()
    for rep in range(2):
        for i in ids:
            srv.submit(i, tag=rep)
        srv.pump()
    done = srv.drain()
    assert len(done) == 2 * len(pool) and all(c["status"] == 0 for c in done)
    # the scene alone in a batch with the server's node chunk (256): the
    # chunk size fixes the order of the |r|^2 partial sums
    for i, sc in enumerate(pool):
        alone = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
        alone.step(2)
        xa, va = alone.state(0)
        xs, vs = srv.state(ids[i])
        assert np.array_equal(xa, xs) and np.array_equal(va, vs), i
        alone.close()
    srv.close()


def test_server_admission_respects_the_budget(fem_lib):
    pool = _pool(6, seed=2)
    probe = fem_lib.Server(shard_max_scenes=1)
    probe.add(pool[0])
    probe.add(pool[1])
    assert probe.admit() == 2
    two = probe.status()["device_bytes"]
    probe.close()
    budget = int(two * 1.6)  # room for about three small scenes, not six
    srv = fem_lib.Server(hbm_budget_bytes=budget, shard_max_scenes=1)
    ids = [srv.add(sc) for sc in pool]
    n1 = srv.admit()
    st = srv.status()
    assert 1 <= n1 < len(pool) and st["device_bytes"] <= budget and st["waiting_scenes"] == len(pool) - n1
    resident = srv.resident()
    assert len(resident) == n1
    # smallest scenes first
    assert max(pool[i].num_tets for i in resident) <= min(pool[i].num_tets for i in ids if i not in resident)
    for i in resident:
        srv.submit(i)
    srv.drain()
    for i in resident:
        srv.remove(i)
    assert srv.status()["device_bytes"] == 0
    assert all(srv.scene_info(i)["state"] == "removed" for i in resident)
    n2 = srv.admit()
    assert n2 >= 1 and srv.status()["device_bytes"] <= budget
    assert len(srv.resident()) == n2
    srv.close()


def test_server_shards_overlap_on_the_device(fem_lib):
    pool = _pool(8, seed=9)
    srv = fem_lib.Server(shard_max_scenes=2)
    ids = [srv.add(sc) for sc in pool]
    srv.admit()
    for i in ids:
        srv.submit(i)
    srv.pump()  # launches every shard at once
    assert srv.status()["busy_shards"] >= 2
    done = srv.drain()
    assert len(done) == len(pool) and srv.status()["max_busy_shards"] == 4
    srv.close()


def test_server_scene_parameter_change_equals_the_batch(fem_lib):
    """fem_server_set_params on a resident scene between requests: the
    scene's results are those of a batch whose mesh takes the same change at
    the same point (the same bits); a change of integrator kind is refused."""
    import dataclasses
    sc = scenes.cantilever_160()
    sc2 = dataclasses.replace(sc, gravity=(0.3, 0.0, -9.81), rel_eps=1e-8, damping_ratio=0.2)
    srv = fem_lib.Server(precision=fem_lib.FEM_PRECISION_MIXED)
    sid = srv.add(sc)
    srv.admit()
    for k in range(3):
        srv.submit(sid, k)
    assert len(srv.drain()) == 3
    srv.set_params(sid, fem_lib.params_for(sc2, fem_lib.FEM_PRECISION_MIXED))
    for k in range(3, 6):
        srv.submit(sid, k)
    done = srv.drain()
    assert len(done) == 3 and all(c["status"] == 0 for c in done)
    bt = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False, chunk_nodes=256)
    bt.step(3)
    bt.set_params(0, fem_lib.params_for(sc2, fem_lib.FEM_PRECISION_MIXED))
    bt.step(3)
    xs, vs = srv.state(sid)
    xb, vb = bt.state(0)
    assert np.array_equal(xs, xb) and np.array_equal(vs, vb)
    with pytest.raises(fem_lib.FemError) as e:
        srv.set_params(sid, fem_lib.params_for(dataclasses.replace(sc, integrator=1), fem_lib.FEM_PRECISION_MIXED))
    assert e.value.code == fem_lib.FEM_E_ARG
