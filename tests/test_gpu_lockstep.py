"""The multi-solid Newton lock-step on the FP64 solid (fem_solid_nr_* and
fem_multi_step, the Leaf's NR_* phases driven as SS_AggregateDSH_Basic::
MultiDSH_Solid3D_Update drives them), through the C ABI, against the
oracle's restatement (pinned bit for bit to the same phases around the
reference's element set and solvers on the CPU).

Three solids step in lock-step -- the cantilever (nr_max_iter 2), the
moving-constraint block (3) and a crushed cube with DAPD rotations, the
C_LCM material and MINRES -- each running 3 NR iterations. Bars: x and v
rel-L2 within max(1e-10, 10 x the oracle's own movement under a 1e-15
change of the initial velocities), capped per scene.
"""

import numpy as np
import pytest

from parity_util import bar_cap, check_bar, perturbed, rel

pytestmark = pytest.mark.gpu
STEPS = 8


def test_multi_step_matches_the_oracle_lock_step(fem_lib, oracle):
    from test_oracle_lockstep import lock_scenes
    scs = lock_scenes()
    dt = scs[0].dt
    gpu = [fem_lib.Solid(sc) for sc in scs]
    orc = [oracle.Solid(sc, "port") for sc in scs]
    noisy = [oracle.Solid(perturbed(sc, 4), "port") for sc in scs]
    for _ in range(STEPS):
        fem_lib.multi_step(gpu, dt, 1)
        oracle.multi_lock_step(orc, dt)
        oracle.multi_lock_step(noisy, dt)
    for sc, g, o, n in zip(scs, gpu, orc, noisy):
        xg, vg = g.state()
        xo, vo = o.state()
        xn, vn = n.state()
        check_bar(f"lock-step {sc.name}", "x", rel(xg, xo), 1e-10, rel(xn, xo), bar_cap(sc))
        check_bar(f"lock-step {sc.name}", "v", rel(vg, vo), 1e-10, rel(vn, vo), bar_cap(sc))
        st = g.stats()
        assert st["nr_iterations"] == 1  # reset by every NR_PreStep, as the Leaf's m_NR_nr_k
        assert abs(st["potential_energy"] - o.last_stats()["potential_energy"]) <= 1e-8 * max(
            abs(o.last_stats()["potential_energy"]), 1e-30)


def test_phases_one_by_one_equal_multi_step(fem_lib):
    """The phases called by the caller (so that contact terms could enter
    between them) give the bits of fem_multi_step."""
    from test_oracle_lockstep import lock_scenes
    scs = lock_scenes()
    dt = scs[0].dt
    a = [fem_lib.Solid(sc) for sc in scs]
    b = [fem_lib.Solid(sc) for sc in scs]
    fem_lib.multi_step(a, dt, 3)
    for _ in range(3):
        for s in b:
            if s.scene.knc_schedule is not None:
                s.set_knc_targets(s.scene.targets_at(s.step_index))
            s.step_index += 1
            s.nr_phase("init", dt)
        for _ in range(3):
            for s in b:
                s.nr_phase("prestep", dt)
                s.nr_phase("midstep", dt)
            for s in b:
                s.nr_phase("poststep", dt)
        for s in b:
            s.nr_phase("end", dt)
    for p, q in zip(a, b):
        xa, va = p.state()
        xb, vb = q.state()
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_phases_need_nr_init_first(fem_lib):
    from risdsdgcfem_thesis_gb300 import scenes
    s = fem_lib.Solid(scenes.cantilever_160())
    with pytest.raises(fem_lib.FemError) as e:
        s.nr_phase("prestep", 1.0 / 60.0)
    assert e.value.code == fem_lib.FEM_E_ARG
    s.nr_phase("init", 1.0 / 60.0)
    with pytest.raises(fem_lib.FemError):
        s.nr_phase("midstep", -1.0)


def test_batch_multi_step_matches_the_oracle_lock_step(fem_lib, oracle):
    """The lock-step over the solids of one FP64 batch (fem_batch_multi_step:
    every phase on all solids at once) against the oracle's restatement;
    the batch sums in another order than the solid, so the floor is the
    oracle's movement under a 1e-13 change of the initial velocities. The
    potential energy is NR_End's, the iterate count reads 1."""
    from test_oracle_lockstep import lock_scenes
    scs = lock_scenes()
    dt = scs[0].dt
    bt = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_FP64)
    orc = [oracle.Solid(sc, "port") for sc in scs]
    noisy = [oracle.Solid(perturbed(sc, 4, eps=1e-13), "port") for sc in scs]
    for _ in range(STEPS):
        bt.multi_step(dt, 1)
        oracle.multi_lock_step(orc, dt)
        oracle.multi_lock_step(noisy, dt)
    for i, (sc, o, n) in enumerate(zip(scs, orc, noisy)):
        xg, vg = bt.state(i)
        xo, vo = o.state()
        xn, vn = n.state()
        check_bar(f"batch lock-step {sc.name}", "x", rel(xg, xo), 1e-10, rel(xn, xo), bar_cap(sc))
        check_bar(f"batch lock-step {sc.name}", "v", rel(vg, vo), 1e-10, rel(vn, vo), bar_cap(sc))
        st = bt.stats(i)
        assert st["nr_iterations"] == 1
        pe = o.last_stats()["potential_energy"]
        assert abs(st["potential_energy"] - pe) <= 1e-8 * max(abs(pe), 1e-30)


def test_batch_phases_one_by_one_equal_multi_step(fem_lib):
    """The batch's phases called by the caller give fem_batch_multi_step's
    bits, and a batch's regular steps go on after a lock-step."""
    from test_oracle_lockstep import lock_scenes
    scs = lock_scenes()
    dt = scs[0].dt
    a = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_FP64)
    b = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_FP64)
    a.multi_step(dt, 3)
    for _ in range(3):
        b.nr_phase("init", dt)
        for _ in range(3):
            b.nr_phase("prestep", dt)
            b.nr_phase("midstep", dt)
            b.nr_phase("poststep", dt)
        b.nr_phase("end", dt)
    for i in range(len(scs)):
        xa, va = a.state(i)
        xb, vb = b.state(i)
        assert np.array_equal(xa, xb) and np.array_equal(va, vb), i
    a.step(2)
    assert all(a.stats(i)["status"] == 0 for i in range(len(scs)))


def test_mixed_batch_multi_step_matches_the_oracle(fem_lib, oracle):
    """The lock-step on the mixed path (its tile blobs take the lock-step's
    factors while it is open): within 1e-5 (x) and 1e-4 (v) of the oracle."""
    from test_oracle_lockstep import lock_scenes
    scs = lock_scenes()
    dt = scs[0].dt
    bt = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_MIXED, chunk_nodes=256)
    orc = [oracle.Solid(sc, "port") for sc in scs]
    for _ in range(STEPS):
        bt.multi_step(dt, 1)
        oracle.multi_lock_step(orc, dt)
    for i, o in enumerate(orc):
        xg, vg = bt.state(i)
        xo, vo = o.state()
        assert rel(xg, xo) <= 1e-5 and rel(vg, vo) <= 1e-4, (i, rel(xg, xo), rel(vg, vo))


def test_batch_phases_keep_their_order(fem_lib):
    from risdsdgcfem_thesis_gb300 import scenes
    bt = fem_lib.Batch([scenes.cantilever_160()], precision=fem_lib.FEM_PRECISION_FP64)
    with pytest.raises(fem_lib.FemError) as e:
        bt.nr_phase("prestep", 1.0 / 60.0)
    assert e.value.code == fem_lib.FEM_E_ARG
    bt.nr_phase("init", 1.0 / 60.0)
    with pytest.raises(fem_lib.FemError) as e:
        bt.step(1)
    assert e.value.code == fem_lib.FEM_E_ARG
    bt.nr_phase("end", 1.0 / 60.0)
    bt.step(1)


def test_batch_lock_step_leaves_out_inactive_solids(fem_lib):
    """The lock-step's phases act on the solids taking part
    (fem_batch_set_active value 1): a solid left out keeps its state, the
    others step as in a batch of their own."""
    from test_oracle_lockstep import lock_scenes
    scs = lock_scenes()
    dt = scs[0].dt
    bt = fem_lib.Batch(scs, precision=fem_lib.FEM_PRECISION_FP64)
    x1, v1 = bt.state(1)
    bt.set_active(np.array([1, 0, 1], np.uint8))
    bt.multi_step(dt, 2)
    xb, vb = bt.state(1)
    assert np.array_equal(xb, x1) and np.array_equal(vb, v1)
    pair = fem_lib.Batch([scs[0], scs[2]], precision=fem_lib.FEM_PRECISION_FP64)
    pair.multi_step(dt, 2)
    for i, j in ((0, 0), (2, 1)):
        xa, va = pair.state(j)
        xg, vg = bt.state(i)
        assert np.array_equal(xa, xg) and np.array_equal(va, vg), i
