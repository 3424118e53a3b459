"""Oracle pinning for the multi-solid Newton lock-step (CPU): the
restatement's NR_Init / NR_PreStep / NR_MidStep / NR_PostStep / NR_End and
the aggregate's loop over them (oracle/fem_oracle.c, orc_multi_lock_step)
against the same phases restated around the reference's own element set,
CG and MINRES (oracle/ref_harness.cpp, LeafDSH_Solid3D_FEM.cpp:2824-3039,
SS_AggregateDSH_Basic.cpp:229-300), bit for bit.

Every solid of the aggregate runs the largest nr_max_iter of the set, with
the dt the aggregate passes; NR_PreStep resets the iterate to x^n each
iteration, so the lock-step differs from Step_FullyImplicitEuler_dx (a
property pinned below).
"""
import dataclasses
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes


def lock_scenes():
    from test_oracle_fie import _fie_block_scene
    cant = dataclasses.replace(scenes.cantilever_160(), nr_max_iter=2)
    block = dataclasses.replace(_fie_block_scene(), integrator=0, nr_max_iter=3)
    crushed = dataclasses.replace(scenes.compressed_cube(n=4, steps=10, ratio=0.4), rotation=1, material=1,
                                  ls_solver=1)
    return [cant, block, crushed]


def _run(oracle, kind, steps, dt):
    solids = [oracle.Solid(sc, kind) for sc in lock_scenes()]
    stats = []
    for _ in range(steps):
        oracle.multi_lock_step(solids, dt)
        stats.append([(s.last_stats()["potential_energy"], s.lock_stats()) for s in solids])
    return solids, stats


def test_lock_step_port_equals_reference_bitwise(oracle):
    if not os.path.exists(oracle.REF_DBL_SO):
        pytest.skip("reference sources not present in this container")
    dt = 1.0 / 60.0
    a, sa = _run(oracle, "port", 8, dt)
    b, sb = _run(oracle, "ref_dbl", 8, dt)
    assert sa == sb
    for p, q in zip(a, b):
        xa, va = p.state()
        xb, vb = q.state()
        assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    # NR_PreStep resets m_NR_nr_k every iteration, so it reads 1 after any
    # lock-step, whatever the iteration count
    assert all(st[1]["nr_iters"] == 1 for st in sa[-1])


def test_lock_step_phases_called_one_by_one_equal_the_loop(oracle):
    dt = 1.0 / 60.0
    loop, _ = _run(oracle, "port", 3, dt)
    solids = [oracle.Solid(sc, "port") for sc in lock_scenes()]
    for _ in range(3):
        for s in solids:
            if s.scene.knc_schedule is not None:
                s.set_knc_targets_at(s.step_index)
            s.step_index += 1
        for s in solids:
            s.nr_phase("init", dt)
        for _ in range(3):
            for s in solids:
                s.nr_phase("prestep", dt)
                s.nr_phase("midstep", dt)
            for s in solids:
                s.nr_phase("poststep", dt)
        for s in solids:
            s.nr_phase("end", dt)
    for p, q in zip(loop, solids):
        assert np.array_equal(p.state()[0], q.state()[0]) and np.array_equal(p.state()[1], q.state()[1])


def test_a_single_lock_step_iteration_is_one_fie_newton_iteration(oracle):
    """With one NR iteration the lock-step is the first Newton iteration of
    Step_FullyImplicitEuler_dx (same b, warm start and solve); with more it
    differs, because NR_PreStep restarts every iteration from x^n."""
    sc = dataclasses.replace(scenes.cantilever_160(), integrator=1, nr_max_iter=1, nr_abs_eps=0.0)
    fie = oracle.Solid(sc, "port")
    lock = oracle.Solid(sc, "port")
    fie.step()
    oracle.multi_lock_step([lock], sc.dt)
    assert np.array_equal(fie.state()[0], lock.state()[0]) and np.array_equal(fie.state()[1], lock.state()[1])
    sc3 = dataclasses.replace(sc, nr_max_iter=3)
    fie3 = oracle.Solid(sc3, "port")
    lock3 = oracle.Solid(sc3, "port")
    fie3.step()
    oracle.multi_lock_step([lock3], sc.dt)
    assert not np.array_equal(fie3.state()[0], lock3.state()[0])
