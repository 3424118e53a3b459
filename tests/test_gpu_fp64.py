"""FP64 drop-in path on the GPU, through the C ABI, against the oracle.

Tolerances (FP64): positions and velocities rel-L2 <= 1e-10 after N steps,
CG iterations within +-1 per step; element-level products rel <= 1e-12.
"""
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes
from parity_util import bar_cap, check_bar

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-10


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_elements_match_golden(fem_lib):
    g = np.load(os.path.join(GOLDEN, "elements_160.npz"))
    sc = scenes.cantilever_160()
    s = fem_lib.Solid(sc)
    s.begin_eval(g["x"])
    R, detF = s.rotations()
    np.testing.assert_allclose(detF, g["detF"], rtol=1e-13, atol=1e-15)
    assert np.abs(R - g["R"]).max() < 1e-12
    # most rotations are bit-identical (rotation.cu is compiled without FMA)
    assert np.mean(np.all(R == g["R"], axis=(1, 2))) > 0.5
    assert rel(s.f_e(), g["f_e"]) < 1e-12
    assert rel(s.df_x(g["dx"]), g["df_x"]) < 1e-12
    assert abs(s.V() - float(g["V"])) < 1e-12 * abs(float(g["V"]))


def test_cantilever_120_steps_matches_reference(fem_lib):
    g = np.load(os.path.join(GOLDEN, "cantilever_160.npz"))
    sc = scenes.cantilever_160()
    s = fem_lib.Solid(sc)
    worst = 0.0
    for k in range(sc.steps):
        st = s.step(1)
        assert abs(st["cg_iterations"] - int(g["iters"][k])) <= 1, (k, st["cg_iterations"], g["iters"][k])
        assert st["status"] == 0
    x, v = s.state()
    ex, ev = rel(x, g["x"][-1]), rel(v, g["v"][-1])
    assert ex <= TOL and ev <= TOL, (ex, ev)
    assert abs(st["elastic_energy"] - g["elastic_energy"][-1]) <= 1e-8 * abs(g["elastic_energy"][-1])
    assert abs(st["potential_energy"] - g["potential_energy"][-1]) <= 1e-8 * abs(g["potential_energy"][-1])


def _perturbed(sc, seed, eps=1e-15):
    import copy
    p = copy.copy(sc)
    v0 = np.zeros_like(sc.rest) if sc.init_vel is None else sc.init_vel
    p.init_vel = v0 + eps * np.abs(sc.rest).max() * np.random.default_rng(seed).standard_normal(sc.rest.shape)
    return p


def _compare_with_port(fem_lib, oracle, sc, steps, tol=TOL, cap=None, assembled=False):
    """GPU vs the oracle restatement over `steps` FixedSteps.

    CG stops on a residual threshold, and on stiff scenes the residual sits on
    a plateau near that threshold: the reference itself then changes its
    iteration count by several when its input moves by 1e-15. The comparison
    is therefore calibrated against the oracle's own noise floor, measured by
    re-running it three times with the initial velocity perturbed by 1e-15
    (relative to the mesh size): the GPU must agree with the oracle within
    max(tol, 10 x that floor) in state and within max(1, 2 x spread + 1) in
    iterations per step."""
    a = fem_lib.Solid(sc)
    a.set_assembled(assembled)
    b = oracle.Solid(sc, "port")
    noisy = [oracle.Solid(_perturbed(sc, seed), "port") for seed in (1, 2, 3)]
    it_gpu, it_orc = [], []
    it_noise = [[] for _ in noisy]
    for k in range(steps):
        it_gpu.append(a.step(1)["cg_iterations"])
        it_orc.append(b.step()["iters"])
        for c, lst in zip(noisy, it_noise):
            lst.append(c.step()["iters"])
    xa, va = a.state()
    xb, vb = b.state()
    noise_x = noise_v = 0.0
    for c in noisy:
        xc, vc = c.state()
        noise_x, noise_v = max(noise_x, rel(xc, xb)), max(noise_v, rel(vc, vb))
    spread = max(abs(i - j) for lst in it_noise for i, j in zip(it_orc, lst))
    ex, ev = rel(xa, xb), rel(va, vb)
    cap = bar_cap(sc) if cap is None else cap
    check_bar(sc.name, "x", ex, tol, noise_x, cap)
    check_bar(sc.name, "v", ev, tol, noise_v, cap)
    worst_it = max(abs(i - j) for i, j in zip(it_gpu, it_orc))
    assert worst_it <= max(1, 2 * spread + 1), (worst_it, spread, it_gpu, it_orc)
    return ex, ev


def test_per_element_material_damped_driven(fem_lib, oracle):
    rng = np.random.default_rng(5)
    sc = scenes.random_block(rng, dims=(5, 3, 4))
    T = sc.num_tets
    sc.young_per_elem = np.exp(rng.uniform(np.log(5e4), np.log(5e5), T))
    sc.poisson_per_elem = rng.uniform(0.25, 0.45, T)
    sc.damping_ratio = 1.0
    sc.init_vel = rng.standard_normal(sc.rest.shape) * 0.1
    base = sc.knc_targets.copy()
    sc.knc_schedule = lambda k: base + np.array([0.0, 0.0, 0.001 * (k + 1)])
    _compare_with_port(fem_lib, oracle, sc, 20)


def test_block_with_initial_velocity(fem_lib, oracle):
    sc = scenes.large_block(n=10)
    _compare_with_port(fem_lib, oracle, sc, 10)


def test_block_on_the_assembled_stiffness(fem_lib, oracle):
    """A block above the one-cluster CG's 8,192 tets (13,720) whose CG takes
    K u from the assembled 3x3-block stiffness (fem_solid_set_assembled),
    rebuilt at every evaluation; within the oracle's bar after 4 steps."""
    sc = scenes.large_block(n=14)
    assert sc.num_tets > 8192
    _compare_with_port(fem_lib, oracle, sc, 4, assembled=True)


def test_assembled_toggle_between_steps(fem_lib):
    """fem_solid_set_assembled switched on and off between steps (its first
    switch-on assembles on the current rotations): a 13,720-tet block stepped
    matrix-free, assembled, then matrix-free again stays as close to the
    same block stepped matrix-free throughout as the oracle stays to itself
    under 1e-15 perturbations on this block (x about 1e-9, v about 2e-6,
    the CG's residual plateau); MINRES the same."""
    for solver in (fem_lib.FEM_LS_CG, fem_lib.FEM_LS_MINRES):
        sc = scenes.large_block(n=14)
        sc.ls_solver = solver
        ref, sw = fem_lib.Solid(sc), fem_lib.Solid(sc)
        for on in (False, True, False, True):
            sw.set_assembled(on)
            ref.step(2)
            sw.step(2)
        xr, vr = ref.state()
        xs, vs = sw.state()
        assert rel(xs, xr) < 1e-8 and rel(vs, vr) < 5e-6, (solver, rel(xs, xr), rel(vs, vr))


def test_compression_with_inversions(fem_lib, oracle):
    sc = scenes.compressed_cube(n=6, steps=30, ratio=0.2)
    _compare_with_port(fem_lib, oracle, sc, 30, tol=1e-9)


def test_free_floating_no_constraints(fem_lib, oracle):
    rng = np.random.default_rng(9)
    sc = scenes.random_block(rng, dims=(3, 3, 3))
    sc.knc_nodes = np.zeros(0, np.uint32)
    sc.knc_targets = np.zeros((0, 3))
    sc.init_vel = rng.standard_normal(sc.rest.shape) * 0.05
    _compare_with_port(fem_lib, oracle, sc, 10)


def test_single_tet(fem_lib, oracle):
    rest = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0, 0, 0.1]], float)
    sc = scenes.Scene(name="one", rest=rest, tets=np.array([[0, 1, 2, 3]], np.uint32), gravity=(0, 0, -9.81),
                      knc_nodes=np.array([0], np.uint32), knc_targets=rest[:1].copy(), rel_eps=1e-10,
                      max_iter=100, steps=5)
    # a lone tet hanging from one node stays close to its rest shape, where
    # F^T F is nearly isotropic and the MSVD's discrete choices (eigenvalue
    # order, flip) turn under 1e-15 changes of the input: the oracle itself
    # moves by ~1e-6 there, so the bar may reach 1e-4 (the GPU matches it to
    # ~1e-16, its rotations being bit-identical)
    _compare_with_port(fem_lib, oracle, sc, 5, cap=1e-4)


def test_host_roundtrip_matches_device_steps(fem_lib):
    sc = scenes.cantilever_160()
    a = fem_lib.Solid(sc)
    b = fem_lib.Solid(sc)
    a.step(3)
    import ctypes as C
    x = np.empty((sc.num_nodes, 3)); v = np.empty((sc.num_nodes, 3))
    st = fem_lib.FemStepStats()
    fem_lib.check(b.lib.fem_solid_step_host(b.h, None, None, 3, x.ctypes.data_as(C.POINTER(C.c_double)),
                                            v.ctypes.data_as(C.POINTER(C.c_double)), C.byref(st)))
    xa, va = a.state()
    assert np.array_equal(xa, x) and np.array_equal(va, v)


def test_deterministic_repeat(fem_lib):
    sc = scenes.large_block(n=8)
    outs = []
    for _ in range(2):
        s = fem_lib.Solid(sc)
        s.step(5)
        outs.append(s.state())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_operator_symmetry_full_size(fem_lib):
    """At the full 60^3 size: A is symmetric on the free rows (d^T A e = e^T A d)
    and the solve reaches the requested relative residual."""
    sc = scenes.large_block(n=60)
    s = fem_lib.Solid(sc)
    st = s.step(1)
    assert st["status"] == 0 and st["rel_residual"] <= sc.rel_eps * 1.0001
    rng = np.random.default_rng(0)
    d = rng.standard_normal(sc.rest.shape)
    e = rng.standard_normal(sc.rest.shape)
    fixed = np.zeros(sc.num_nodes, bool); fixed[sc.knc_nodes] = True
    d[fixed] = 0; e[fixed] = 0
    dt = sc.dt
    Ad = s.apply_A(1.0, dt * dt, d)
    Ae = s.apply_A(1.0, dt * dt, e)
    lhs, rhs = float(np.sum(e * Ad)), float(np.sum(d * Ae))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
    assert float(np.sum(d * Ad)) > 0
