"""fem_solid_apply_A_noalloc (static device scratch) against fem_solid_apply_A,
through the C ABI. Tolerance: the FP64 bar of the other GPU tests, rel-L2
<= 1e-10. Collected last on purpose: it must pass alone in a fresh process and
after every other test in the same process.

The entry point exists for callers that cannot allocate device memory at the
moment they call it (a fixed-rate loop, a process whose device memory another
allocator holds), so the test also checks that device free memory does not
move across its calls."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes
from risdsdgcfem_thesis_gb300.scenes import Scene, grid_mesh
from parity_util import rel

pytestmark = pytest.mark.gpu

MATERIALS = {"c_wrp": 0, "c_lcm": 1}


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _noalloc(lib, h, factor_M, factor_K, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    q = np.full(d.shape, np.nan)
    rc = lib.fem_solid_apply_A_noalloc(h, factor_M, factor_K, _ptr(d), _ptr(q))
    assert rc == 0, lib.fem_last_error().decode()
    return q


def _solid(fem_lib, sc, material):
    return fem_lib.Solid(dataclasses.replace(sc, material=MATERIALS[material]))


def _free_bytes():
    torch = pytest.importorskip("torch")
    free, _total = torch.cuda.mem_get_info(0)
    return free


@pytest.mark.parametrize("material", sorted(MATERIALS))
def test_noalloc_apply_A_matches_apply_A_on_two_calls_in_a_row(fem_lib, material):
    lib = fem_lib.load()
    sc = scenes.large_block(n=12)  # 8640 tets
    s = _solid(fem_lib, sc, material)
    s.step(2)  # rotations (and, under C_LCM, F) of a deformed state
    rng = np.random.default_rng(17)
    dt = sc.dt
    d1 = rng.standard_normal(sc.rest.shape)
    d2 = rng.standard_normal(sc.rest.shape)
    ref1 = s.apply_A(1.0, dt * dt, d1)
    ref2 = s.apply_A(1.3, 2 * dt * dt, d2)
    free0 = _free_bytes()
    q1 = _noalloc(lib, s.h, 1.0, dt * dt, d1)
    q2 = _noalloc(lib, s.h, 1.3, 2 * dt * dt, d2)
    assert _free_bytes() == free0, "device free memory moved across the no-alloc calls"
    assert rel(q1, ref1) <= 1e-10, rel(q1, ref1)
    assert rel(q2, ref2) <= 1e-10, rel(q2, ref2)
    # the second call's scratch replaced the first's: a smaller solid next
    small = _solid(fem_lib, scenes.cantilever_160(), material)
    small.step(1)
    d3 = rng.standard_normal((small.N, 3))
    ref3 = small.apply_A(1.0, dt * dt, d3)
    q3 = _noalloc(lib, small.h, 1.0, dt * dt, d3)
    assert rel(q3, ref3) <= 1e-10, rel(q3, ref3)


def test_noalloc_apply_A_at_the_size_limit(fem_lib):
    """A 3 x 17 x 257 bar of 65,535 tets (one below the limit) fills the
    static scratch up to its last slot."""
    lib = fem_lib.load()
    a, b, c = 3, 17, 257
    rest, tets, ijk = grid_mesh(a, b, c, 0.01, 0.001, 3)
    assert tets.shape[0] == 65535
    fixed = np.flatnonzero(ijk[:, 2] == 0).astype(np.uint32)
    sc = Scene(name="bar_3x17x257", rest=rest, tets=tets, young=2e5, poisson=0.35, density=1000.0,
               gravity=(0.0, 0.0, -9.81), rel_eps=1e-6, abs_eps=0.0, max_iter=50, steps=1,
               knc_nodes=fixed, knc_targets=rest[fixed].copy(), grid=(a, b, c), h=0.01)
    s = fem_lib.Solid(sc)
    s.step(1)
    rng = np.random.default_rng(5)
    d = rng.standard_normal(sc.rest.shape)
    ref = s.apply_A(1.0, sc.dt * sc.dt, d)
    free0 = _free_bytes()
    q = _noalloc(lib, s.h, 1.0, sc.dt * sc.dt, d)
    q_again = _noalloc(lib, s.h, 1.0, sc.dt * sc.dt, d)
    assert _free_bytes() == free0
    assert rel(q, ref) <= 1e-10, rel(q, ref)
    assert np.array_equal(q, q_again)


def test_noalloc_apply_A_rejects_solids_over_the_limit(fem_lib):
    lib = fem_lib.load()
    sc = scenes.large_block(n=24)  # 69120 tets > 65536
    assert sc.num_tets > 65536
    s = fem_lib.Solid(sc)
    d = np.zeros(sc.rest.shape)
    q = np.zeros(sc.rest.shape)
    rc = lib.fem_solid_apply_A_noalloc(s.h, 1.0, 1e-4, _ptr(d), _ptr(q))
    assert rc == fem_lib.FEM_E_ARG
    assert b"at most 65536" in lib.fem_last_error()
