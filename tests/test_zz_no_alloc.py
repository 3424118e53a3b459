"""fem_solid_apply_A_noalloc (static device scratch) against fem_solid_apply_A,
through the C ABI. Tolerance: the FP64 bar of the other GPU tests, rel-L2
<= 1e-10. Collected last on purpose: it must pass alone in a fresh process and
after every other test in the same process."""
import ctypes as C

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes
from parity_util import rel

pytestmark = pytest.mark.gpu


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _noalloc(lib, h, factor_M, factor_K, d):
    d = np.ascontiguousarray(d, dtype=np.float64)
    q = np.full(d.shape, np.nan)
    rc = lib.fem_solid_apply_A_noalloc(h, factor_M, factor_K, _ptr(d), _ptr(q))
    assert rc == 0, lib.fem_last_error().decode()
    return q


def test_noalloc_apply_A_matches_apply_A_on_two_calls_in_a_row(fem_lib):
    lib = fem_lib.load()
    sc = scenes.large_block(n=12)  # 8640 tets
    s = fem_lib.Solid(sc)
    s.step(2)  # rotations of a deformed state
    rng = np.random.default_rng(17)
    dt = sc.dt
    d1 = rng.standard_normal(sc.rest.shape)
    d2 = rng.standard_normal(sc.rest.shape)
    ref1 = s.apply_A(1.0, dt * dt, d1)
    ref2 = s.apply_A(1.3, 2 * dt * dt, d2)
    q1 = _noalloc(lib, s.h, 1.0, dt * dt, d1)
    q2 = _noalloc(lib, s.h, 1.3, 2 * dt * dt, d2)
    assert rel(q1, ref1) <= 1e-10, rel(q1, ref1)
    assert rel(q2, ref2) <= 1e-10, rel(q2, ref2)
    # the second call's scratch replaced the first's: a smaller solid next
    small = fem_lib.Solid(scenes.cantilever_160())
    small.step(1)
    d3 = rng.standard_normal((small.N, 3))
    ref3 = small.apply_A(1.0, dt * dt, d3)
    q3 = _noalloc(lib, small.h, 1.0, dt * dt, d3)
    assert rel(q3, ref3) <= 1e-10, rel(q3, ref3)


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
