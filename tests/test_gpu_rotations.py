"""Rotations of the mixed path against the FP64 path on the same positions,
through fem_batch_get_rotations (the batch form of the solid's
fem_solid_get_rotations).

The mixed path evaluates the MSVD in double-float arithmetic (FP64 for
degenerate or nearly isotropic F) and stores R in FP32; the FP64 path runs
the FP64 MSVD. Tolerance: agreement to the FP32 rounding of R,
max |R_mixed - R_fp64| <= 2e-6 (the worst case seen over 1.6 M random F, a
near-degenerate compressed element, was 8e-7); det F is evaluated in FP64
by both paths from the same positions and must be equal bit for bit.
"""
import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

pytestmark = pytest.mark.gpu


def _rotation(rng):
    q = rng.standard_normal(4)
    w, x, y, z = q / np.linalg.norm(q)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _deformed(sc, rng, kind):
    X = sc.rest.copy()
    c = X.mean(axis=0)
    h = sc.h
    if kind == "rest":
        return X
    if kind == "rigid_small_strain":  # a rotation and a 1e-4 smooth strain
        G = np.eye(3) + 1e-4 * rng.standard_normal((3, 3))
        return c + (X - c) @ (_rotation(rng) @ G).T
    if kind == "nearly_isotropic":  # a rotation and a 1e-8 strain: F^T F close to the identity
        G = np.eye(3) + 1e-8 * rng.standard_normal((3, 3))
        return c + (X - c) @ (_rotation(rng) @ G).T
    if kind == "compressed":  # squashed to 30 % in z, sheared
        G = np.array([[1.0, 0.2, 0.1], [0.0, 1.0, 0.3], [0.0, 0.0, 0.3]])
        return c + (X - c) @ G.T
    if kind == "noisy":  # node noise of 0.2 h: some elements nearly degenerate or inverted
        return X + 0.2 * h * rng.standard_normal(X.shape)
    if kind == "twisted":  # rotation angle varying along z
        z = (X[:, 2] - X[:, 2].min()) / max(np.ptp(X[:, 2]), 1e-12)
        ang = 1.5 * z
        ca, sa = np.cos(ang), np.sin(ang)
        d = X - c
        out = X.copy()
        out[:, 0] = c[0] + ca * d[:, 0] - sa * d[:, 1]
        out[:, 1] = c[1] + sa * d[:, 0] + ca * d[:, 1]
        return out
    raise ValueError(kind)


KINDS = ["rest", "rigid_small_strain", "nearly_isotropic", "compressed", "noisy", "twisted"]


def test_mixed_rotations_match_fp64_rotations(fem_lib):
    rng = np.random.default_rng(11)
    scs = [scenes.random_block(rng, lo=4, hi=9, idx=i) for i in range(len(KINDS))]
    xs = [_deformed(sc, rng, k) for sc, k in zip(scs, KINDS)]
    out = {}
    for prec in (fem_lib.FEM_PRECISION_FP64, fem_lib.FEM_PRECISION_MIXED):
        b = fem_lib.Batch(scs, precision=prec, compute_energy=False)
        try:
            for i, x in enumerate(xs):
                b.set_state(i, x=x, v=np.zeros_like(x))
            b.step(1)  # BeginEvaluation at the positions set
            out[prec] = [b.rotations(i) for i in range(len(scs))]
        finally:
            b.close()
    for i, kind in enumerate(KINDS):
        R64, d64 = out[fem_lib.FEM_PRECISION_FP64][i]
        Rm, dm = out[fem_lib.FEM_PRECISION_MIXED][i]
        assert R64.shape == (scs[i].num_tets, 3, 3)
        assert np.all(np.isfinite(R64)) and np.all(np.isfinite(Rm)), kind
        assert np.array_equal(d64, dm), kind
        err = float(np.abs(Rm - R64).max())
        assert err <= 2e-6, (kind, err)
        if kind == "rest":
            assert np.abs(R64 - np.eye(3)).max() < 1e-12
        if kind in ("rigid_small_strain", "nearly_isotropic"):
            # close to the rigid rotation applied (up to the strain and the
            # reference's non-orthonormal R = U V^T)
            assert np.abs(R64 - R64[0]).max() < 1e-3, kind
