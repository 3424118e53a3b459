"""Synthetic tetrahedral scenes for the corotational FEM step.

The reference's own meshes (the armadillo/horse/box scenes of its example
player) are not available, so every workload here is a seeded grid of cubes,
each cube split into 5 tetrahedra. Cube (i, j, k) uses one of two mirror
splits chosen by the parity of i + j + k, so neighbouring cubes share face
diagonals and the mesh is conforming. Nodes are numbered x-fastest:
node(i, j, k) = i + (a + 1) * (j + (b + 1) * k).

A scene is the input of the reference's Solid3D creation path
(bs/Solid3D.h:27-158): rest positions, tets, material (E, nu, rho, damping
ratio), gravity, fixed or driven nodes (KinematicNodeConstraintSet3
position constraints), and solver settings (fixed dt, CG tolerances).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Callable, List, Optional

import numpy as np

# Corner numbering of a unit cube: bit 0 -> x, bit 1 -> y, bit 2 -> z.
_CUBE = np.array([[(c >> 0) & 1, (c >> 1) & 1, (c >> 2) & 1] for c in range(8)], dtype=np.int64)
# Split A: centre tet (0,3,5,6); split B: centre tet (1,2,4,7).
_SPLIT_A = [(0, 1, 3, 5), (0, 2, 6, 3), (0, 4, 5, 6), (3, 5, 6, 7), (0, 3, 6, 5)]
_SPLIT_B = [(1, 0, 4, 2), (1, 3, 2, 7), (1, 5, 7, 4), (2, 4, 7, 6), (1, 2, 4, 7)]


def _oriented(split):
    """Reorder each tet so det(r1-r0, r2-r0, r3-r0) > 0 on the unit cube."""
    out = []
    for t in split:
        p = _CUBE[list(t)].astype(np.float64)
        d = np.linalg.det(np.stack([p[1] - p[0], p[2] - p[0], p[3] - p[0]], axis=1))
        assert abs(d) > 0.5 / 6
        out.append(t if d > 0 else (t[0], t[2], t[1], t[3]))
    return out


_SPLIT_A = _oriented(_SPLIT_A)
_SPLIT_B = _oriented(_SPLIT_B)


@dataclasses.dataclass
class Scene:
    """One solid: mesh, material, constraints and solver settings."""

    name: str
    rest: np.ndarray            # (N, 3) float64, AoS
    tets: np.ndarray            # (T, 4) uint32
    young: float = 1e5
    poisson: float = 0.3
    young_per_elem: Optional[np.ndarray] = None   # (T,) float64 or None
    poisson_per_elem: Optional[np.ndarray] = None
    density: float = 1000.0
    damping_ratio: float = 0.0
    gravity: tuple = (0.0, 0.0, 0.0)
    dt: float = 1.0 / 60.0
    rel_eps: float = 1e-6
    abs_eps: float = 0.0
    max_iter: int = 500
    steps: int = 60
    knc_nodes: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint32))
    knc_targets: Optional[np.ndarray] = None       # (K, 3) initial targets
    # Optional per-step driver: step index (0-based, before the step) ->
    # (K, 3) targets for the constraints.
    knc_schedule: Optional[Callable[[int], np.ndarray]] = None
    init_vel: Optional[np.ndarray] = None          # (N, 3)
    grid: tuple = (0, 0, 0)
    h: float = 0.0
    # Time integrator (enum fem_integrator: 0 QIE_V, 1 FIE_DX, 2 FIE_DX
    # quasi-static) and the Newton settings of the FIE integrators.
    integrator: int = 0
    nr_max_iter: int = 3
    nr_abs_eps: float = 1e-6
    # Rotation method (enum fem_rotation: 0 MSVD, 1 DAPD) and the DAPD
    # degeneration threshold on det F and offset factors (the reference's
    # defaults: 0.1f, 1, 0, 2).
    # Linear solver of the step (enum fem_ls_solver: 0 CG, 1 MINRES).
    ls_solver: int = 0
    # Material model (enum fem_material: 0 C_WRP, 1 C_LCM, 2 C_LCMH, 3 C_CCM)
    # and C_LCMH's blend radius (the reference's m_ECIE_k_factor, default 1).
    material: int = 0
    ecie_k_factor: float = 1.0
    rotation: int = 0
    dapd_threshold: float = float(np.float32(0.1))
    dapd_L: float = 1.0
    dapd_NL: float = 0.0
    dapd_exponent: float = 2.0

    @property
    def num_nodes(self) -> int:
        return int(self.rest.shape[0])

    @property
    def num_tets(self) -> int:
        return int(self.tets.shape[0])

    def targets_at(self, step: int) -> np.ndarray:
        if self.knc_schedule is not None:
            return np.ascontiguousarray(self.knc_schedule(step), dtype=np.float64)
        return self.knc_targets


def grid_mesh(a: int, b: int, c: int, h: float, jitter: float, seed: int):
    """(rest, tets, ijk) for an a x b x c grid of cubes of edge h, 5 tets each,
    every node coordinate jittered uniformly in [-jitter, jitter]."""
    nx, ny, nz = a + 1, b + 1, c + 1
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ijk = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.int64)
    rng = np.random.default_rng(seed)
    rest = ijk.astype(np.float64) * h
    if jitter > 0:
        rest = rest + rng.uniform(-jitter, jitter, size=rest.shape)

    ci, cj, ck = np.meshgrid(np.arange(a), np.arange(b), np.arange(c), indexing="ij")
    cubes = np.stack([ci.ravel(), cj.ravel(), ck.ravel()], axis=1)
    # cube order: x fastest, then y, then z (spatially coherent)
    order = np.lexsort((cubes[:, 0], cubes[:, 1], cubes[:, 2]))
    cubes = cubes[order]
    corner_nodes = np.empty((cubes.shape[0], 8), np.int64)
    for cnr in range(8):
        ii = cubes[:, 0] + _CUBE[cnr, 0]
        jj = cubes[:, 1] + _CUBE[cnr, 1]
        kk = cubes[:, 2] + _CUBE[cnr, 2]
        corner_nodes[:, cnr] = ii + nx * (jj + ny * kk)
    parity = (cubes.sum(axis=1) & 1).astype(bool)
    tA = np.array(_SPLIT_A, np.int64)
    tB = np.array(_SPLIT_B, np.int64)
    tets = np.where(parity[:, None, None], corner_nodes[:, tB], corner_nodes[:, tA])
    tets = tets.reshape(-1, 4).astype(np.uint32)
    return rest, tets, ijk


def _face_nodes(ijk: np.ndarray, dims, face: str) -> np.ndarray:
    a, b, c = dims
    axis = "xyz".index(face[0])
    hi = face[1] == "+"
    lim = (a, b, c)[axis] if hi else 0
    return np.nonzero(ijk[:, axis] == lim)[0].astype(np.uint32)


def cantilever_160() -> Scene:
    """8x2x2 cubes of 0.1 m, 5 tets each (160 tets, 81 nodes), jitter 0.01 m
    (seed 0); E=1e5, nu=0.3, rho=1000, gravity -9.81 z; x=0 face fixed;
    dt=1/60, CG rel 1e-8 (abs 0), max 200 iterations, 120 steps."""
    rest, tets, ijk = grid_mesh(8, 2, 2, 0.1, 0.01, 0)
    fixed = _face_nodes(ijk, (8, 2, 2), "x-")
    return Scene(name="cantilever_8x2x2", rest=rest, tets=tets, young=1e5, poisson=0.3,
                 density=1000.0, gravity=(0.0, 0.0, -9.81), rel_eps=1e-8, abs_eps=0.0,
                 max_iter=200, steps=120, knc_nodes=fixed, knc_targets=rest[fixed].copy(),
                 grid=(8, 2, 2), h=0.1)


def large_block(n: int = 60, seed: int = 0) -> Scene:
    """n^3 cubes of 0.01 m (n=60: 1.08M tets, 226,981 nodes), jitter 0.1 h;
    per-element E log-uniform [5e4, 5e5], nu uniform [0.25, 0.45]; bottom
    (z=0) face fixed, top-face nodes start at v=(1,0,0); CG rel 1e-6, 60 steps."""
    h = 0.01
    rest, tets, ijk = grid_mesh(n, n, n, h, 0.1 * h, seed)
    rng = np.random.default_rng(seed + 1)
    T = tets.shape[0]
    young = np.exp(rng.uniform(math.log(5e4), math.log(5e5), size=T))
    poisson = rng.uniform(0.25, 0.45, size=T)
    fixed = _face_nodes(ijk, (n, n, n), "z-")
    top = _face_nodes(ijk, (n, n, n), "z+")
    v0 = np.zeros_like(rest)
    v0[top, 0] = 1.0
    return Scene(name=f"block_{n}x{n}x{n}", rest=rest, tets=tets, young_per_elem=young,
                 poisson_per_elem=poisson, density=1000.0, rel_eps=1e-6, abs_eps=0.0,
                 max_iter=500, steps=60, knc_nodes=fixed, knc_targets=rest[fixed].copy(),
                 init_vel=v0, grid=(n, n, n), h=h)


def compressed_cube(n: int = 40, steps: int = 120, ratio: float = 0.4) -> Scene:
    """n^3 cubes of 0.01 m (n=40: 320k tets, 68,921 nodes), E=2e5, nu=0.45;
    bottom face fixed, top face driven by position constraints to `ratio`
    of the initial height, linearly over `steps` steps; CG rel 1e-6."""
    h = 0.01
    rest, tets, ijk = grid_mesh(n, n, n, h, 0.1 * h, 0)
    bottom = _face_nodes(ijk, (n, n, n), "z-")
    top = _face_nodes(ijk, (n, n, n), "z+")
    nodes = np.concatenate([bottom, top]).astype(np.uint32)
    base = rest[nodes].copy()
    nb = bottom.shape[0]
    height = n * h

    def schedule(step: int) -> np.ndarray:
        s = min(step + 1, steps) / float(steps)
        t = base.copy()
        t[nb:, 2] = base[nb:, 2] - s * (1.0 - ratio) * height
        return t

    return Scene(name=f"compress_{n}x{n}x{n}", rest=rest, tets=tets, young=2e5, poisson=0.45,
                 density=1000.0, rel_eps=1e-6, abs_eps=0.0, max_iter=500, steps=steps,
                 knc_nodes=nodes, knc_targets=base.copy(), knc_schedule=schedule,
                 grid=(n, n, n), h=h)


def sheared_crush(n: int = 4, steps: int = 30, ratio: float = 0.15, shear: float = 0.3, h: float = 0.1,
                  rotation: int = 1) -> Scene:
    """n^3 cubes of h (default 10 cm: large enough that DAPD's collapse axis
    passes the reference's absolute area test, so its offset rotation runs),
    E=2e5, nu=0.45; bottom face fixed, top face driven to `ratio` of the
    height while it slides by `shear` of the height in x, linearly over
    `steps` steps; DAPD rotations; CG rel 1e-8."""
    rest, tets, ijk = grid_mesh(n, n, n, h, 0.1 * h, 0)
    bottom = _face_nodes(ijk, (n, n, n), "z-")
    top = _face_nodes(ijk, (n, n, n), "z+")
    nodes = np.concatenate([bottom, top]).astype(np.uint32)
    base = rest[nodes].copy()
    nb = bottom.shape[0]
    height = n * h

    def schedule(step: int) -> np.ndarray:
        s = min(step + 1, steps) / float(steps)
        t = base.copy()
        t[nb:, 2] = base[nb:, 2] - s * (1.0 - ratio) * height
        t[nb:, 0] = base[nb:, 0] + s * shear * height
        return t

    return Scene(name=f"sheared_crush_{n}x{n}x{n}", rest=rest, tets=tets, young=2e5, poisson=0.45, density=1000.0,
                 rel_eps=1e-8, abs_eps=0.0, max_iter=500, steps=steps, knc_nodes=nodes, knc_targets=base.copy(),
                 knc_schedule=schedule, grid=(n, n, n), h=h, rotation=rotation)


def from_geo(path: str, fixed_below: Optional[float] = None, **scene_kwargs) -> Scene:
    """A Scene from the tet-solid shape of a shape file (.geo, as the
    reference's TetGen converter writes it), read by fem_geo_read: the
    shape's float vertices and its tets in the shape's order, the order in
    which a reference solid adds them to its element set.
    fixed_below: nodes with z <= this become fixed position constraints."""
    from . import capi
    rest, tets, _ = capi.geo_read(path)
    knc = np.zeros(0, np.uint32)
    if fixed_below is not None:
        knc = np.nonzero(rest[:, 2] <= fixed_below)[0].astype(np.uint32)
    name = scene_kwargs.pop("name", "geo_" + path.rsplit("/", 1)[-1])
    return Scene(name=name, rest=rest, tets=tets, knc_nodes=knc, knc_targets=rest[knc].copy(), **scene_kwargs)


def random_block(rng: np.random.Generator, lo: int = 4, hi: int = 30, idx: int = 0,
                 dims=None) -> Scene:
    """One mesh of the batched workload: a x b x c cubes (uniform in [lo, hi]),
    h = 0.01, jitter 0.1 h; per-mesh E log-uniform [1e4, 1e6], nu uniform
    [0.2, 0.45]; one random face fixed; CG rel 1e-6."""
    if dims is None:
        dims = tuple(int(x) for x in rng.integers(lo, hi + 1, size=3))
    a, b, c = dims
    h = 0.01
    rest, tets, ijk = grid_mesh(a, b, c, h, 0.1 * h, int(rng.integers(0, 2**31)))
    young = float(math.exp(rng.uniform(math.log(1e4), math.log(1e6))))
    poisson = float(rng.uniform(0.2, 0.45))
    face = ["x-", "x+", "y-", "y+", "z-", "z+"][int(rng.integers(0, 6))]
    fixed = _face_nodes(ijk, dims, face)
    return Scene(name=f"mesh{idx}_{a}x{b}x{c}", rest=rest, tets=tets, young=young, poisson=poisson,
                 density=1000.0, gravity=(0.0, 0.0, -9.81), rel_eps=1e-6, abs_eps=0.0, max_iter=500,
                 steps=60, knc_nodes=fixed, knc_targets=rest[fixed].copy(), grid=dims, h=h)


def batch_scenes(count: int = 1024, seed: int = 0, lo: int = 4, hi: int = 30) -> List[Scene]:
    """The batched workload: `count` independent uneven meshes."""
    rng = np.random.default_rng(seed)
    return [random_block(rng, lo, hi, idx=i) for i in range(count)]


def sized_block(rng: np.random.Generator, target_tets: float, idx: int = 0) -> Scene:
    """A mesh of the served pool: nearest 5*a*b*c to `target_tets` with a
    near-cubic aspect, material and fixed face as random_block."""
    cubes = max(1.0, target_tets / 5.0)
    a = max(1, int(round(cubes ** (1.0 / 3.0))))
    b = max(1, int(round(math.sqrt(cubes / a))))
    c = max(1, int(round(cubes / (a * b))))
    return random_block(rng, idx=idx, dims=(a, b, c))


def served_pool(count: int = 4096, seed: int = 0, lo: float = 200.0, hi: float = 200000.0) -> List[Scene]:
    """The served pool: `count` scenes whose sizes are drawn log-uniform in
    [lo, hi] tets, each realised as the nearest 5*a*b*c block (material and
    fixed face as the batched workload)."""
    rng = np.random.default_rng(seed)
    targets = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    return [sized_block(rng, float(t), idx=i) for i, t in enumerate(targets)]


def write_tetgen(rest: np.ndarray, tets: np.ndarray, base_path: str, base_index: int = 1,
                 node_attributes: int = 0, boundary_markers: bool = False) -> None:
    """Write base_path.node / base_path.ele in TetGen's format (ids from
    base_index; optional zero attributes and markers, which readers skip)."""
    rest = np.asarray(rest, dtype=np.float64)
    tets = np.asarray(tets, dtype=np.int64)
    with open(base_path + ".node", "w") as f:
        f.write(f"{rest.shape[0]} 3 {node_attributes} {1 if boundary_markers else 0}\n")
        extra = " 0" * node_attributes + (" 0" if boundary_markers else "")
        for i, p in enumerate(rest):
            f.write(f"{i + base_index} {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}{extra}\n")
        f.write("# written by risdsdgcfem_thesis_gb300.scenes.write_tetgen\n")
    with open(base_path + ".ele", "w") as f:
        f.write(f"{tets.shape[0]} 4 0\n")
        for e, t in enumerate(tets):
            f.write(f"{e + base_index} {t[0] + base_index} {t[1] + base_index} {t[2] + base_index} "
                    f"{t[3] + base_index}\n")


def from_tetgen(base_path: str, natural_scale: float = 0.0, fixed_below: Optional[float] = None,
                **scene_kwargs) -> Scene:
    """A Scene from base_path.node / base_path.ele, read by the library's
    fem_tetgen_read (the reference converter's semantics: float positions,
    tets with det <= 0 dropped, optional natural scale and centering).
    fixed_below: nodes with z <= this become fixed position constraints."""
    from . import capi
    rest, tets, _ = capi.read_tetgen(base_path + ".node", base_path + ".ele", natural_scale)
    knc = np.zeros(0, np.uint32)
    if fixed_below is not None:
        knc = np.nonzero(rest[:, 2] <= fixed_below)[0].astype(np.uint32)
    name = scene_kwargs.pop("name", "tetgen_" + base_path.rsplit("/", 1)[-1])
    return Scene(name=name, rest=rest, tets=tets, knc_nodes=knc, knc_targets=rest[knc].copy(), **scene_kwargs)
