"""TetGen mesh ingest (fem_tetgen_read), CPU only: the reference converter's
semantics (examples/tetgen2geo/main.cpp) restated here in numpy as the
checker -- base index from the first node id, float positions, skipped
attributes and markers, tets with float det <= 0 dropped
(EditableTetSolidShape3::AddTetrahedron, Geo/shape/TetSolidShape3.cpp:
278-307), the "-nsac" natural scale over the float AABB merged node by node
(Geo/bv/GAABB.h:27-50) -- plus the error cases and a round trip through
the solver's oracle.
"""
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes

CUBE_NODE = """# a unit cube, ids from 1, one attribute and a boundary marker per node
8 3 1 1
1 0.0 0.0 0.0 7.5 1
2 1.0 0.0 0.0 7.5 1
3 0.0 1.0 0.0 7.5 1
4 1.0 1.0 0.0 7.5 1
5 0.0 0.0 1.0 7.5 1
6 1.0 0.0 1.0 7.5 1
7 0.0 1.0 1.0 7.5 1
8 1.0 1.0 1.0 7.5 1
"""
# a positively oriented 5-tet split of the cube, one attribute per tet, plus
# one tet given with the wrong orientation
CUBE_ELE = """6 4 1
1 1 2 4 6 0.5
2 1 3 7 4 0.5
3 1 5 6 7 0.5
4 4 7 6 8 0.5
5 1 4 7 6 0.5
6 1 4 2 6 0.5
# trailing comment, as TetGen writes
"""


def _write(tmp_path, name, node, ele):
    base = str(tmp_path / name)
    with open(base + ".node", "w") as f:
        f.write(node)
    with open(base + ".ele", "w") as f:
        f.write(ele)
    return base


def _converter(node_text, ele_text, natural_scale=0.0):
    """The reference converter's arithmetic in float32 (test-side restatement)."""
    def toks(text):
        out = []
        for line in text.splitlines():
            out += line.split("#", 1)[0].split()
        return out
    t = toks(node_text)
    n, dim, na, nb = (int(v) for v in t[:4])
    k = 4
    pos = np.empty((n, 3), np.float32)
    base = None
    for i in range(n):
        vid = int(t[k])
        base = vid if base is None else base
        pos[i] = [np.float32(float(v)) for v in t[k + 1:k + 4]]
        k += 4 + na + nb
    t = toks(ele_text)
    ne, npt, ea = (int(v) for v in t[:3])
    k = 3
    kept, dropped = [], 0
    for _ in range(ne):
        v = [int(x) - base for x in t[k + 1:k + 5]]
        k += 5 + ea
        c = [pos[v[j]] - pos[v[0]] for j in (1, 2, 3)]
        m = np.array([[c[0][0], c[1][0], c[2][0]], [c[0][1], c[1][1], c[2][1]], [c[0][2], c[1][2], c[2][2]]],
                     np.float32)
        f = np.float32
        det = (m[0, 0] * m[1, 1] * m[2, 2] - m[0, 0] * m[2, 1] * m[1, 2] + m[1, 0] * m[2, 1] * m[0, 2]
               - m[1, 0] * m[0, 1] * m[2, 2] + m[2, 0] * m[0, 1] * m[1, 2] - m[2, 0] * m[1, 1] * m[0, 2])
        if f(det) <= 0:
            dropped += 1
        else:
            kept.append(v)
    if natural_scale > 0:
        half = np.float32(0.5)
        c = half * (pos[0] + pos[0])
        h = half * (pos[0] - pos[0])
        for p in pos[1:]:
            lo, hi = c - h, c + h
            lo = np.where(p < lo, p, lo)
            hi = np.where(p > hi, p, hi)
            c, h = half * (lo + hi), half * (hi - lo)
        s = np.float32(natural_scale) / np.max(np.float32(2) * h)
        pos = s * (pos + (-c))
    return pos.astype(np.float64), np.array(kept, np.uint32).reshape(-1, 4), dropped


def test_reads_cube_like_the_converter(fem_lib, tmp_path):
    base = _write(tmp_path, "cube", CUBE_NODE, CUBE_ELE)
    rest, tets, dropped = fem_lib.read_tetgen(base + ".node", base + ".ele")
    r_rest, r_tets, r_dropped = _converter(CUBE_NODE, CUBE_ELE)
    assert np.array_equal(rest, r_rest) and np.array_equal(tets, r_tets)
    assert dropped == r_dropped == 1 and tets.shape == (5, 4)
    assert tets.min() == 0 and tets.max() == 7  # base-1 ids made base-0


def test_natural_scale_and_center(fem_lib, tmp_path):
    rng = np.random.default_rng(0)
    rest0, tets0, _ = scenes.grid_mesh(3, 2, 2, 0.37, 0.05, 1)
    rest0 = rest0 * 3.1 + np.array([5.0, -2.0, 0.25])
    base = str(tmp_path / "block")
    scenes.write_tetgen(rest0, tets0, base, base_index=0, node_attributes=2, boundary_markers=True)
    node, ele = open(base + ".node").read(), open(base + ".ele").read()
    rest, tets, dropped = fem_lib.read_tetgen(base + ".node", base + ".ele", natural_scale=2.0)
    r_rest, r_tets, r_dropped = _converter(node, ele, natural_scale=2.0)
    assert np.array_equal(rest, r_rest) and np.array_equal(tets, r_tets) and dropped == r_dropped == 0
    ext = rest.max(axis=0) - rest.min(axis=0)
    assert abs(ext.max() - 2.0) < 1e-5
    assert np.abs(0.5 * (rest.max(axis=0) + rest.min(axis=0))).max() < 1e-5
    assert rng is not None


def test_round_trip_through_the_oracle(fem_lib, oracle, tmp_path):
    """A grid block written as TetGen files, read back, and stepped by the
    oracle: the same result as the block built directly, up to the float
    rounding of the positions."""
    sc0 = scenes.random_block(np.random.default_rng(2), dims=(3, 2, 2))
    base = str(tmp_path / "rt")
    scenes.write_tetgen(sc0.rest, sc0.tets, base)
    sc = scenes.from_tetgen(base, young=sc0.young, poisson=sc0.poisson, density=sc0.density,
                            gravity=(0.0, 0.0, -9.81), dt=sc0.dt, rel_eps=1e-10, max_iter=400)
    sc0.gravity, sc0.rel_eps, sc0.max_iter = (0.0, 0.0, -9.81), 1e-10, 400
    assert np.array_equal(sc.tets, sc0.tets)
    assert np.array_equal(sc.rest, sc0.rest.astype(np.float32).astype(np.float64))
    fixed = np.asarray(sc0.knc_nodes)
    sc.knc_nodes, sc.knc_targets = fixed.astype(np.uint32), sc.rest[fixed].copy()
    a, b = oracle.Solid(sc, "port"), oracle.Solid(sc0, "port")
    for _ in range(5):
        a.step()
        b.step()
    xa, _ = a.state()
    xb, _ = b.state()
    assert np.abs(xa - xb).max() < 1e-6 * np.abs(xb).max()


@pytest.mark.parametrize("node,ele,code,words", [
    ("4 2 0 0\n1 0 0\n2 1 0\n3 0 1\n4 1 1\n", "1 4 0\n1 1 2 3 4\n", "FEM_E_ARG", "dimension"),
    (CUBE_NODE, "1 10 0\n1 1 2 3 4 5 6 7 8 1 2\n", "FEM_E_ARG", "4 nodes"),
    (CUBE_NODE, "1 4 0\n1 1 2 3 9\n", "FEM_E_INDEX", "outside"),
    (CUBE_NODE, "2 4 0\n1 1 2 4 6\n", "FEM_E_ARG", "malformed"),
    ("8 3 0 0\n1 0 0 zero\n", CUBE_ELE, "FEM_E_ARG", "malformed"),
])
def test_rejects_bad_files(fem_lib, tmp_path, node, ele, code, words):
    base = _write(tmp_path, "bad", node, ele)
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.read_tetgen(base + ".node", base + ".ele")
    assert e.value.code == getattr(fem_lib, code) and words in str(e.value)


def test_missing_file(fem_lib, tmp_path):
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.read_tetgen(str(tmp_path / "none.node"), str(tmp_path / "none.ele"))
    assert e.value.code == fem_lib.FEM_E_ARG and "cannot open" in str(e.value)


def test_header_promising_more_than_the_file_holds(fem_lib, tmp_path):
    """A .node header claiming a billion nodes fails on the missing lines."""
    base = _write(tmp_path, "short", "1000000000 3 0 0\n1 0 0 0\n", CUBE_ELE)
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.read_tetgen(base + ".node", base + ".ele")
    assert e.value.code == fem_lib.FEM_E_ARG and "malformed node 1" in str(e.value)


def test_natural_scale_of_coincident_nodes_is_rejected(fem_lib, tmp_path):
    """-nsac on nodes that span no extent (one point) has nothing to scale
    to: an error instead of the converter's division by zero."""
    node = "4 3 0 0\n1 0.5 0.5 0.5\n2 0.5 0.5 0.5\n3 0.5 0.5 0.5\n4 0.5 0.5 0.5\n"
    base = _write(tmp_path, "point", node, "1 4 0\n1 1 2 3 4\n")
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.read_tetgen(base + ".node", base + ".ele", natural_scale=1.0)
    assert e.value.code == fem_lib.FEM_E_ARG and "no extent" in str(e.value)
    # without the option the file reads (its one tet is dropped as flat)
    rest, tets, dropped = fem_lib.read_tetgen(base + ".node", base + ".ele")
    assert rest.shape == (4, 3) and tets.shape == (0, 4) and dropped == 1
