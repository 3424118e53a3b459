"""Tet-solid shapes and shape files (fem_tetshape_rebuild, fem_geo_write,
fem_geo_read, fem_tetgen_to_geo), CPU only, against the reference's own
geometry code: oracle/geo_harness.cpp drives the reference's
EditableTetSolidShape3 (AddTetrahedron, the -nsac transform, EndEdition:
Geo/shape/TetSolidShape3.cpp:262-845) and ShapeLibrary text save
(Geo/shape/ShapeLibrary.cpp:332-360, util/ItemStreamSerialization.cpp) as
examples/tetgen2geo/main.cpp does; the files must agree byte for byte
except the per-vertex byte the reference leaves uninitialised."""
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes


def _ref(oracle):
    if not os.path.exists(oracle.GEO_REF_SO):
        pytest.skip("reference sources not present in this container")


def _raw_ele(path):
    rows = [l.split() for l in open(path) if l.strip() and not l.lstrip().startswith("#")]
    n = int(rows[0][0])
    return np.array([[int(v) for v in r[1:5]] for r in rows[1:1 + n]], dtype=np.int64)


def _compare_files(mine, ref):
    a = open(mine).read().splitlines()
    b = open(ref).read().splitlines()
    assert len(a) == len(b)
    for la, lb in zip(a, b):
        if la.strip().startswith("vec_v "):
            assert len(la) == len(lb)  # one byte per vertex, unused by the reference
        else:
            assert la == lb, (la[:80], lb[:80])


def _meshes():
    # a jittered block with interior vertices (several layers)
    rest, tets, _ = scenes.grid_mesh(6, 5, 4, 0.01, 0.001, 3)
    yield "block", rest, tets, 0.0
    # the same with a tet given inverted (dropped), a node no tet uses
    # (removed) and the converter's -nsac 2
    t2 = tets.copy()
    t2[7] = t2[7][[0, 2, 1, 3]]
    r2 = np.vstack([rest, [[0.5, 0.5, 0.5]]])
    yield "inverted_unused_nsac", r2, t2, 2.0
    # a thin slab: every vertex on the boundary, one layer
    rest, tets, _ = scenes.grid_mesh(7, 3, 1, 0.02, 0.0, 0)
    yield "slab", rest, tets, 0.0


@pytest.mark.parametrize("case", ["block", "inverted_unused_nsac", "slab"])
def test_shape_file_equals_the_reference_converter(fem_lib, oracle, tmp_path, case):
    _ref(oracle)
    name, rest, tets, nsac = next(m for m in _meshes() if m[0] == case)
    base = str(tmp_path / name)
    scenes.write_tetgen(rest, tets, base, base_index=1)
    mine, ref = str(tmp_path / "mine.geo"), str(tmp_path / "ref.geo")
    fem_lib.tetgen_to_geo(base, mine, natural_scale=nsac)
    pos, _, _ = fem_lib.read_tetgen(base + ".node", base + ".ele")
    assert oracle.geo_ref_convert(pos, _raw_ele(base + ".ele") - 1, nsac, ref) == 0
    _compare_files(mine, ref)


def test_rebuild_arrays_and_read_back(fem_lib, tmp_path):
    _, rest, tets, _ = next(_meshes())
    s = fem_lib.tetshape_rebuild(rest, tets)
    V, T = s["rest"].shape[0], s["tets"].shape[0]
    assert V == rest.shape[0] and T == tets.shape[0]
    # the output tets are the input tets in layer order
    assert np.array_equal(s["node_of"][s["tets"]], tets[s["tet_of"]])
    # layers tile the tets, lowest first, and every boundary vertex is layer 0
    first, count = s["layers"][:, 0], s["layers"][:, 1]
    assert first[0] == 0 and np.array_equal(first[1:], np.cumsum(count)[:-1]) and count.sum() == T
    assert len(s["layers"]) > 1
    # neighbours are symmetric and share the opposite face's three vertices
    nb = s["neighbors"]
    for t in range(T):
        for i in range(4):
            n = nb[t, i]
            if n == 0xFFFFFFFF:
                continue
            face = set(s["tets"][t][[(i + 1) % 4, (i + 2) % 4, (i + 3) % 4]])
            assert t in nb[n] and face <= set(s["tets"][n])
    # boundary faces: one per face without a neighbour, oriented outwards
    assert s["bfaces"].shape[0] == int((nb == 0xFFFFFFFF).sum())
    x = s["rest"]
    cen = x[s["tets"]].mean(axis=1).mean(axis=0)
    out = 0
    for f in s["bfaces"]:
        nrm = np.cross(x[f[1]] - x[f[0]], x[f[2]] - x[f[0]])
        out += np.dot(nrm, x[f].mean(axis=0) - cen) > 0
    assert out == len(s["bfaces"])
    path = str(tmp_path / "a.geo")
    fem_lib.geo_write(path, rest, tets)
    xr, tr, nr = fem_lib.geo_read(path)
    assert np.array_equal(tr, s["tets"]) and np.array_equal(nr, s["neighbors"])
    assert np.array_equal(xr, x.astype(np.float32).astype(np.float64))


def test_solid_from_the_shape_file_steps_like_the_rebuilt_mesh(fem_lib, oracle, tmp_path):
    """The element order a reference solid gets from the shape file, through
    the oracle: the same step as the arrays from fem_tetshape_rebuild."""
    _, rest, tets, _ = next(_meshes())
    path = str(tmp_path / "b.geo")
    fem_lib.geo_write(path, rest, tets)
    xr, tr, _ = fem_lib.geo_read(path)
    s = fem_lib.tetshape_rebuild(rest.astype(np.float32).astype(np.float64), tets)
    fixed = np.nonzero(xr[:, 2] <= xr[:, 2].min() + 1e-6)[0].astype(np.uint32)
    mk = lambda r, t: scenes.Scene(name="shape", rest=r, tets=t, knc_nodes=fixed, knc_targets=r[fixed].copy(),
                                   gravity=(0.0, 0.0, -9.81))
    a, b = oracle.Solid(mk(xr, tr), "port"), oracle.Solid(mk(s["rest"], s["tets"]), "port")
    for _ in range(3):
        assert a.step() == b.step()
    assert np.array_equal(a.state()[0], b.state()[0])


def test_shape_file_errors(fem_lib, tmp_path):
    _, rest, tets, _ = next(_meshes())
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.geo_read(str(tmp_path / "missing.geo"))
    assert e.value.code == fem_lib.FEM_E_ARG
    good = str(tmp_path / "g.geo")
    fem_lib.geo_write(good, rest, tets)
    text = open(good).read()
    for bad in (text.replace("version 3u", "version 2u"),
                text.replace("num_t ", "num_t 1"),
                text.replace("vec_t ^", "vec_t ^G"),
                text.replace("}\n", "")):
        p = str(tmp_path / "bad.geo")
        open(p, "w").write(bad)
        with pytest.raises(fem_lib.FemError) as e:
            fem_lib.geo_read(p)
        assert e.value.code == fem_lib.FEM_E_ARG
    big, bt, _ = scenes.grid_mesh(60, 20, 12, 0.01, 0.0, 0)  # 72,000 tets > 65534
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.geo_write(str(tmp_path / "big.geo"), big, bt)
    assert e.value.code == fem_lib.FEM_E_ARG
    bad_tets = tets.copy()
    bad_tets[0, 0] = rest.shape[0]
    with pytest.raises(fem_lib.FemError) as e:
        fem_lib.tetshape_rebuild(rest, bad_tets)
    assert e.value.code == fem_lib.FEM_E_INDEX
