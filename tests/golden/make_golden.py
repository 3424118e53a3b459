"""Generates tests/golden/*.npz from the reference's own FP64 code.

Run in a container that has the reference sources (the oracle Makefile
compiles them into oracle/_ref/): python tests/golden/make_golden.py

Fixtures (all from oracle/_ref/libfemref_dbl.so, the reference translation
units with Mal's Sqrt/Sin/Cos/ATan2 at double precision, except where noted):
  cantilever_160.npz   x, v after each of 120 FixedSteps of the 160-tet
                       cantilever; per-step CG iterations, residuals, energies.
  elements_160.npz     per-element R, f_e, df_x(dx), V on a deformed state of the
                       same mesh (bent, twisted, 3 elements inverted).
  literal_fp64.npz     the reference FP64 build as written (float-rounded Mal
                       math): per-step iterations and energies of the same
                       scene (the rotations are NaN at rest, so CG stops at 0).
  fie_160.npz          the fully-implicit Euler (Newton, Delta x) integrator:
                       x, v after each of 30 FixedSteps of the cantilever with
                       3 Newton iterations per step, then 5 quasi-static steps;
                       per-step CG and Newton statistics, energies.
  fie_block.npz        the same integrator on a 5x3x4 block with per-element
                       E and nu, damping, an initial velocity and a moving
                       constraint: per-step statistics, final x and v.

  dapd_cube.npz        the DAPD rotation (ms::fem::Params::eRM_DAPD, threshold
                       0.1f) on a 6^3-cube block crushed to 15 % of its height
                       over 30 steps (elements invert): per-step statistics,
                       final x, v and per-element direction of collapse, with
                       the QIE integrator (prefix qie_) and FIE (fie_). The
                       directions of collapse are the restatement's, whose x
                       and v equal the reference build's bit for bit.

  minres.npz           the MINRES linear solver (ns::ILSS_MINRES) in place of CG:
                       the cantilever with QIE (60 steps, prefix qie_) and FIE
                       (20 steps, fie_), and the moving-constraint block of
                       fie_block.npz with QIE (12 steps, block_): per-step
                       statistics, final x and v.

  lcm.npz              the C_LCM material (first Piola-Kirchhoff linear
                       corotational) in place of C_WRP: the cantilever with
                       QIE (60 steps, qie_) and FIE (20 steps, fie_), and the
                       moving-constraint block with QIE (12 steps, block_).

  materials.npz        the C_LCMH (LCM/WRP hybrid, m_ECIE_k_factor 1 and 0.05)
                       and C_CCM materials: the cantilever with QIE (30 steps;
                       prefixes lcmh_, lcmh_k005_, ccm_) and the moving-
                       constraint block with QIE (12 steps, lcmh_block_,
                       ccm_block_).

python tests/golden/make_golden.py fie      writes only the two FIE fixtures;
python tests/golden/make_golden.py materials  only the C_LCMH / C_CCM fixture;
python tests/golden/make_golden.py lcm      only the C_LCM fixture;
python tests/golden/make_golden.py dapd     only the DAPD fixture;
python tests/golden/make_golden.py minres   only the MINRES fixture.
"""
import dataclasses
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import pyoracle as O  # noqa: E402
from risdsdgcfem_thesis_gb300 import scenes  # noqa: E402


def deformed_state(sc, seed=7):
    """A bent and twisted configuration with a few inverted elements."""
    rng = np.random.default_rng(seed)
    x = sc.rest.copy()
    L = x[:, 0].max()
    s = x[:, 0] / L
    x[:, 2] -= 0.15 * s ** 2                       # bend
    ang = 0.6 * s                                  # twist about the x axis
    yc, zc = x[:, 1] - 0.1, x[:, 2] - 0.1
    x[:, 1] = 0.1 + np.cos(ang) * yc - np.sin(ang) * zc
    x[:, 2] = 0.1 + np.sin(ang) * yc + np.cos(ang) * zc
    x += rng.uniform(-0.004, 0.004, size=x.shape)
    # invert three elements by pushing one node through the opposite face
    for e in (17, 80, 141):
        t = sc.tets[e]
        c = x[t[1:]].mean(axis=0)
        x[t[0]] = c + 1.5 * (c - x[t[0]])
    return x


def _stat_arrays(stats, prefix=""):
    out = {}
    for key, dt in (("iters", np.int32), ("rel_res", np.float64), ("abs_res", np.float64),
                    ("elastic_energy", np.float64), ("potential_energy", np.float64),
                    ("nr_iters", np.int32), ("nr_rel", np.float64), ("nr_abs", np.float64)):
        out[prefix + key] = np.array([s[key] for s in stats], dt)
    return out


def fie_block_scene():
    rng = np.random.default_rng(5)
    sc = scenes.random_block(rng, dims=(5, 3, 4))
    T = sc.num_tets
    sc.young_per_elem = np.exp(rng.uniform(np.log(5e4), np.log(5e5), T))
    sc.poisson_per_elem = rng.uniform(0.25, 0.45, T)
    sc.damping_ratio = 1.0
    sc.init_vel = rng.standard_normal(sc.rest.shape) * 0.1
    base = sc.knc_targets.copy()
    sc.knc_schedule = lambda k: base + np.array([0.0, 0.0, 0.002 * (k + 1)])
    sc.steps = 12
    sc.integrator = 1
    sc.nr_max_iter = 4
    return sc


def fie_fixtures():
    sc = scenes.cantilever_160()
    sc.integrator = 1
    ref = O.Solid(sc, "ref_dbl")
    xs, vs, stats = [], [], []
    for _ in range(30):
        stats.append(ref.step())
        x, v = ref.state()
        xs.append(x)
        vs.append(v)
    qs = O.Solid(dataclasses.replace(sc, integrator=2), "ref_dbl")
    qstats = [qs.step() for _ in range(5)]
    xq, vq = qs.state()
    np.savez_compressed(os.path.join(HERE, "fie_160.npz"), x=np.array(xs), v=np.array(vs), xq=xq, vq=vq,
                        **_stat_arrays(stats), **_stat_arrays(qstats, "q_"))
    sc = fie_block_scene()
    ref = O.Solid(sc, "ref_dbl")
    stats = ref.run()
    x, v = ref.state()
    np.savez_compressed(os.path.join(HERE, "fie_block.npz"), x=x, v=v, **_stat_arrays(stats))


def dapd_scene(integrator):
    return dataclasses.replace(scenes.compressed_cube(n=6, steps=30, ratio=0.15), rotation=1,
                               integrator=integrator)


def dapd_fixture():
    out = {}
    for prefix, integ in (("qie_", 0), ("fie_", 1)):
        sc = dapd_scene(integ)
        ref = O.Solid(sc, "ref_dbl")
        port = O.Solid(sc, "port")
        stats = []
        for _ in range(30):
            stats.append(ref.step())
            assert port.step() == stats[-1]
        x, v = ref.state()
        xp, vp = port.state()
        assert np.array_equal(x, xp) and np.array_equal(v, vp)
        out.update(_stat_arrays(stats, prefix))
        out[prefix + "x"] = x
        out[prefix + "v"] = v
        out[prefix + "doc"] = port.doc()
    np.savez_compressed(os.path.join(HERE, "dapd_cube.npz"), **out)


def minres_cases():
    cant = scenes.cantilever_160()
    return (("qie_", dataclasses.replace(cant, ls_solver=1), 60),
            ("fie_", dataclasses.replace(cant, ls_solver=1, integrator=1), 20),
            ("block_", dataclasses.replace(fie_block_scene(), ls_solver=1, integrator=0), 12))


def minres_fixture():
    out = {}
    for prefix, sc, steps in minres_cases():
        ref = O.Solid(sc, "ref_dbl")
        stats = [ref.step() for _ in range(steps)]
        x, v = ref.state()
        out.update(_stat_arrays(stats, prefix))
        out[prefix + "x"] = x
        out[prefix + "v"] = v
    np.savez_compressed(os.path.join(HERE, "minres.npz"), **out)


def lcm_cases():
    cant = scenes.cantilever_160()
    return (("qie_", dataclasses.replace(cant, material=1), 60),
            ("fie_", dataclasses.replace(cant, material=1, integrator=1), 20),
            ("block_", dataclasses.replace(fie_block_scene(), material=1, integrator=0), 12))


def lcm_fixture():
    out = {}
    for prefix, sc, steps in lcm_cases():
        ref = O.Solid(sc, "ref_dbl")
        stats = [ref.step() for _ in range(steps)]
        x, v = ref.state()
        out.update(_stat_arrays(stats, prefix))
        out[prefix + "x"] = x
        out[prefix + "v"] = v
    np.savez_compressed(os.path.join(HERE, "lcm.npz"), **out)


def material_cases():
    cant = scenes.cantilever_160()
    block = dataclasses.replace(fie_block_scene(), integrator=0)
    return (("lcmh_", dataclasses.replace(cant, material=2), 30),
            ("lcmh_k005_", dataclasses.replace(cant, material=2, ecie_k_factor=0.05), 30),
            ("ccm_", dataclasses.replace(cant, material=3), 30),
            ("lcmh_block_", dataclasses.replace(block, material=2), 12),
            ("ccm_block_", dataclasses.replace(block, material=3), 12))


def materials_fixture():
    out = {}
    for prefix, sc, steps in material_cases():
        ref = O.Solid(sc, "ref_dbl")
        stats = [ref.step() for _ in range(steps)]
        x, v = ref.state()
        out.update(_stat_arrays(stats, prefix))
        out[prefix + "x"] = x
        out[prefix + "v"] = v
    np.savez_compressed(os.path.join(HERE, "materials.npz"), **out)


def main():
    O.build(reference=True)
    if sys.argv[1:] == ["materials"]:
        materials_fixture()
        print("wrote the C_LCMH / C_CCM fixture to", HERE)
        return
    if sys.argv[1:] == ["lcm"]:
        lcm_fixture()
        print("wrote the C_LCM fixture to", HERE)
        return
    if sys.argv[1:] == ["minres"]:
        minres_fixture()
        print("wrote the MINRES fixture to", HERE)
        return
    if sys.argv[1:] == ["fie"]:
        fie_fixtures()
        print("wrote FIE fixtures to", HERE)
        return
    if sys.argv[1:] == ["dapd"]:
        dapd_fixture()
        print("wrote the DAPD fixture to", HERE)
        return
    fie_fixtures()
    dapd_fixture()
    minres_fixture()
    lcm_fixture()
    materials_fixture()
    sc = scenes.cantilever_160()

    ref = O.Solid(sc, "ref_dbl")
    xs, vs, stats = [], [], []
    for _ in range(sc.steps):
        stats.append(ref.step())
        x, v = ref.state()
        xs.append(x)
        vs.append(v)
    np.savez_compressed(os.path.join(HERE, "cantilever_160.npz"), x=np.array(xs), v=np.array(vs),
                        iters=np.array([s["iters"] for s in stats], np.int32),
                        rel_res=np.array([s["rel_res"] for s in stats]),
                        abs_res=np.array([s["abs_res"] for s in stats]),
                        elastic_energy=np.array([s["elastic_energy"] for s in stats]),
                        potential_energy=np.array([s["potential_energy"] for s in stats]))

    xd = deformed_state(sc)
    tes = O.RefElementSet(sc, dbl=True)
    tes.begin_eval(xd)
    R = tes.rotations()
    fe = tes.f_e()
    dx = np.random.default_rng(3).standard_normal(xd.shape)
    dfx = tes.df_x(dx)
    V = tes.V()
    port = O.Solid(sc, "port")
    port.begin_eval(xd)
    np.savez_compressed(os.path.join(HERE, "elements_160.npz"), x=xd, dx=dx, R=R, f_e=fe, df_x=dfx, V=np.array(V),
                        detF=port.detF())

    lit = O.Solid(sc, "ref")
    lst = [lit.step() for _ in range(5)]
    xl, vl = lit.state()
    np.savez_compressed(os.path.join(HERE, "literal_fp64.npz"), iters=np.array([s["iters"] for s in lst], np.int32),
                        elastic_energy=np.array([s["elastic_energy"] for s in lst]), x=xl, v=vl)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()
