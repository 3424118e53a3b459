"""Parity at the configs' own sizes (the oracle restatement on all host
threads, bit-identical to its serial form).

* C2, the 60^3 block (1.08M tets): the plain FP64 solid against the oracle
  for 2 steps -- the second ends at the 500-iteration cap in both -- within
  max(1e-10, 10 x the oracle's own movement under a 1e-15 input change).
* C2 mixed: the batched mixed path against the FP64 solid for the config's
  60 steps, within 1e-5 (x rel-L2; v normalised by the run's peak |v|).
* C3: meshes of the 1024-mesh workload -- the largest (126k tets), the
  stiffest (E ~ 1e6), two that end every step at the CG cap, and four more --
  stepped 3 times by the mixed batch against the oracle, within 1e-5.
"""
import os

import numpy as np
import pytest

from risdsdgcfem_thesis_gb300 import scenes
from parity_util import bar_cap, check_bar, perturbed, rel

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
C3_PICKS = (122, 869, 21, 950, 426, 163, 630, 5)


def test_fp64_solid_matches_oracle_at_full_c2_size(fem_lib, oracle):
    sc = scenes.large_block(n=60)
    assert sc.num_tets == 1_080_000
    g = fem_lib.Solid(sc)
    o = oracle.Solid(sc, "port").set_threads(THREADS)
    p = oracle.Solid(perturbed(sc, 1), "port").set_threads(THREADS)
    for _ in range(2):
        a, b, c = g.step(1), o.step(), p.step()
        assert abs(a["cg_iterations"] - b["iters"]) <= max(1, 2 * abs(c["iters"] - b["iters"]) + 1)
    xg, vg = g.state()
    xo, vo = o.state()
    xp, vp = p.state()
    check_bar("C2 60^3 fp64 solid, 2 steps", "x", rel(xg, xo), 1e-10, rel(xp, xo), bar_cap(sc))
    check_bar("C2 60^3 fp64 solid, 2 steps", "v", rel(vg, vo), 1e-10, rel(vp, vo), bar_cap(sc))


def test_mixed_matches_fp64_at_full_c2_size_over_the_config_steps(fem_lib):
    sc = scenes.large_block(n=60)
    mix = fem_lib.Batch([sc], precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False)
    f64 = fem_lib.Solid(sc, compute_energy=False)
    vpeak = 0.0
    for _ in range(sc.steps):
        mix.step(1)
        f64.step(1)
        assert mix.stats(0)["status"] == 0
        vpeak = max(vpeak, float(np.linalg.norm(f64.state()[1])))
    xm, vm = mix.state(0)
    xf, vf = f64.state()
    check_bar("C2 60^3 mixed vs fp64, 60 steps", "x", rel(xm, xf), 1e-5, 0.0)
    check_bar("C2 60^3 mixed vs fp64, 60 steps", "v", float(np.linalg.norm(vm - vf)) / vpeak, 1e-5, 0.0)


def test_mixed_matches_oracle_on_meshes_of_the_batched_workload(fem_lib, oracle):
    allsc = scenes.batch_scenes(1024)
    picks = [allsc[i] for i in C3_PICKS]
    assert max(s.num_tets for s in allsc) == picks[0].num_tets  # the largest
    assert max(s.young for s in allsc) == picks[1].young        # the stiffest
    b = fem_lib.Batch(picks, precision=fem_lib.FEM_PRECISION_MIXED, compute_energy=False)
    orcs = [oracle.Solid(s, "port").set_threads(THREADS) for s in picks]
    vpeak = np.zeros(len(picks))
    capped = 0
    for _ in range(3):
        b.step(1)
        for i, o in enumerate(orcs):
            st = o.step()
            capped += st["iters"] >= picks[i].max_iter
            vpeak[i] = max(vpeak[i], float(np.linalg.norm(o.state()[1])))
    assert capped >= 6  # two meshes end every step at the cap
    for i, o in enumerate(orcs):
        xm, vm = b.state(i)
        xo, vo = o.state()
        name = f"C3 mesh {C3_PICKS[i]} {picks[i].name} mixed vs oracle"
        check_bar(name, "x", rel(xm, xo), 1e-5, 0.0)
        check_bar(name, "v", float(np.linalg.norm(vm - vo)) / vpeak[i], 1e-5, 0.0)
