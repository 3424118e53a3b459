"""Small workloads over every kernel family, run by test_gpu_bounds_check.py
twice: in a child process on the index-checking library
(FEMGB_BOUNDS_CHECK=1, libfemtet_gb300_bounds.so) and in the test process on
the normal one. Writes the final states to an .npz and prints, as one JSON
line, the index-check counts read after each workload.

    python tests/bounds_workload.py OUT.npz
"""
import dataclasses
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from risdsdgcfem_thesis_gb300 import capi, scenes  # noqa: E402


def _blocks():
    rng = np.random.default_rng(5)
    return [scenes.random_block(rng, idx=i, dims=d) for i, d in enumerate([(6, 5, 4), (9, 4, 5), (5, 5, 5)])]


def workloads():
    """(name, callable returning {array name: array})."""

    def solid(sc, steps, assembled=False):
        def run():
            s = capi.Solid(sc)
            s.set_assembled(assembled)
            s.step(steps)
            x, v = s.state()
            s.close()
            return {"x": x, "v": v}
        return run

    def batch(precision):
        def run():
            scs = _blocks()
            b = capi.Batch(scs, precision, reorder=True)
            b.step(2)
            out = {}
            for i in range(len(scs)):
                out[f"x{i}"], out[f"v{i}"] = b.state(i)
            b.close()
            return out
        return run

    def server():
        scs = _blocks()
        srv = capi.Server(capi.FEM_PRECISION_MIXED)
        ids = [srv.add(sc) for sc in scs]
        srv.admit()
        for i in ids:
            srv.submit(i, i)
            srv.submit(i, 100 + i)
        srv.drain()
        out = {}
        for i in ids:
            out[f"x{i}"], out[f"v{i}"] = srv.state(i)
        srv.close()
        return out

    cant = scenes.cantilever_160()
    blk = scenes.compressed_cube(n=4, steps=10, ratio=0.6)
    crush = dataclasses.replace(scenes.compressed_cube(n=6, steps=30, ratio=0.15), rotation=capi.FEM_ROTATION_DAPD)
    return [
        ("solid_msvd_cg", solid(cant, 5)),
        ("solid_dapd", solid(crush, 28)),
        ("solid_lcm", solid(dataclasses.replace(blk, material=capi.FEM_MATERIAL_C_LCM), 4)),
        ("solid_minres", solid(dataclasses.replace(cant, ls_solver=capi.FEM_LS_MINRES), 4)),
        ("solid_minres_assembled", solid(dataclasses.replace(blk, ls_solver=capi.FEM_LS_MINRES), 4, True)),
        ("solid_fie", solid(dataclasses.replace(cant, integrator=capi.FEM_INTEGRATOR_FIE_DX), 3)),
        ("batch_fp64", batch(capi.FEM_PRECISION_FP64)),
        ("batch_mixed", batch(capi.FEM_PRECISION_MIXED)),
        ("server_mixed", server),
    ]


def main(out_path):
    capi.load()
    arrays, counts = {}, {}
    for name, run in workloads():
        for k, a in run().items():
            arrays[f"{name}.{k}"] = a
        counts[name] = capi.bounds_check_status()
    np.savez(out_path, **arrays)
    print(json.dumps(counts))


if __name__ == "__main__":
    main(sys.argv[1])
