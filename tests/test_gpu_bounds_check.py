"""The index-checking build (-DFEM_BOUNDS_CHECK, bounds.cuh) on small
workloads of every kernel family: the FP64 solid (MSVD with the one-cluster
CG, DAPD through its collapse branch, C_LCM, MINRES matrix-free and on the
assembled stiffness, FIE), the FP64 and mixed batches and the served path.
Every data-dependent index the kernels read from a table (element node ids,
node CSR entries, assembled blocks' columns and contributions, tile node
lists, tile-local ids and CSR entries, partial slots, constraint nodes) is
checked against its limit; no
check may fire, and the results agree with the normal library's to 1e-5 of
each array's largest entry (the checks change which index an out-of-range
access would use, not the formulas; the compiler may still contract a
multiply-add differently around the added branches, and the CG solves to
1e-6 carry such rounding differences into the states).

The checking build runs in a child process (the two libraries export the
same symbols, so one process loads one of them)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_index_checks_stay_silent_and_change_no_result(fem_lib, tmp_path):
    from risdsdgcfem_thesis_gb300 import build
    build.build_bounds_check()
    out = tmp_path / "bounds.npz"
    env = dict(os.environ, FEMGB_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_workload.py"), str(out)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    counts = json.loads(r.stdout.strip().splitlines()[-1])
    for name, c in counts.items():
        assert c["enabled"], name
        assert c["failures"] == 0, (name, c)
    checked = np.load(out)

    sys.path.insert(0, HERE)
    import bounds_workload
    assert not fem_lib.bounds_check_status()["enabled"]
    for name, run in bounds_workload.workloads():
        for k, a in run().items():
            b = checked[f"{name}.{k}"]
            scale = max(np.abs(a).max(), 1e-30)
            assert np.abs(a - b).max() <= 1e-5 * scale, (name, k, np.abs(a - b).max() / scale)
