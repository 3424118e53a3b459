"""The ctypes mirrors of the C ABI's structs (risdsdgcfem_thesis_gb300/capi.py)
have the sizes and field offsets that include/fem_tet.h gives them: a small C
program compiled against the header prints both, with no GPU."""
import ctypes as C
import json
import os
import shutil
import subprocess

import pytest

from risdsdgcfem_thesis_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {
    "fem_params": capi.FemParams,
    "fem_step_stats": capi.FemStepStats,
    "fem_batch_options": capi.FemBatchOptions,
    "fem_server_options": capi.FemServerOptions,
    "fem_server_completion": capi.FemServerCompletion,
    "fem_server_status": capi.FemServerStatus,
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "fem_tet.h"', "int main(void) {",
             'printf("{");']
    first = True
    for cname, cls in STRUCTS.items():
        fields = [f[0] for f in cls._fields_]
        parts = [f'\\"{f}\\": %zu' for f in fields]
        fmt = ("" if first else ", ") + f'\\"{cname}\\": {{\\"sizeof\\": %zu, ' + ", ".join(parts) + "}"
        args = [f"sizeof({cname})"] + [f"offsetof({cname}, {f})" for f in fields]
        lines.append(f'printf("{fmt}", {", ".join(args)});')
        first = False
    lines += ['printf("}\\n");', "return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)


def test_ctypes_structs_match_the_header(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, cls in STRUCTS.items():
        got = layout[cname]
        assert C.sizeof(cls) == got["sizeof"], (cname, C.sizeof(cls), got["sizeof"])
        for f in cls._fields_:
            assert getattr(cls, f[0]).offset == got[f[0]], (cname, f[0])
