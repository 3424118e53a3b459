import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build(reference=os.path.isdir(pyoracle.REFERENCE_SRC))
    return pyoracle


@pytest.fixture(scope="session")
def fem_lib():
    from risdsdgcfem_thesis_gb300 import build, capi
    build.build()
    capi.load()
    return capi


def pytest_terminal_summary(terminalreporter):
    """The effective bars of the calibrated parity comparisons that ran."""
    try:
        from parity_util import BARS
    except ImportError:
        return
    if not BARS:
        return
    terminalreporter.write_sep("-", "calibrated parity bars (measured <= max(tol, 10 x oracle floor))")
    for case, qty, measured, bar, floor in BARS:
        terminalreporter.write_line(f"{case:<48} {qty:<4} measured {measured:9.3g}  bar {bar:9.3g}  floor {floor:9.3g}")
