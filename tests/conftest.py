import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    """Builds libyaptgpu.so and the CPU oracle once per session."""
    from yapt_gb300 import build as B
    B.build_lib()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return True


@pytest.fixture(scope="session")
def py_yapt(built):
    """The pybind11 module (YAPT's Python surface), built next to the library."""
    from yapt_gb300 import build as B
    B.build_pybind()
    from yapt_gb300 import py_yapt as Y
    return Y


LUT_NAMES = ["ss", "ss_avg", "ssms", "ssms_avg", "trans_denser", "trans_lighter", "trans_avg_denser",
             "trans_avg_lighter", "sheen"]


@pytest.fixture(scope="session")
def host_luts(built):
    from yapt_gb300 import _native as N
    return {n: N.host_table(n) for n in LUT_NAMES}
