import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels")


@pytest.fixture(scope="session")
def pkg():
    from tests.pkgload import load_package
    return load_package()


@pytest.fixture(scope="session")
def native(pkg):
    """The built CUDA library (compiled for sm_103a by halign-4_gb300/build.py)."""
    pkg.build_library()
    return pkg.lib()


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.oracle import reference_or_none
    r = reference_or_none()
    if r is None:
        pytest.skip("reference sources not available on this host")
    return r


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    d = ROOT / "tests" / "golden"

    class G:
        meta = json.loads((d / "meta.json").read_text())

        @staticmethod
        def load(name):
            return np.load(d / name, allow_pickle=False)
    return G


@pytest.fixture(scope="session")
def gpu(pkg, native):
    if pkg.device_count() == 0:
        pytest.skip("no CUDA device")
    return pkg
