import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pic-deposition_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")

for p in (ORACLE, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the kernels through the C ABI)")
    config.addinivalue_line("markers", "slow: full-size (benchmark-shape) case")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    return oracle


@pytest.fixture(scope="session")
def port(oracle_mod):
    return oracle_mod.Port()


@pytest.fixture(scope="session")
def ref(oracle_mod):
    if not oracle_mod.Ref.available():
        if oracle_mod.reference_src() is not None:
            oracle_mod.build(ref=True)
        else:
            pytest.skip("reference sources not present here (oracle/_ref unavailable)")
    try:
        return oracle_mod.Ref()
    except OSError as e:  # built for another machine
        pytest.skip(f"oracle/_ref does not load here: {e}")


@pytest.fixture(scope="session")
def pg():
    import pic_gb300

    pic_gb300.lib()
    return pic_gb300
