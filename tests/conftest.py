import gzip
import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gbc():
    """The product library, built in-tree (fails loudly if it cannot be)."""
    from bc_gb300 import build
    build.build()
    import bc_gb300
    bc_gb300.lib()
    return bc_gb300


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def datasets(tmp_path_factory):
    """Shipped reference datasets (gzip'd fixtures) unpacked to a temp dir."""
    d = tmp_path_factory.mktemp("datasets")
    out = {}
    src = os.path.join(GOLDEN, "datasets")
    for f in sorted(os.listdir(src)):
        name = f[:-3]
        p = d / name
        with gzip.open(os.path.join(src, f), "rb") as a, open(p, "wb") as b:
            shutil.copyfileobj(a, b)
        out[name] = str(p)
    return out


@pytest.fixture(scope="session")
def gpu(gbc):
    if gbc.device_count() < 1:
        pytest.fail("no CUDA device visible for a test marked gpu")
    return gbc
