import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: longer statistical runs")


@pytest.fixture(scope="session")
def built():
    """Builds libpsim_gb300.so and the CPU oracle once per session."""
    from psim_gb300 import build
    from oracle import oracle
    build.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    from psim_gb300 import api
    if api.device_count() < 1:
        pytest.fail("no CUDA device visible to libpsim_gb300 (GPU tests need a GB300)")
    return True


def model_path(name: str) -> str:
    """A fixture model file: tests/golden/models/<name>.json, or its gzipped form written out
    as plain JSON into a per-user temporary directory."""
    plain = os.path.join(GOLDEN, "models", name + ".json")
    if os.path.exists(plain) or not os.path.exists(plain + ".gz"):
        return plain
    import tempfile
    directory = os.path.join(tempfile.gettempdir(), f"psim_gb300_models_{os.getuid()}")
    os.makedirs(directory, exist_ok=True)
    return demo_model_path(name, directory)


def demo_model_path(name: str, directory: str) -> str:
    """One of the reference's own demo models (tests/golden/models/<name>.json.gz), written
    out as plain JSON into ``directory``."""
    import gzip
    out = os.path.join(directory, name + ".json")
    if not os.path.exists(out):
        with gzip.open(os.path.join(GOLDEN, "models", name + ".json.gz"), "rb") as f, open(out, "wb") as g:
            g.write(f.read())
    return out
