import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 machine)")


GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden_files(prefix=""):
    """Force-path fixtures (the md_* dynamics, rdf_* histogram and dump_*
    file fixtures are named explicitly by their own tests)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and f.startswith(prefix) and not f.startswith(("md_", "rdf_", "dump_")))


@pytest.fixture(scope="session")
def port_built():
    from oracle import port
    port.build()
    return port
