import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (run with -m gpu)")


@pytest.fixture(scope="session")
def ref():
    from oracle import bls12_377
    return bls12_377


@pytest.fixture(scope="session")
def ocpu():
    from oracle import cpu
    cpu.lib()
    return cpu


@pytest.fixture(scope="session")
def kats():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_kats.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def engine():
    """The GPU engine (libdriver.so); built on demand so a fresh box only needs the sources."""
    from hardcaml_zprize_gb300 import build
    build.build()
    import hardcaml_zprize_gb300 as eng
    eng.load_library()
    return eng
