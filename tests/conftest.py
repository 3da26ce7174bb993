"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU.

The oracle (oracle/) is the checker: it is imported here only to compare the
device results against the reference semantics.
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "ph-core_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs through libphcuda.so)")


@pytest.fixture(scope="session")
def ora():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def kats():
    with open(os.path.join(ROOT, "tests", "golden", "reference_kats.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def cu():
    """The device backend; GPU tests only."""
    import phase_cu

    phase_cu.init()
    return phase_cu


def lit_from_json(x):
    """Golden literal -> region literal object understood by both sides."""
    from phase_cu.region import R

    if "i" in x:
        return x["i"]
    return R(x["f"], x["l"], x["s"], x["x"])
