import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TESTS = os.path.join(ROOT, "tests")
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(TESTS, "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """The native library, built in-tree if it is missing or stale."""
    from siting_gb300 import build as b

    b.build()
    import siting_gb300 as sg

    sg.load()
    return sg


@pytest.fixture(scope="session")
def oracle():
    from oracle_bind import Oracle, build_port

    build_port()
    return Oracle("port")


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def ctx(native):
    c = native.Context(0)
    yield c
    c.close()


def dem_bin_path():
    """The reference's sample DEM, where its files are staged (oracle/_ref/src)."""
    from oracle_bind import ref_dem_bin

    return ref_dem_bin()


def make_dem(spec, n):
    """DEM of a golden case: seeded fBm, a flat DEM, or the sample dem.bin."""
    if "flat" in spec:
        return np.full(n * n, spec["flat"], np.uint16)
    if "file" in spec:
        p = dem_bin_path()
        if p is None:
            pytest.skip("dem.bin not available on this machine")
        return np.fromfile(p, np.uint16)
    import siting_gb300 as sg

    kw = {k: v for k, v in spec.items() if k != "seed"}
    return sg.fbm_dem(n, spec["seed"], **kw)
