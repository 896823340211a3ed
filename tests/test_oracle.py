"""The CPU oracle (oracle/siting_oracle.c) pinned against the reference.

* golden.json holds the outputs of the reference's own seqsite (compiled from
  its sources) for seeded synthetic DEMs and the reference's sample DEM; the
  oracle must reproduce every stage bit for bit.
* Where the reference library is built on this machine, random small cases
  are also compared stage by stage against it directly.
"""
import hashlib

import numpy as np
import pytest

from conftest import make_dem
from oracle_bind import Oracle, observers_text, reference_available


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _cases(golden_path):
    import json

    with open(golden_path) as f:
        return json.load(f)["cases"]


def pytest_generate_tests(metafunc):
    if "gcase" in metafunc.fixturenames:
        from conftest import GOLDEN

        cases = _cases(GOLDEN)
        metafunc.parametrize("gcase", cases, ids=[c["name"] for c in cases])


def test_oracle_matches_reference_golden(gcase, oracle, native):
    n, roi, h, ntests, bw, nw0, iv = gcase["args"]
    dem = make_dem(gcase["dem"], n)
    assert sha(dem) == gcase["dem_sha256"], "input DEM differs from the one the fixture used"
    r = oracle.run(dem, n, roi, h, ntests, bw, nw0, iv)
    assert r["geo"].nwanted == gcase["nwanted"]
    assert sha(r["vix"]) == gcase["vix_sha256"]
    assert int(r["vix"].sum(dtype=np.int64)) == gcase["vix_sum"]
    assert sha(r["obs"]) == gcase["obs_sha256"]
    assert sha(r["sheds"]) == gcase["sheds_sha256"]
    assert sha(r["selected"]) == gcase["selected_sha256"]
    assert r["nused"] == gcase["nused"]
    assert r["cumarea"] == gcase["cumarea"]
    assert hashlib.md5(observers_text(r["obs"], r["selected"], n)).hexdigest() == \
        gcase["observers_md5"]


def test_known_answer_md5s_recorded(golden):
    """The sample DEM's observers files (reference runs `1000 50 100 50 10 10000 {0,1}`)."""
    by = {c["name"]: c for c in golden["cases"]}
    if "dem_bin_iv0" not in by:
        pytest.skip("fixture generated without dem.bin")
    assert by["dem_bin_iv0"]["observers_md5"] == "0f0e2cd59b33eaa3dbeae4f78d261f05"
    assert by["dem_bin_iv1"]["observers_md5"] == "ff6affb15ab1f99489f8cafb79a84701"
    assert (by["dem_bin_iv0"]["nused"], by["dem_bin_iv1"]["nused"]) == (235, 270)


def test_coverage_equals_union_of_selected(oracle, native):
    dem = native.fbm_dem(150, 21, octaves=7, range_max=6000)
    r = oracle.run(dem, 150, 20, 15, 24, 10, 225, 1)
    assert oracle.union_count(150, 20, r["obs"], r["sheds"], r["selected"]) == r["cumarea"]


def test_oracle_thread_count_independent(oracle, native):
    dem = native.fbm_dem(120, 5, octaves=6, range_max=4000)
    oracle.lib.oracle_set_threads(1)
    a = oracle.run(dem, 120, 14, 10, 20, 10, 144, 1)
    oracle.lib.oracle_set_threads(0)
    import os

    oracle.lib.oracle_set_threads(os.cpu_count() or 1)
    b = oracle.run(dem, 120, 14, 10, 20, 10, 144, 1)
    for k in ("vix", "obs", "sheds", "selected"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.skipif(not reference_available(), reason="reference library not built here")
@pytest.mark.parametrize("seed", [101, 102, 103, 104])
def test_oracle_matches_reference_random(seed, oracle, native):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(40, 140))
    roi = int(rng.integers(3, 40))
    h = int(rng.integers(0, 60))
    ntests = int(rng.integers(1, 40))
    bw = int(rng.integers(8, 30))
    nw0 = int(rng.integers(20, 400))
    iv = int(rng.integers(0, 2))
    dem = native.fbm_dem(n, seed, octaves=int(rng.integers(3, 9)),
                         range_max=int(rng.integers(100, 20000)))
    ref = Oracle("reference")
    g = oracle.geometry(n, bw, nw0)
    if g.too_small:
        pytest.skip("geometry rejected by the reference")
    a = oracle.run(dem, n, roi, h, ntests, bw, nw0, iv)
    b = ref.run(dem, n, roi, h, ntests, bw, nw0, iv)
    for k in ("vix", "obs", "sheds", "selected"):
        assert np.array_equal(a[k], b[k]), k
    assert a["cumarea"] == b["cumarea"]


def test_reciprocal_identity_exhaustive():
    """(float)(1.0/d) == 1.0f/(float)d for every |d| the VIX stage can see (roi <= 10000)."""
    d = np.arange(1, 20001, dtype=np.float64)
    a = (1.0 / d).astype(np.float32)
    b = np.float32(1.0) / d.astype(np.float32)
    assert np.array_equal(a, b)


def test_oracle_matches_reference_golden_c2_4096(oracle, native, golden):
    """The oracle at the benchmark's full 4096^2 size (65 536 observers,
    intervis 1) against the outputs the reference's seqsite recorded."""
    cases = {c["name"]: c for c in golden.get("fullsize", [])}
    if "c2_4096" not in cases:
        pytest.skip("no full-size fixture")
    test_oracle_matches_reference_golden(cases["c2_4096"], oracle, native)


# The workloads' DEM recipes: (nrows, seed, octaves, ridged weight, range).
DEM_RECIPES = [(1000, 1000, 8, 0.0, 10000), (4096, 4096, 10, 0.3, 30000),
               (16384, 16384, 12, 0.0, 40000)]


@pytest.mark.parametrize("n,seed,octaves,ridged,rmax", DEM_RECIPES,
                         ids=["c1_1000", "c2_4096", "c4_16384"])
def test_oracle_dem_generator_equals_library(oracle, native, n, seed, octaves, ridged, rmax):
    """The CPU baseline builds its inputs with the oracle's own generator, so
    that it never loads the library: both must give the same bytes."""
    a = oracle.fbm_dem(n, seed, octaves=octaves, ridged_weight=ridged, range_max=rmax)
    b = native.fbm_dem(n, seed, octaves=octaves, ridged_weight=ridged, range_max=rmax)
    assert np.array_equal(a, b)
