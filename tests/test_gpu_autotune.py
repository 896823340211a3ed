"""Autotuner: the tuned plans are valid, used by later calls, and never
change results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotuned_runs_match_oracle(native, oracle):
    p = native.Params(nrows=600, roi=60, height=40, ntests=48, bw=16, nwanted0=2048, intervis=1)
    dem = native.fbm_dem(600, 61, octaves=8, range_max=15000)
    with native.Context(0) as ctx:
        plan = ctx.autotune(p, dem, sample_rows=600)  # the whole DEM: SITE is tuned too
        assert plan.vix_tile in (16, 32, 64) and plan.vix_smem in (0, 1)
        assert plan.shed_smem in (0, 1, 2) and plan.site_ctas >= 1
        obs, sel, res = ctx.run(p, dem)
        want = oracle.run(dem, p.nrows, p.roi, p.height, p.ntests, p.bw, p.nwanted0, p.intervis)
        assert np.array_equal(obs, want["obs"]) and np.array_equal(sel, want["selected"])
        assert (res.nusedsheds, res.cumarea) == (want["nused"], want["cumarea"])


def test_autotuned_batch_matches_plain(native):
    jobs = [(native.Params(nrows=n, roi=r, height=30, ntests=32, bw=16, nwanted0=n * n // 64,
                           intervis=j % 2), native.fbm_dem(n, 70 + j))
            for j, (n, r) in enumerate([(320, 40), (480, 40), (256, 90)])]
    with native.Context(0) as plain, native.Context(0) as tuned:
        for p, d in jobs:
            tuned.autotune(p, d, sample_rows=256)
        out_t = tuned.run_batch([p for p, _ in jobs], [d for _, d in jobs])
        for (p, d), (obs, sel, res) in zip(jobs, out_t):
            o, s, r = plain.run(p, d)
            assert np.array_equal(obs, o) and np.array_equal(sel, s)
            assert (res.nusedsheds, res.cumarea) == (r.nusedsheds, r.cumarea)
        tuned.autotune_clear()
