"""Serving loop: every job's results are identical alone and in the mix, the
HBM budget is enforced at admission and per batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(native, n_jobs, seed, sizes=(96, 360), rois=(8, 60)):
    """Windows of one larger raster (submitted with a row pitch, no copy) and
    contiguous DEMs, mixed parameters as in the serving workload."""
    rng = np.random.default_rng(seed)
    raster = native.fbm_dem(1024, 5000 + seed, octaves=8, range_max=20000).reshape(1024, 1024)
    jobs = []
    for j in range(n_jobs):
        n = int(np.exp(rng.uniform(np.log(sizes[0]), np.log(sizes[1]))))
        p = native.Params(nrows=n, roi=int(rng.integers(*rois)), height=int(rng.integers(5, 80)),
                          ntests=int(rng.integers(16, 80)), bw=int(rng.choice([8, 16, 32])),
                          nwanted0=max(1, n * n // 128), intervis=int(rng.integers(0, 2)))
        if j % 2 == 0:
            x0, y0 = (int(v) for v in rng.integers(0, 1024 - n, size=2))
            dem = raster[x0:x0 + n, y0:y0 + n]  # a view: row pitch 1024
        else:
            dem = native.fbm_dem(n, 7000 + 10 * seed + j, octaves=7)
        jobs.append((p, dem))
    return jobs


def test_served_jobs_equal_single_runs(ctx, native):
    jobs = _jobs(native, 12, 1)
    with native.Server(0, hbm_budget=4 << 30, max_batch_jobs=5) as srv:
        tickets = [srv.submit(p, d) for p, d in jobs]
        out = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(jobs) and st["refused"] == 0
    assert max(info.batch_jobs for _, _, info in out) <= 5
    for (p, dem), (obs, sel, info) in zip(jobs, out):
        o1, s1, r1 = ctx.run(p, np.ascontiguousarray(dem).ravel())
        assert np.array_equal(obs, o1) and np.array_equal(sel, s1)
        assert (info.result.nusedsheds, info.result.cumarea) == (r1.nusedsheds, r1.cumarea)
        assert info.t_submit <= info.t_start <= info.t_done


def test_served_jobs_match_oracle(native, oracle):
    jobs = _jobs(native, 4, 2, sizes=(100, 200))
    with native.Server(0, hbm_budget=2 << 30) as srv:
        tickets = [srv.submit(p, d) for p, d in jobs]
        out = [srv.wait(t, timeout=300) for t in tickets]
    for (p, dem), (obs, sel, info) in zip(jobs, out):
        want = oracle.run(np.ascontiguousarray(dem).ravel(), p.nrows, p.roi, p.height, p.ntests,
                          p.bw, p.nwanted0, p.intervis)
        assert np.array_equal(obs, want["obs"]) and np.array_equal(sel, want["selected"])
        assert (info.result.nusedsheds, info.result.cumarea) == (want["nused"], want["cumarea"])


def test_budget_admission_and_batch_split(ctx, native):
    small = [native.Params(nrows=256, roi=20, height=30, ntests=32, bw=16, nwanted0=512,
                           intervis=j % 2) for j in range(6)]
    one = ctx.batch_workspace_bytes(small[:1])
    two = ctx.batch_workspace_bytes(small[:2])
    assert two > one > 0
    budget = two + (two - one) // 2  # two jobs fit a batch, three do not
    assert ctx.batch_workspace_bytes(small[:3]) > budget
    big = native.Params(nrows=1024, roi=60, height=30, ntests=32, bw=16, nwanted0=8192)
    dems = [native.fbm_dem(256, 40 + j) for j in range(6)]
    with native.Server(0, hbm_budget=budget) as srv:
        with pytest.raises(native.SitingError) as e:
            srv.submit(big, native.fbm_dem(1024, 3))
        assert e.value.status == native.ENOMEM
        tickets = [srv.submit(p, d) for p, d in zip(small, dems)]
        out = [srv.wait(t, timeout=300) for t in tickets]
        st = srv.stats()
    assert st["refused"] == 1 and st["completed"] == 6
    assert all(info.batch_jobs <= 2 for _, _, info in out)
    assert st["peak_workspace"] <= budget
    for p, d, (obs, sel, info) in zip(small, dems, out):
        o1, s1, _ = ctx.run(p, d)
        assert np.array_equal(obs, o1) and np.array_equal(sel, s1)


def test_wait_unknown_ticket_and_timeout(native):
    p = native.Params(nrows=128, roi=10, height=20, ntests=16, bw=16, nwanted0=64)
    with native.Server(0, hbm_budget=1 << 30) as srv:
        t = srv.submit(p, native.fbm_dem(128, 9))
        obs, sel, info = srv.wait(t, timeout=120)
        assert info.status == native.OK
        with pytest.raises(native.SitingError):  # released by the first wait
            srv.wait(t, timeout=0)
        t2 = srv.submit(p, native.fbm_dem(128, 10))
        try:
            srv.wait(t2, timeout=0.0)
        except TimeoutError:  # still queued or running: the ticket stays valid
            srv.wait(t2, timeout=120)


def test_request_admitted_mid_flight_overlaps_and_matches_solo(ctx, native):
    """Continuous admission: a small request submitted while a large job is on
    the GPU starts before that job ends, finishes before it (its stages and
    selection overlap the large job's on the device) and gives the same
    result as a solo run."""
    import time

    big = native.Params(nrows=4096, roi=150, height=100, ntests=100, bw=16, nwanted0=65536,
                        intervis=1)
    small = native.Params(nrows=256, roi=20, height=30, ntests=32, bw=16, nwanted0=512,
                          intervis=1)
    big_dem = native.fbm_dem(4096, 41, octaves=10, range_max=20000)
    small_dem = native.fbm_dem(256, 42, octaves=7, range_max=5000)
    with native.Server(0, hbm_budget=16 << 30) as srv:
        srv.wait(srv.submit(small, small_dem), timeout=300)  # warm: modules loaded
        tb = srv.submit(big, big_dem)
        time.sleep(0.005)  # the large job's stages are on the GPU by now
        ts = srv.submit(small, small_dem)
        obs_s, sel_s, info_s = srv.wait(ts, timeout=300)
        obs_b, sel_b, info_b = srv.wait(tb, timeout=300)
    assert info_s.status == native.OK and info_b.status == native.OK
    assert info_s.t_start < info_b.t_done, "admitted only after the large job ended"
    assert info_s.t_done < info_b.t_done, "did not overlap the large job"
    assert info_s.batch_jobs >= 2  # two jobs in flight at its admission
    o1, s1, r1 = ctx.run(small, small_dem)
    assert np.array_equal(obs_s, o1) and np.array_equal(sel_s, s1)
    assert (info_s.result.nusedsheds, info_s.result.cumarea) == (r1.nusedsheds, r1.cumarea)
    o2, s2, r2 = ctx.run(big, big_dem)
    assert np.array_equal(obs_b, o2) and np.array_equal(sel_b, s2)
