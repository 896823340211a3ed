"""Batched form: every job of a mixed batch equals the oracle (and so the
plain single-job path) bit for bit, whatever the launch plan."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixed_jobs(native, n_jobs, seed, sizes=(96, 400), rois=(8, 60)):
    """A mix in the shape of the batched workload: log-uniform sides (multiples
    of 8 and not), per-job amplitude, roi, height, targets, bw, nwanted =
    cells/64 and alternating intervis."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        n = int(np.exp(rng.uniform(np.log(sizes[0]), np.log(sizes[1]))))
        if j % 3 == 0:
            n = (n + 31) // 32 * 32
        p = native.Params(nrows=n, roi=int(rng.integers(*rois)), height=int(rng.integers(5, 60)),
                          ntests=int(rng.choice([16, 32, 64])), bw=int(rng.choice([8, 16, 32])),
                          nwanted0=max(1, n * n // 64), intervis=j % 2)
        dem = native.fbm_dem(n, 900 + seed * 100 + j, octaves=7,
                             range_max=int(rng.integers(2000, 30000)))
        jobs.append((p, dem))
    return jobs


def _check_job(oracle, p, dem, obs, sel, res):
    want = oracle.run(dem, p.nrows, p.roi, p.height, p.ntests, p.bw, p.nwanted0, p.intervis)
    assert np.array_equal(obs, want["obs"]), "observers differ"
    assert np.array_equal(sel, want["selected"]), \
        f"selection differs in {int(np.count_nonzero(sel != want['selected']))} entries"
    assert (res.nusedsheds, res.cumarea) == (want["nused"], want["cumarea"])


def test_batch_matches_oracle(ctx, oracle, native):
    jobs = _mixed_jobs(native, 10, 1)
    out = ctx.run_batch([p for p, _ in jobs], [d for _, d in jobs])
    for (p, dem), (obs, sel, res) in zip(jobs, out):
        _check_job(oracle, p, dem, obs, sel, res)


@pytest.mark.parametrize("plan", [
    dict(vix_tile=16, vix_smem=1, shed_smem=1, site_ctas=1),
    dict(vix_tile=64, vix_smem=0, shed_smem=0, site_ctas=3),
    dict(vix_tile=32, vix_smem=1, shed_smem=-1, site_ctas=16),
    dict(vix_tile=16, vix_smem=1, shed_smem=2, site_ctas=2),
])
def test_batch_plans_do_not_change_results(ctx, oracle, native, plan):
    jobs = _mixed_jobs(native, 5, 2)
    plans = [native.Plan(**plan)] * len(jobs)
    out = ctx.run_batch([p for p, _ in jobs], [d for _, d in jobs], plans)
    for (p, dem), (obs, sel, res) in zip(jobs, out):
        _check_job(oracle, p, dem, obs, sel, res)


def test_batch_dev_matches_host(ctx, native):
    torch = pytest.importorskip("torch")
    jobs = _mixed_jobs(native, 6, 3)
    host = ctx.run_batch([p for p, _ in jobs], [d for _, d in jobs])
    d_dems = [torch.from_numpy(d.view(np.int16)).cuda() for _, d in jobs]
    geos = [native.block_geometry(p.nrows, p.bw, p.nwanted0) for p, _ in jobs]
    d_obs = [torch.empty(g.nwanted, dtype=torch.int32, device="cuda") for g in geos]
    d_sel = [torch.empty(g.nwanted, dtype=torch.uint8, device="cuda") for g in geos]
    torch.cuda.synchronize()
    res = ctx.run_batch_dev([p for p, _ in jobs], d_dems, d_obs, d_sel)
    for (obs, sel, r0), o, s, r1 in zip(host, d_obs, d_sel, res):
        assert np.array_equal(o.cpu().numpy(), obs)
        assert np.array_equal(s.cpu().numpy(), sel)
        assert (r0.nusedsheds, r0.cumarea) == (r1.nusedsheds, r1.cumarea)


def test_batch_equals_single_job_runs(ctx, native):
    jobs = _mixed_jobs(native, 4, 4, sizes=(200, 520), rois=(20, 90))
    out = ctx.run_batch([p for p, _ in jobs], [d for _, d in jobs])
    for (p, dem), (obs, sel, res) in zip(jobs, out):
        o2, s2, r2 = ctx.run(p, dem)
        assert np.array_equal(obs, o2) and np.array_equal(sel, s2)
        assert (res.nusedsheds, res.cumarea) == (r2.nusedsheds, r2.cumarea)


def test_batch_large_roi(ctx, oracle, native):
    """roi 150-200: windows beyond shared memory take the L1 paths."""
    jobs = _mixed_jobs(native, 3, 5, sizes=(420, 520), rois=(150, 201))
    out = ctx.run_batch([p for p, _ in jobs], [d for _, d in jobs])
    for (p, dem), (obs, sel, res) in zip(jobs, out):
        _check_job(oracle, p, dem, obs, sel, res)


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_modes_match_oracle(ctx, oracle, native, mode):
    """Multi-job VIX and FINDMAX grids (1) and one launch per stage and job
    (2) give the same results; small block widths give many FINDMAX blocks
    per job and non-multiple sides make blocks straddle VIX tiles."""
    jobs = _mixed_jobs(native, 8, 6, sizes=(90, 300), rois=(5, 40))
    for k, (n, bw, roi) in enumerate(((40, 1, 5), (97, 2, 9), (150, 3, 14), (211, 5, 20))):
        dem = native.fbm_dem(n, 7700 + k, octaves=6, range_max=9000)
        jobs[k] = (native.Params(nrows=n, roi=roi, height=25, ntests=32, bw=bw,
                                 nwanted0=max(1, n * n // 64), intervis=k % 2), dem)
    ctx.set_batch_mode(mode)
    try:
        out = ctx.run_batch([p for p, _ in jobs], [d for _, d in jobs])
    finally:
        ctx.set_batch_mode(0)
    for (p, dem), (obs, sel, res) in zip(jobs, out):
        _check_job(oracle, p, dem, obs, sel, res)


def test_batch_graph_replay_matches_eager_and_oracle(ctx, oracle, native):
    """The device-resident batch is captured as a CUDA graph on its first call
    and replayed on the next identical one; a changed buffer is captured
    anew; replays, eager launches and the oracle agree."""
    torch = pytest.importorskip("torch")
    jobs = _mixed_jobs(native, 6, 7)
    params = [p for p, _ in jobs]
    d_dems = [torch.from_numpy(d.view(np.int16)).cuda() for _, d in jobs]
    geos = [native.block_geometry(p.nrows, p.bw, p.nwanted0) for p in params]
    d_obs = [torch.empty(g.nwanted, dtype=torch.int32, device="cuda") for g in geos]
    d_sel = [torch.empty(g.nwanted, dtype=torch.uint8, device="cuda") for g in geos]
    torch.cuda.synchronize()
    c0, r0 = ctx.batch_graph_stats()
    res1 = ctx.run_batch_dev(params, d_dems, d_obs, d_sel)
    obs1 = [o.cpu().numpy() for o in d_obs]
    sel1 = [s.cpu().numpy() for s in d_sel]
    for o, s in zip(d_obs, d_sel):
        o.fill_(-1)
        s.fill_(7)
    torch.cuda.synchronize()
    res2 = ctx.run_batch_dev(params, d_dems, d_obs, d_sel)
    c1, r1 = ctx.batch_graph_stats()
    assert (c1, r1) == (c0 + 1, r0 + 1), "second identical call should replay the graph"
    for k in range(len(jobs)):
        assert np.array_equal(d_obs[k].cpu().numpy(), obs1[k])
        assert np.array_equal(d_sel[k].cpu().numpy(), sel1[k])
        assert (res1[k].nusedsheds, res1[k].cumarea) == (res2[k].nusedsheds, res2[k].cumarea)
    # a new output buffer for one job: captured again, same results
    d_sel[0] = torch.zeros_like(d_sel[0])
    ctx.run_batch_dev(params, d_dems, d_obs, d_sel)
    assert ctx.batch_graph_stats()[0] == c1 + 1
    assert np.array_equal(d_sel[0].cpu().numpy(), sel1[0])
    ctx.set_batch_graphs(False)
    try:
        res3 = ctx.run_batch_dev(params, d_dems, d_obs, d_sel)
    finally:
        ctx.set_batch_graphs(True)
    for k, ((p, dem), r) in enumerate(zip(jobs, res3)):
        assert (r.nusedsheds, r.cumarea) == (res1[k].nusedsheds, res1[k].cumarea)
        _check_job(oracle, p, dem, obs1[k], sel1[k], r)


def test_batch_knobs_reject_bad_values(ctx, native):
    for mode in (-1, 3):
        with pytest.raises(native.SitingError):
            ctx.set_batch_mode(mode)
    assert native.load().siting_ctx_set_batch_graphs(ctx.h, 2) == native.EINVAL
