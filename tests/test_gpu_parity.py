"""CUDA path vs the CPU oracle, bit for bit, through the C ABI.

Every stage (VIX bytes, observers and the VIX array FINDMAX leaves behind,
every viewshed word, the selection, the observer count and the covered-cell
count) must equal the oracle's on the same inputs; the oracle itself is pinned
to the reference by test_oracle.py.  Disagreeing cells / words are counted in
the failure message.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, dem_bin_path, make_dem

pytestmark = pytest.mark.gpu


def _diff(name, got, want):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape, f"{name}: shape {got.shape} != {want.shape}"
    bad = int(np.count_nonzero(got != want))
    assert bad == 0, f"{name}: {bad} of {want.size} entries differ (first at " \
                     f"{int(np.argmax(got != want))})"


def pytest_generate_tests(metafunc):
    if "gcase" in metafunc.fixturenames:
        import json

        from conftest import GOLDEN

        with open(GOLDEN) as f:
            cases = json.load(f)["cases"]
        metafunc.parametrize("gcase", cases, ids=[c["name"] for c in cases])


def test_stages_match_oracle(gcase, ctx, oracle, native):
    n, roi, h, ntests, bw, nw0, iv = gcase["args"]
    dem = make_dem(gcase["dem"], n)
    want = oracle.run(dem, n, roi, h, ntests, bw, nw0, iv)
    g = native.block_geometry(n, bw, nw0)

    vix = ctx.calc_vix(n, dem, roi, h, h, ntests)
    _diff("vix", vix, want["vix"])
    v2 = vix.copy()
    obs = ctx.find_max(n, v2, g.blocksize, g.nwanted, g.nblocks, g.nwantedperblock)
    _diff("obs", obs, want["obs"])
    _diff("vix after findmax", v2, want["vix_after"])
    sheds = ctx.calc_sheds(n, dem, roi, h, h, obs)
    _diff("sheds", sheds, want["sheds"])
    sel, res = ctx.site_it(n, roi, iv, obs, sheds)
    _diff("selected", sel, want["selected"])
    assert (res.nusedsheds, res.cumarea) == (want["nused"], want["cumarea"])
    # and the reference's own recorded outputs
    assert hashlib.sha256(sel.tobytes()).hexdigest() == gcase["selected_sha256"]


def test_pipeline_matches_oracle(gcase, ctx, oracle, native):
    n, roi, h, ntests, bw, nw0, iv = gcase["args"]
    dem = make_dem(gcase["dem"], n)
    p = native.Params(nrows=n, roi=roi, height=h, ntests=ntests, bw=bw, nwanted0=nw0, intervis=iv)
    obs, sel, res = ctx.run(p, dem)
    assert hashlib.sha256(obs.tobytes()).hexdigest() == gcase["obs_sha256"]
    assert hashlib.sha256(sel.tobytes()).hexdigest() == gcase["selected_sha256"]
    assert (res.nusedsheds, res.cumarea) == (gcase["nused"], gcase["cumarea"])
    assert hashlib.md5(native.observers_text(obs, sel, n)).hexdigest() == gcase["observers_md5"]


@pytest.mark.parametrize("iv,md5", [(0, "0f0e2cd59b33eaa3dbeae4f78d261f05"),
                                    (1, "ff6affb15ab1f99489f8cafb79a84701")])
def test_cli_known_answers_on_sample_dem(native, tmp_path, iv, md5):
    path = dem_bin_path()
    if path is None:
        pytest.skip("dem.bin not available on this machine")
    out = tmp_path / "observers.txt"
    r = subprocess.run([native.CLI_PATH, "1000", "50", "100", "50", "10", "10000", str(iv), path,
                        str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert hashlib.md5(out.read_bytes()).hexdigest() == md5
    keys = [tok.split(":")[0] for tok in r.stdout.split()]
    assert keys == ["input", "vix", "findmax", "viewshed", "nusedsheds", "coverage", "site",
                    "output", "total"]


def test_cli_synthetic_matches_oracle(native, oracle, tmp_path):
    n = 320
    dem = native.fbm_dem(n, 77, octaves=7, range_max=8000)
    dem.tofile(tmp_path / "d.bin")
    r = subprocess.run([native.CLI_PATH] + [str(v) for v in (n, 24, 20, 30, 10, 900, 1)] +
                       ["d.bin", "o.txt"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout
    want = oracle.run(dem, n, 24, 20, 30, 10, 900, 1)
    assert (tmp_path / "o.txt").read_bytes() == native.observers_text(want["obs"],
                                                                      want["selected"], n)
    assert f"nusedsheds:{want['nused']} " in r.stdout


def test_run_dev_device_buffers(ctx, oracle, native):
    torch = pytest.importorskip("torch")
    n, roi, h, ntests, bw, nw0, iv = 264, 22, 18, 28, 12, 400, 1
    dem = native.fbm_dem(n, 31, octaves=7, range_max=7000)
    want = oracle.run(dem, n, roi, h, ntests, bw, nw0, iv)
    g = native.block_geometry(n, bw, nw0)
    d_dem = torch.from_numpy(dem.view(np.int16)).cuda()
    d_obs = torch.empty(g.nwanted, dtype=torch.int32, device="cuda")
    d_sel = torch.empty(g.nwanted, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    p = native.Params(nrows=n, roi=roi, height=h, ntests=ntests, bw=bw, nwanted0=nw0, intervis=iv)
    res = ctx.run_dev(p, d_dem, d_obs, d_sel)
    ctx.sync()
    _diff("obs", d_obs.cpu().numpy(), want["obs"])
    _diff("selected", d_sel.cpu().numpy(), want["selected"])
    assert (res.nusedsheds, res.cumarea) == (want["nused"], want["cumarea"])


@pytest.mark.parametrize("n", [257, 250, 1])
def test_unaligned_and_tiny_dems_dev(ctx, oracle, native, n):
    """Rows whose byte length is not a multiple of 16 go through the pitched copy."""
    torch = pytest.importorskip("torch")
    roi, h, ntests = 13, 9, 21
    dem = native.fbm_dem(n, 5 + n, octaves=6, range_max=5000)
    want = oracle.vix(dem, n, roi, h, h, ntests)
    d_dem = torch.from_numpy(dem.view(np.int16)).cuda()
    d_vix = torch.empty(n * n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.calc_vix_dev(n, d_dem, roi, h, h, ntests, d_vix)
    ctx.sync()
    _diff("vix", d_vix.cpu().numpy(), want)


@pytest.mark.parametrize("roi", [1, 2, 3, 59, 60, 64, 100, 104, 127, 130, 151, 152, 200])
def test_viewshed_roi_range(ctx, oracle, native, roi):
    """Default plans: whole windows staged (roi < 60), half windows staged
    (roi 60..151, three launch shapes), whole windows through L1 (larger)."""
    n = 300
    dem = native.fbm_dem(n, roi, octaves=7, range_max=9000)
    rng = np.random.default_rng(roi)
    obs = np.sort(rng.choice(n * n, 40, replace=False)).astype(np.int32)
    obs[:4] = [0, n - 1, n * n - 1, n * (n - 1)]  # corners
    obs[4:8] = [n // 2, n * (n // 2), n * (n // 2) + n - 1, n * (n - 1) + n // 2]  # edge midpoints
    want = oracle.sheds(dem, n, roi, 30, 30, obs)
    got = ctx.calc_sheds(n, dem, roi, 30, 30, obs)
    _diff("sheds", got, want)


@pytest.mark.parametrize("roi", [1, 5, 50, 100, 120])
def test_viewshed_window_forms_agree(ctx, oracle, native, roi):
    """Half windows, the whole window staged and the whole window through L1
    (plans 1, 2 and 0) give the oracle's sheds, on a flat-topped DEM whose
    ties and horizontal sight lines stress the row shared by the halves."""
    n = 260
    dem = native.fbm_dem(n, 7 * roi, octaves=6, range_max=3000)
    dem.reshape(n, n)[100:160, 90:170] = 1500  # a plateau: equal elevations along straight rays
    rng = np.random.default_rng(roi + 1)
    obs = np.sort(rng.choice(n * n, 24, replace=False)).astype(np.int32)
    obs[:3] = [130 * n + 130, 100 * n + 90, 159 * n + 169]
    obs.sort()
    want = oracle.sheds(dem, n, roi, 12, 12, obs)
    for smem in (1, 2, 0):
        ctx.autotune_clear()
        ctx.autotune_set(roi, 1, native.Plan(shed_smem=smem))
        _diff(f"sheds (plan {smem})", ctx.calc_sheds(n, dem, roi, 12, 12, obs), want)
    ctx.autotune_clear()
    with pytest.raises(native.SitingError):
        ctx.autotune_set(roi, 1, native.Plan(shed_smem=3))


@pytest.mark.parametrize("roi,ntests", [(1, 1), (3, 1000), (124, 40), (160, 33)])
def test_vix_parameter_range(ctx, oracle, native, roi, ntests):
    n = 180
    dem = native.fbm_dem(n, 1000 + roi, octaves=7, range_max=20000)
    _diff("vix", ctx.calc_vix(n, dem, roi, 7, 3, ntests), oracle.vix(dem, n, roi, 7, 3, ntests))


@pytest.mark.parametrize("iv", [0, 1])
def test_site_stage_on_any_observer_order(ctx, oracle, native, iv):
    """site_it on candidates in arbitrary order (no block structure)."""
    n, roi = 220, 18
    dem = native.fbm_dem(n, 61, octaves=7, range_max=6000)
    rng = np.random.default_rng(iv)
    obs = rng.choice(n * n, 700, replace=False).astype(np.int32)
    sheds = oracle.sheds(dem, n, roi, 12, 12, obs)
    want_sel, want_n, want_c = oracle.site(n, roi, iv, obs, sheds)
    sel, res = ctx.site_it(n, roi, iv, obs, sheds)
    _diff("selected", sel, want_sel)
    assert (res.nusedsheds, res.cumarea) == (want_n, want_c)


def test_site_cta_count_does_not_change_results(ctx, oracle, native):
    n, roi, h, ntests, bw, nw0, iv = 400, 30, 25, 24, 10, 1600, 1
    dem = native.fbm_dem(n, 88, octaves=8, range_max=9000)
    p = native.Params(nrows=n, roi=roi, height=h, ntests=ntests, bw=bw, nwanted0=nw0, intervis=iv)
    want = oracle.run(dem, n, roi, h, ntests, bw, nw0, iv)
    try:
        for G in (1, 3, 16, 150):
            ctx.set_site_ctas(G)
            obs, sel, res = ctx.run(p, dem)
            _diff(f"selected G={G}", sel, want["selected"])
            assert res.cumarea == want["cumarea"]
    finally:
        ctx.set_site_ctas(0)


def test_hbm_budget_refusal(native):
    with native.Context(0, hbm_budget=1 << 20) as c:
        p = native.Params(nrows=512, roi=20, height=10, ntests=8, bw=16, nwanted0=1024)
        dem = native.fbm_dem(512, 1)
        with pytest.raises(native.SitingError) as e:
            c.run(p, dem)
        assert e.value.status == 2 and "budget" in e.value.message


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_waits_expire_and_context_survives(native, which):
    """A wait whose condition is never met gives up after its limit, the host
    reads SITING_ETIMEOUT, and the same context then runs a job normally."""
    p = native.Params(nrows=128, roi=10, height=20, ntests=16, bw=16, nwanted0=64)
    dem = native.fbm_dem(128, 5)
    with native.Context(0) as c:
        assert c.selftest_wait(which, 1 << 22) == native.ETIMEOUT
        obs, sel, res = c.run(p, dem)
        obs2, sel2, _ = native.Context(0).run(p, dem)
        assert np.array_equal(obs, obs2) and np.array_equal(sel, sel2)
