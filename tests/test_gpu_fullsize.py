"""The 16384^2 workload (roi 200, 64 targets, bw 32, 262 144 observers,
intervis 0) at full size: too large for the oracle end to end on the CPU, so
each stage is checked through properties that do not depend on the size.

* VIX: 20 000 random cells recomputed by the oracle, bit for bit;
* FINDMAX: the oracle's FINDMAX over the GPU's full VIX raster gives the same
  observers and the same zeroed VIX;
* VIEWSHED: 1 500 random observers' sheds recomputed by the oracle;
* SITE: the oracle's greedy selection over the GPU's 5.9 GB of sheds gives
  the same selection, observer count and covered cells, and the covered cells
  equal the union of the selected sheds.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, ROI, HEIGHT, NTESTS, BW, NWANTED0, INTERVIS = 16384, 200, 150, 64, 32, 262144, 0


def test_c4_16384_stagewise(native, oracle, ctx):
    torch = pytest.importorskip("torch")
    if torch.cuda.get_device_properties(0).total_memory < (24 << 30):
        pytest.skip("needs ~10 GB of device memory")
    dem = native.fbm_dem(N, 16384, octaves=12, range_max=40000)
    geo = native.block_geometry(N, BW, NWANTED0)
    nr = 2 * ROI + 1
    per = nr * ((nr + 63) // 64)
    d_dem = torch.from_numpy(dem.view(np.int16)).cuda()
    d_vix = torch.empty(N * N, dtype=torch.uint8, device="cuda")
    d_obs = torch.empty(geo.nwanted, dtype=torch.int32, device="cuda")
    d_sheds = torch.empty(geo.nwanted * per, dtype=torch.int64, device="cuda")
    d_sel = torch.empty(geo.nwanted, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    ctx.calc_vix_dev(N, d_dem, ROI, HEIGHT, HEIGHT, NTESTS, d_vix)
    ctx.sync()
    vix = d_vix.cpu().numpy()
    rng = np.random.default_rng(16384)
    cells = rng.integers(0, N * N, size=20000)
    want = oracle.vix_cells(dem, N, ROI, HEIGHT, HEIGHT, NTESTS, cells)
    assert np.array_equal(vix[cells], want), \
        f"VIX differs at {int(np.count_nonzero(vix[cells] != want))} of 20000 sampled cells"

    ctx.find_max_dev(N, d_vix, geo.blocksize, geo.nwanted, geo.nblocks, geo.nwantedperblock, d_obs)
    ctx.sync()
    o_geo = oracle.geometry(N, BW, NWANTED0)
    want_obs, want_vix = oracle.find_max(vix, N, o_geo)
    obs = d_obs.cpu().numpy()
    assert np.array_equal(obs, want_obs)
    assert np.array_equal(d_vix.cpu().numpy(), want_vix)

    ctx.calc_sheds_dev(N, d_dem, ROI, HEIGHT, HEIGHT, geo.nwanted, d_obs, d_sheds)
    ctx.sync()
    sheds = d_sheds.cpu().numpy().view(np.uint64)
    pick = np.sort(rng.choice(geo.nwanted, size=1500, replace=False))
    want_sh = oracle.sheds(dem, N, ROI, HEIGHT, HEIGHT, obs[pick]).reshape(len(pick), per)
    got_sh = sheds.reshape(geo.nwanted, per)[pick]
    bad = np.nonzero((got_sh != want_sh).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} of 1500 sampled viewsheds differ (first: observer {pick[bad[0]]})"

    res = ctx.site_it_dev(N, ROI, INTERVIS, geo.nwanted, d_obs, d_sheds, d_sel)
    sel = d_sel.cpu().numpy()
    want_sel, nused, cumarea = oracle.site(N, ROI, INTERVIS, obs, sheds)[:3]
    assert np.array_equal(sel, want_sel)
    assert (res.nusedsheds, res.cumarea) == (nused, cumarea)
    assert oracle.union_count(N, ROI, obs, sheds, sel) == cumarea
    assert 100.0 * cumarea / (N * N) > 95.0


def _bit_count(a):
    """Set bits of an array (numpy >= 2 has a vectorised popcount)."""
    if hasattr(np, "bitwise_count"):
        return int(np.bitwise_count(a).sum(dtype=np.int64))
    table = np.array([bin(i).count("1") for i in range(256)], np.int64)
    return int(table[np.ascontiguousarray(a).view(np.uint8)].sum())


def _fullsize_case(golden, name):
    for c in golden.get("fullsize", []):
        if c["name"] == name:
            return c
    pytest.skip(f"no full-size fixture {name}")


def test_c2_4096_matches_reference_outputs(native, ctx, golden):
    """The benchmark's headline job (4096^2 fBm + ridged noise, roi 100, 100
    targets, bw 16, 65 536 observers, intervis 1) against the outputs the
    reference's own seqsite recorded for it: every stage's bytes (VIX,
    observers, every viewshed word, selection), the observer count, the
    covered cells and the observers file (siting.cpp:501-626 at intervis 1,
    where the multi-pick rounds and the intervis cut are stressed hardest)."""
    import hashlib

    c = _fullsize_case(golden, "c2_4096")
    n, roi, h, ntests, bw, nw0, iv = c["args"]
    spec = {k: v for k, v in c["dem"].items() if k != "seed"}
    dem = native.fbm_dem(n, c["dem"]["seed"], **spec)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    assert sha(dem) == c["dem_sha256"], "input DEM differs from the fixture's"
    g = native.block_geometry(n, bw, nw0)
    assert g.nwanted == c["nwanted"]

    vix = ctx.calc_vix(n, dem, roi, h, h, ntests)
    assert int(vix.sum(dtype=np.int64)) == c["vix_sum"]
    assert sha(vix) == c["vix_sha256"], "VIX differs from the reference's"
    obs = ctx.find_max(n, vix.copy(), g.blocksize, g.nwanted, g.nblocks, g.nwantedperblock)
    assert sha(obs) == c["obs_sha256"], "observers differ from the reference's"
    sheds = ctx.calc_sheds(n, dem, roi, h, h, obs)
    assert _bit_count(sheds) == c["shed_bits"]
    assert sha(sheds) == c["sheds_sha256"], "viewsheds differ from the reference's"
    sel, res = ctx.site_it(n, roi, iv, obs, sheds)
    assert (res.nusedsheds, res.cumarea) == (c["nused"], c["cumarea"])
    assert sha(sel) == c["selected_sha256"], "selection differs from the reference's"

    # and the whole pipeline in one call, as the benchmark runs it
    p = native.Params(nrows=n, roi=roi, height=h, ntests=ntests, bw=bw, nwanted0=nw0, intervis=iv)
    obs2, sel2, res2 = ctx.run(p, dem)
    assert sha(obs2) == c["obs_sha256"] and sha(sel2) == c["selected_sha256"]
    assert (res2.nusedsheds, res2.cumarea) == (c["nused"], c["cumarea"])
    assert hashlib.md5(native.observers_text(obs2, sel2, n)).hexdigest() == c["observers_md5"]
