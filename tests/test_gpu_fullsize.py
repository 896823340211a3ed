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
