"""The allocation-free SITE entry point against the regular one.

siting_site_it_noalloc serves callers that cannot allocate device memory on
their call path, such as a serving loop that reserves its whole HBM budget at
start-up, or an application whose memory pool (PyTorch's caching allocator,
for instance) already owns the GPU's memory.  It takes its scratch from a
fixed array in the library's device image instead.  Its results must equal
those of siting_site_it_dev, which allocates its workspace, bit for bit (and
both the CPU oracle's selection); two calls in a row check that the shared
array is reset between calls.

This file is collected last so that a stop-at-first-failure run has already
run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(native, oracle, n, roi, h, ntests, bw, nw0, seed):
    dem = native.fbm_dem(n, seed, octaves=7, range_max=8000)
    want = oracle.run(dem, n, roi, h, ntests, bw, nw0, 0)
    return want["obs"], want["sheds"]


def _oracle_selection(oracle, n, roi, iv, obs, sheds):
    """The CPU oracle's SITE on the same candidates (seqsite semantics)."""
    sel, nused, cumarea = oracle.site(n, roi, iv, obs, sheds)[:3]
    return sel, nused, cumarea


@pytest.mark.parametrize("iv", [0, 1])
def test_noalloc_site_matches_allocating_entry(native, oracle, iv):
    torch = pytest.importorskip("torch")
    n, roi = 360, 22
    obs, sheds = _case(native, oracle, n, roi, 18, 24, 12, 900, 404 + iv)
    torch.cuda.set_device(0)
    d_obs = torch.from_numpy(obs).cuda()
    d_sheds = torch.from_numpy(sheds.view(np.int64)).cuda()
    d_sel_ref = torch.empty(len(obs), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    with native.Context(0) as ctx:
        ref = ctx.site_it_dev(n, roi, iv, len(obs), d_obs, d_sheds, d_sel_ref)
        ctx.sync()
    sel_ref = d_sel_ref.cpu().numpy()
    assert ref.nusedsheds == int(sel_ref.sum()) > 0
    # and both against the CPU oracle
    sel_o, nused_o, cum_o = _oracle_selection(oracle, n, roi, iv, obs, sheds)
    assert np.array_equal(sel_ref, sel_o) and (ref.nusedsheds, ref.cumarea) == (nused_o, cum_o)

    lib = native.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # the second call reuses the shared scratch array
        d_sel = torch.full((len(obs),), 7, dtype=torch.uint8, device="cuda")
        res = native._ResultC()
        rc = lib.siting_site_it_noalloc(n, roi, iv, len(obs), d_obs.data_ptr(),
                                        d_sheds.data_ptr(), d_sel.data_ptr(), stream,
                                        C.byref(res))
        assert rc == 0, f"call {call}: status {rc}"
        sel = d_sel.cpu().numpy()
        assert np.array_equal(sel, sel_ref), f"call {call}: selection differs"
        assert (res.nusedsheds, res.cumarea) == (ref.nusedsheds, ref.cumarea), f"call {call}"


def test_noalloc_rejects_jobs_beyond_its_scratch(native):
    torch = pytest.importorskip("torch")
    # a 20000^2 coverage bitmap alone needs 50 MB, beyond the 16 MiB array
    d = torch.zeros(16, dtype=torch.int64, device="cuda")
    res = native._ResultC()
    rc = native.load().siting_site_it_noalloc(20000, 10, 0, 1, d.data_ptr(), d.data_ptr(),
                                              d.data_ptr(), None, C.byref(res))
    assert rc == 2  # SITING_ENOMEM


def test_noalloc_flags_bad_observer_indices_before_site(native):
    torch = pytest.importorskip("torch")
    # one index past the DEM and one negative: the index check runs before
    # SITE and the call returns SITING_EINVAL without reading through them
    n, roi = 64, 5
    nr = 2 * roi + 1
    obs = torch.tensor([0, n * n + 5, 7, -3], dtype=torch.int32, device="cuda")
    sheds = torch.zeros(len(obs) * nr, dtype=torch.int64, device="cuda")
    sel = torch.full((len(obs),), 7, dtype=torch.uint8, device="cuda")
    res = native._ResultC()
    rc = native.load().siting_site_it_noalloc(n, roi, 0, len(obs), obs.data_ptr(),
                                              sheds.data_ptr(), sel.data_ptr(), None,
                                              C.byref(res))
    assert rc == 1  # SITING_EINVAL
    assert res.nusedsheds == 0 and int(sel.sum().item()) == 0
