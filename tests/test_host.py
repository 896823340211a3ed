"""Host-side logic of the native library and CLI (no GPU needed)."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def header_functions():
    with open(os.path.join(ROOT, "include", "siting.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(siting_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(native):
    lib = native.load()
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("field,value,msg", [
    ("nrows", 0, "Unreasonable value for nrows"),
    ("nrows", 20001, "Unreasonable value for nrows"),
    ("roi", 0, "Unreasonable value for roi."),
    ("roi", 10001, "Unreasonable value for roi."),
    ("height", -1, "Unreasonable value for tht."),
    ("height", 1000001, "Unreasonable value for tht."),
    ("ntests", 0, "Unreasonable value for ntests."),
    ("ntests", 1001, "Unreasonable value for ntests."),
    ("bw", 9, "Unreasonable value for blocksize0."),
    ("bw", 2001, "Unreasonable value for blocksize0."),
    ("nwanted0", 99, "Unreasonable value for nwanted0."),
    ("nwanted0", 2000001, "Unreasonable value for nwanted0."),
    ("intervis", 2, "Unreasonable value for intervis."),
])
def test_validation_messages_match_reference(native, field, value, msg):
    """siting.cpp:680-686: same checks, same messages (CLI form)."""
    p = native.Params(nrows=1000, roi=50, height=100, ntests=50, bw=10, nwanted0=10000)
    setattr(p, field, value)
    assert native.validate(p, lib_form=False) == msg


def test_last_block_too_small(native):
    p = native.Params(nrows=100, roi=5, height=1, ntests=5, bw=10, nwanted0=2000000)
    assert native.validate(p, lib_form=False) == \
        "The last block is too small for nwantedperblock."


def test_library_form_accepts_small_bw(native):
    p = native.Params(nrows=512, roi=25, height=20, ntests=32, bw=8, nwanted0=4096)
    assert native.validate(p, lib_form=False) == "Unreasonable value for blocksize0."
    assert native.validate(p, lib_form=True) is None


@pytest.mark.parametrize("n,bw,nw", [(1000, 10, 10000), (4096, 16, 65536), (16384, 32, 262144),
                                     (999, 13, 7777), (257, 11, 500), (2048, 32, 65536),
                                     (1531, 8, 36624), (100, 20, 300), (3000, 2000, 100)])
def test_geometry_matches_oracle(native, oracle, n, bw, nw):
    g = native.block_geometry(n, bw, nw)
    o = oracle.geometry(n, bw, nw)
    assert (g.blocksize, g.nblocks, g.nwantedperblock, g.nwanted) == \
        (o.blocksize, o.nblocks, o.nwantedperblock, o.nwanted)


def test_fbm_is_deterministic(native, golden):
    a = native.fbm_dem(300, 9, octaves=8)
    b = native.fbm_dem(300, 9, octaves=8)
    c = native.fbm_dem(300, 10, octaves=8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() == 0 and a.max() == 10000
    # the fixture DEMs regenerate byte for byte
    for case in golden["cases"]:
        spec = case["dem"]
        if "seed" not in spec:
            continue
        n = case["args"][0]
        kw = {k: v for k, v in spec.items() if k != "seed"}
        d = native.fbm_dem(n, spec["seed"], **kw)
        assert hashlib.sha256(d.tobytes()).hexdigest() == case["dem_sha256"], case["name"]


def test_observer_file_format(native, tmp_path):
    obs = np.array([5, 1003, 2999, 7], np.int32)
    sel = np.array([1, 0, 1, 1], np.uint8)
    p = tmp_path / "o.txt"
    native.write_observers(str(p), 1000, obs, sel)
    assert p.read_bytes() == b"0,5\n2,999\n0,7\n" == native.observers_text(obs, sel, 1000)


def test_read_dem_round_trip_and_short_file(native, tmp_path):
    d = native.fbm_dem(64, 3)
    p = tmp_path / "d.bin"
    d.tofile(p)
    assert np.array_equal(native.read_dem(str(p), 64), d)
    with pytest.raises(native.SitingError):
        native.read_dem(str(p), 65)


def _cli(args, cwd):
    return subprocess.run([os.path.join(ROOT, "siting_gb300", "cusite")] + [str(a) for a in args],
                          capture_output=True, text=True, cwd=cwd)


def test_cli_argument_errors(native, tmp_path):
    r = _cli(["1000", "50"], tmp_path)
    assert r.returncode == 1
    assert r.stdout.splitlines() == [
        "argc=3",
        "ERROR: SITE requires 9 arguments: nrows, roi, oht/tht, ntests, blocksize, nwanted, "
        "intervis, infile, outfile"]
    r = _cli([0, 50, 100, 50, 10, 10000, 0, "in", "out"], tmp_path)
    assert (r.returncode, r.stdout) == (1, "ERROR: Unreasonable value for nrows\n")
    r = _cli([100, 50, 100, 50, 8, 10000, 0, "in", "out"], tmp_path)
    assert (r.returncode, r.stdout) == (1, "ERROR: Unreasonable value for blocksize0.\n")
    r = _cli([100, 50, 100, 50, 10, 10000, 0, "missing.bin", "out"], tmp_path)
    assert (r.returncode, r.stdout.splitlines()[-1]) == (1, "ERROR: Input failed")


def test_trunc_based_round_matches_roundf():
    """The kernels' (int)roundf(v) is trunc(v + copysign(0.5 - 2^-25, v)) in
    FP32.  Checked here against exact half-away-from-zero rounding (in
    float64) on every float near a half-integer below 2^12 and on a random
    sample of all floats below 2^31."""
    rng = np.random.default_rng(7)
    halves = (np.arange(-4096, 4096, dtype=np.float64) + 0.5).astype(np.float32)
    near = halves.view(np.int32)[:, None] + np.arange(-64, 65, dtype=np.int32)[None, :]
    bits = rng.integers(0, 2**32, size=4_000_000, dtype=np.uint64).astype(np.uint32)
    v = np.concatenate([near.ravel().view(np.float32), bits.view(np.float32)])
    v = v[np.isfinite(v) & (np.abs(v) < 2.0**31 - 128)]
    h = np.where(np.signbit(v), np.float32(-0.49999997), np.float32(0.49999997)).astype(np.float32)
    got = np.trunc(v + h).astype(np.int64)  # float32 + float32: one IEEE rounding
    x = v.astype(np.float64)
    want = (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)
    assert np.array_equal(got, want)


def test_server_refuses_without_device(native):
    """Without a usable GPU the serving loop reports EDEVICE instead of
    falling back to anything else."""
    try:
        native.Context(0).close()
        pytest.skip("a GPU is present")
    except native.SitingError:
        pass
    with pytest.raises(native.SitingError) as e:
        native.Server(0, hbm_budget=1 << 30)
    assert e.value.status == native.EDEVICE


def test_noalloc_site_checks_arguments_on_the_host(native):
    """The allocation-free SITE entry point rejects bad arguments before any
    device work, and an empty job succeeds without touching a device."""
    import ctypes as C

    lib = native.load()
    res = native._ResultC()
    res.nusedsheds = 99
    buf = C.c_void_p(16)  # never dereferenced: every call below returns first
    for args in [(0, 10, 0, 1), (20001, 10, 0, 1), (100, 0, 0, 1), (100, 10, 2, 1),
                 (100, 10, 0, -1)]:
        assert lib.siting_site_it_noalloc(*args, buf, buf, buf, None, C.byref(res)) == 1
    assert lib.siting_site_it_noalloc(100, 10, 0, 5, None, buf, buf, None, C.byref(res)) == 1
    assert lib.siting_site_it_noalloc(100, 10, 1, 0, None, None, None, None, C.byref(res)) == 0
    assert (res.nusedsheds, res.cumarea, res.site_rounds) == (0, 0, 0)


def test_batch_knobs_reject_a_missing_context(native):
    """The batched form's knobs check their context before anything else."""
    import ctypes as C

    lib = native.load()
    c, r = C.c_longlong(), C.c_longlong()
    assert lib.siting_ctx_set_batch_mode(None, 1) == native.EINVAL
    assert lib.siting_ctx_set_batch_graphs(None, 1) == native.EINVAL
    assert lib.siting_ctx_batch_graph_stats(None, C.byref(c), C.byref(r)) == native.EINVAL


def test_autotune_set_checks_its_arguments(native):
    """A pinned plan needs a context and fields in range (no device work)."""
    import ctypes as C

    lib = native.load()
    pc = native.Plan(shed_smem=2).c()
    assert lib.siting_autotune_set(None, 100, 16, C.byref(pc)) == native.EINVAL
