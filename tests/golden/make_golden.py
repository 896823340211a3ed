"""Generates tests/golden/golden.json from the reference itself.

Run where the reference sources are available (they are compiled from their
own files by oracle/Makefile into oracle/_ref/libsitingref.so, seqsite
semantics):

    python tests/golden/make_golden.py

Each case is a seeded synthetic DEM (siting_gb300.fbm_dem, or a flat DEM) plus
the nine CLI parameters.  For each, the reference's outputs of every stage are
recorded as sha256 digests (VIX bytes, observers, every viewshed word, the
selection), with the observer count, the covered-cell count and the md5 of the
observers file.  The reference's sample DEM (dem.bin) is recorded the same way
when it is present.

The full-size cases (key "fullsize": the 4096^2 workload, roi 100, 65 536
observers, intervis 1) take minutes of sequential reference time each; they
are (re)generated alone with

    python tests/golden/make_golden.py --fullsize

which keeps the small cases as they are.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle_bind import Oracle, observers_text, ref_dem_bin  # noqa: E402

# (name, dem spec, nrows, roi, height, ntests, bw, nwanted0, intervis)
CASES = [
    ("fbm96_iv0", {"seed": 1, "octaves": 6, "range_max": 2000}, 96, 12, 10, 16, 10, 64, 0),
    ("fbm96_iv1", {"seed": 1, "octaves": 6, "range_max": 2000}, 96, 12, 10, 16, 10, 64, 1),
    ("fbm128_bw8", {"seed": 2, "octaves": 7, "range_max": 5000}, 128, 30, 5, 40, 8, 400, 1),
    ("roi_over_n", {"seed": 3, "octaves": 5, "range_max": 1500}, 64, 80, 20, 10, 16, 64, 0),
    ("flat80", {"flat": 1000}, 80, 10, 1, 8, 10, 100, 0),
    ("zero64_h0_iv1", {"flat": 0}, 64, 9, 0, 12, 10, 100, 1),
    ("npb12_iv1", {"seed": 4, "octaves": 6, "range_max": 4000}, 100, 15, 12, 20, 20, 300, 1),
    ("ridged200", {"seed": 5, "octaves": 8, "range_max": 9000, "ridged_weight": 0.3}, 200, 25, 30,
     32, 16, 256, 0),
    ("odd257_iv1", {"seed": 6, "octaves": 8, "range_max": 12000}, 257, 17, 25, 24, 11, 500, 1),
    ("c1_fbm1000", {"seed": 11, "octaves": 8, "range_max": 10000}, 1000, 50, 100, 50, 10, 10000, 0),
]



# The full-size workloads: (name, dem spec, nrows, roi, height, ntests, bw,
# nwanted0, intervis).  c2_4096 is the benchmark's headline job: 4096^2 fBm
# with 10 octaves and ridged noise at weight 0.3, range 0-30000.
FULLSIZE = [
    ("c2_4096", {"seed": 4096, "octaves": 10, "ridged_weight": 0.3, "range_max": 30000},
     4096, 100, 200, 100, 16, 65536, 1),
]


def make_dem(spec, n):
    if "flat" in spec:
        return np.full(n * n, spec["flat"], np.uint16)
    import siting_gb300 as sg
    kw = {k: v for k, v in spec.items() if k != "seed"}
    return sg.fbm_dem(n, spec["seed"], **kw)


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def record(orc: Oracle, dem, n, roi, h, ntests, bw, nw0, iv):
    r = orc.run(dem, n, roi, h, ntests, bw, nw0, iv)
    g = r["geo"]
    return {
        "dem_sha256": sha(dem),
        "nwanted": g.nwanted,
        "vix_sha256": sha(r["vix"]),
        "vix_sum": int(r["vix"].sum(dtype=np.int64)),
        "obs_sha256": sha(r["obs"]),
        "sheds_sha256": sha(r["sheds"]),
        "shed_bits": int(np.bitwise_count(r["sheds"]).sum(dtype=np.int64)),
        "selected_sha256": sha(r["selected"]),
        "nused": int(r["nused"]),
        "cumarea": int(r["cumarea"]),
        "observers_md5": hashlib.md5(observers_text(r["obs"], r["selected"], n)).hexdigest(),
    }


def fullsize(orc: Oracle):
    path = os.path.join(HERE, "golden.json")
    with open(path) as f:
        out = json.load(f)
    out["fullsize"] = []
    for name, spec, n, roi, h, ntests, bw, nw0, iv in FULLSIZE:
        dem = make_dem(spec, n)
        rec = record(orc, dem, n, roi, h, ntests, bw, nw0, iv)
        rec.update(name=name, dem=spec, args=[n, roi, h, ntests, bw, nw0, iv])
        out["fullsize"].append(rec)
        print(name, rec["nused"], rec["cumarea"], rec["observers_md5"], flush=True)
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


def main():
    orc = Oracle("reference")
    if "--fullsize" in sys.argv:
        fullsize(orc)
        return
    out = {"generator": "reference siting.cpp built -DSEQ -ffp-contract=off (oracle/Makefile ref)",
           "cases": []}
    for name, spec, n, roi, h, ntests, bw, nw0, iv in CASES:
        dem = make_dem(spec, n)
        rec = record(orc, dem, n, roi, h, ntests, bw, nw0, iv)
        rec.update(name=name, dem=spec, args=[n, roi, h, ntests, bw, nw0, iv])
        out["cases"].append(rec)
        print(name, rec["nused"], rec["cumarea"], flush=True)
    if ref_dem_bin():
        dem = np.fromfile(ref_dem_bin(), np.uint16)
        for iv in (0, 1):
            rec = record(orc, dem, 1000, 50, 100, 50, 10, 10000, iv)
            rec.update(name=f"dem_bin_iv{iv}", dem={"file": "dem.bin"},
                       args=[1000, 50, 100, 50, 10, 10000, iv])
            out["cases"].append(rec)
            print(rec["name"], rec["nused"], rec["cumarea"], rec["observers_md5"], flush=True)
    path = os.path.join(HERE, "golden.json")
    if os.path.exists(path):
        with open(path) as f:
            out["fullsize"] = json.load(f).get("fullsize", [])
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
