"""Benchmark: DEM cells/s of the VIX -> FINDMAX -> VIEWSHED -> SITE pipeline.

Workload (default): one 4096 x 4096 uint16 DEM, seeded fBm (10 octaves,
persistence 0.5, lacunarity 2, base wavelength 256) blended with ridged noise
at weight 0.3, range 0-30000; roi=100, height=200, targets=100, bw=16,
nwanted=65536, intervis=1.

One step = one whole siting job.  `value` is n^2 / device time with the DEM
resident in HBM (siting_run_dev); `e2e` is the same metric through
siting_run with page-locked host buffers (DEM upload and observer/selection
download inside the timed region).  Between timed steps the L2 is flushed by
writing a 512 MiB buffer.  Under torchrun each rank runs an independent
replica (its own DEM seed): value = all ranks' cells / max rank time.

`--impl reference` times the reference's own CPU implementation (siting.cpp
built with OpenMP from its staged sources, in library form, every host
thread) on the same whole workload, without loading this library; its line
also carries one run of `ompsite` as the reference's makefile builds it
(50 threads, hard-coded).  The default line's `cpu_baseline` is one whole
job of the same library-form run.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c2_4096": dict(nrows=4096, roi=100, height=200, ntests=100, bw=16, nwanted0=65536,
                    intervis=1, octaves=10, ridged=0.3, range_max=30000, seed=4096),
    "c2_2048": dict(nrows=2048, roi=100, height=200, ntests=100, bw=16, nwanted0=16384,
                    intervis=1, octaves=10, ridged=0.3, range_max=30000, seed=2048),
    "c1_1000": dict(nrows=1000, roi=50, height=100, ntests=50, bw=10, nwanted0=10000,
                    intervis=0, octaves=8, ridged=0.0, range_max=10000, seed=1000),
    "c4_16384": dict(nrows=16384, roi=200, height=150, ntests=64, bw=32, nwanted0=262144,
                     intervis=0, octaves=12, ridged=0.0, range_max=40000, seed=16384),
    # a small job for quick checks of the harness itself
    "fbm_256": dict(nrows=256, roi=20, height=30, ntests=32, bw=16, nwanted0=256,
                    intervis=1, octaves=7, ridged=0.0, range_max=5000, seed=256),
}
METRIC = "DEM cells/s end-to-end"

# The batched workload: 64 DEMs, sides log-uniform in [512, 2048] rounded to a
# multiple of 32, amplitude U[2000, 30000], roi U[25, 150], height U[20, 300],
# targets in {32, 64, 128}, bw in {8, 16, 32}, nwanted = cells/64, intervis
# alternating, one seed per DEM.
def batch_jobs(njobs=64, seed=64, lo=512, hi=2048):
    import siting_gb300 as sg

    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(njobs):
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))) / 32)) * 32
        amp = int(rng.integers(2000, 30001))
        p = sg.Params(nrows=n, roi=int(rng.integers(25, 151)), height=int(rng.integers(20, 301)),
                      ntests=int(rng.choice([32, 64, 128])), bw=int(rng.choice([8, 16, 32])),
                      nwanted0=n * n // 64, intervis=j % 2)
        jobs.append((p, dict(seed=seed * 1000 + j, range_max=amp)))
    return jobs


def make_dem(w, seed_offset=0):
    import siting_gb300 as sg

    return sg.fbm_dem(w["nrows"], w["seed"] + seed_offset, octaves=w["octaves"],
                      ridged_weight=w["ridged"], range_max=w["range_max"])


def params(w):
    import siting_gb300 as sg

    return sg.Params(nrows=w["nrows"], roi=w["roi"], height=w["height"], ntests=w["ntests"],
                     bw=w["bw"], nwanted0=w["nwanted0"], intervis=w["intervis"])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def site_algorithmic_bytes(nrows, roi, obs, order, nsheds):
    """Reference SITE traffic (the rescoring work of siting.cpp:537-604).

    Sum over rounds of, for every rescored candidate, its shed (nr*nwpr words)
    plus its coverage window (nr*(lastword-firstword+1) words), plus per pick
    the union's read-modify-write (2*nr*(nwpr+1) words) and the area/used
    scan (nwanted*(4+1) bytes)."""
    nr = 2 * roi + 1
    nwpr = (nr + 63) // 64
    x = (obs // nrows).astype(np.int64)
    y = (obs % nrows).astype(np.int64)
    fw = np.floor_divide(y - roi, 64)
    lw = (y + roi) // 64
    per_cand = (nr * nwpr + nr * (lw - fw + 1)) * 8
    used = np.zeros(nsheds, bool)
    total = int(per_cand.sum())  # round 1: every candidate
    lim = 4 * roi * roi
    for t, p in enumerate(order):
        used[p] = True
        total += 2 * nr * (nwpr + 1) * 8 + nsheds * 5
        if t + 1 < len(order):  # the next round rescores neighbours of p
            m = (~used) & ((x - x[p]) ** 2 + (y - y[p]) ** 2 <= lim)
            total += int(per_cand[m].sum())
    return total


def max_over_ranks(values, device):
    """Element-wise maximum over the ranks of the initialised process group
    (the slowest replica sets the whole job's time); unchanged on one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def workload_config(args, w, world, nwanted):
    """The `config` of a bench line: the workload and its parameters."""
    return {"workload": args.workload, "nrows": w["nrows"], "roi": w["roi"],
            "height": w["height"], "targets": w["ntests"], "bw": w["bw"], "nwanted": nwanted,
            "intervis": w["intervis"],
            "dem": f"fbm {w['octaves']} octaves, ridged {w['ridged']}, 0-{w['range_max']}",
            "parallelism": f"replicas{world}", "l2": "flushed (512 MiB write) between steps"}


def run_gpu(args, w):
    import torch

    import siting_gb300 as sg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    n = w["nrows"]
    p = params(w)
    g = sg.block_geometry(n, w["bw"], w["nwanted0"])
    dem = make_dem(w, seed_offset=rank)
    ctx = sg.Context(local)
    if args.site_ctas:
        ctx.set_site_ctas(args.site_ctas)
    plan_desc = "library default"
    if args.autotune:  # one-off, before the clock: plans timed on a corner of the DEM
        plan_desc = "autotuned " + str(ctx.autotune(p, dem, sample_rows=args.autotune_rows))
    if args.shed_plan is not None:  # a VIEWSHED window form pinned for this job's roi
        pinned = sg.Plan(shed_smem=args.shed_plan)
        ctx.autotune_set(w["roi"], w["ntests"], pinned)
        plan_desc = "pinned " + str(pinned)
    stream = torch.cuda.ExternalStream(ctx.stream)

    # device-resident buffers
    d_dem = torch.from_numpy(dem.view(np.int16)).to(f"cuda:{local}")
    d_obs = torch.empty(g.nwanted, dtype=torch.int32, device=f"cuda:{local}")
    d_sel = torch.empty(g.nwanted, dtype=torch.uint8, device=f"cuda:{local}")
    # pinned host buffers for the end-to-end form
    h_dem = torch.from_numpy(dem.view(np.int16)).pin_memory()
    h_obs = torch.empty(g.nwanted, dtype=torch.int32).pin_memory()
    h_sel = torch.empty(g.nwanted, dtype=torch.uint8).pin_memory()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    def timed(fn):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), r

    dev_step = lambda: ctx.run_dev(p, d_dem, d_obs, d_sel)  # noqa: E731
    e2e_step = lambda: ctx.run_into(p, h_dem, h_obs, h_sel)  # noqa: E731

    for _ in range(args.warmup):
        timed(dev_step)
        timed(e2e_step)
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    dev_ms, e2e_ms, stage = [], [], []
    for _ in range(args.steps):
        ms, r = timed(dev_step)
        dev_ms.append(ms)
        stage.append(r)
    for _ in range(args.steps):
        ms, _ = timed(e2e_step)
        e2e_ms.append(ms)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()

    mean_dev = sum(dev_ms) / len(dev_ms)
    mean_e2e = sum(e2e_ms) / len(e2e_ms)
    mean_dev, mean_e2e = max_over_ranks([mean_dev, mean_e2e], f"cuda:{local}")
    r = stage[-1]
    stage_ms = {k: sum(getattr(x, "ms_" + k) for x in stage) / len(stage)
                for k in ("vix", "findmax", "viewshed", "site")}
    out = {
        "metric": METRIC, "value": world * n * n / (mean_dev / 1e3), "unit": "cells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mean_dev, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32/u64", "data": "synthetic",
        "config": workload_config(args, w, world, g.nwanted),
        "plan": plan_desc,
        "e2e": {"value": world * n * n / (mean_e2e / 1e3), "unit": "cells/s",
                "ms_per_step": mean_e2e, "h2d_bytes_per_step": n * n * 2,
                "d2h_bytes_per_step": g.nwanted * 5},
        "gpu_launches": 10 * args.steps,  # 5 kernels per job, device and e2e jobs
        "observers_per_s": world * g.nwanted / (mean_dev / 1e3),
        "stages_ms": stage_ms,
        "site": {"nusedsheds": r.nusedsheds, "coverage": r.coverage, "rounds": r.site_rounds,
                 "phase_cycles": ctx.last_site_phase_cycles()},
        "clocks": clk,
    }
    return out, (dem, d_obs, d_sel, r, ctx, g), stage_ms


# Compulsory HBM bytes per cell / per observer of each stage (DEM read once,
# outputs written once), the algorithmic traffic the roofline divides by time.
def stage_bytes(w, nwanted, site_bytes):
    """Algorithmic HBM bytes of each stage: VIX, FINDMAX and VIEWSHED read their
    inputs and write their outputs once; SITE's are the reference's rescoring
    traffic (site_algorithmic_bytes)."""
    n, roi = w["nrows"], w["roi"]
    nr = 2 * roi + 1
    shed = nr * ((nr + 63) // 64) * 8
    cells = n * n
    return {
        "vix": cells * 3,                       # DEM uint16 in, VIX uint8 out
        "findmax": cells * 1 + nwanted * 4,     # VIX in, observers out
        "viewshed": cells * 2 + nwanted * (4 + shed),  # DEM + observers in, sheds out
        "site": site_bytes,
    }


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# ncu: VIX, VIEWSHED (shed_half_kernel) and SITE captured at full size.
NCU_TRAFFIC = {
    "c2_4096": {"vix": 33720064 + 1536, "viewshed": 33861632 + 361607680,
                "site": 2494835712 + 10062080},
}

# Warp instructions per unit of work of the two issue-bound stages, from ncu
# (smsp__inst_executed.sum of one launch / its units) on the 2048^2 captures
# with roi 100 and 100 targets: per target for VIX (vix_kernel), per observer
# for VIEWSHED (shed_half_kernel, both halves).  Keyed by the parameters they
# were measured with.
ISSUE_WORK = {
    ("vix", 100, 100): (2.058e9 / (2048 * 2048 * 100), "target"),
    ("viewshed", 100, 100): (1.398323148e9 / 16384, "observer"),
}
ISSUE_SLOTS_PER_SM = 4  # one warp instruction per cycle from each SM sub-partition

ROOFLINE_NOTES = {
    "vix": "VIX is bound by SM instruction issue, not HBM: its compulsory traffic is 3 B/cell; "
           "achieved = warp instructions per target (ncu) x targets / stage time, peak = SMs x "
           "4 issue slots x the median SM clock of the timed region",
    "viewshed": "VIEWSHED is bound by SM instruction issue (one dependent chain per ray); "
                "achieved = warp instructions per observer (ncu) x observers / stage time",
    "site": "SITE's algorithmic bytes are the reference's rescoring traffic (every rescored "
            "candidate's shed and coverage window per pick); this kernel updates gains by "
            "per-pick deltas and reads less (traffic); it is bound by the latency of its "
            "dependent rounds, not by HBM",
}


def roofline(out, w, state, peaks, stage_ms_mean):
    """Roofline of the dominant stage (largest mean device time), and every
    stage's HBM and (for VIX and VIEWSHED) issue-slot fractions."""
    import torch

    dem, d_obs, d_sel, r, ctx, g = state
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "measured" if "hbm_gbs" in peaks else "fallback"
    obs = d_obs.cpu().numpy()
    order = ctx.last_pick_order(g.nwanted)
    site_ref_bytes = site_algorithmic_bytes(w["nrows"], w["roi"], obs, order, g.nwanted)
    sb = stage_bytes(w, g.nwanted, site_ref_bytes)
    traffic = NCU_TRAFFIC.get(out["config"]["workload"], {})
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = out["clocks"].get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    issue_peak = sms * ISSUE_SLOTS_PER_SM * mhz * 1e6  # warp instructions / s
    units = {"vix": w["nrows"] ** 2 * w["ntests"], "viewshed": g.nwanted}
    stages = {}
    for k, ms in stage_ms_mean.items():
        ach = sb[k] / (ms / 1e3) / 1e9
        st = {"ms": ms, "alg_bytes": sb[k], "achieved_gbs": ach, "hbm_frac": ach / hbm}
        if k in traffic:
            st["dram_bytes"] = traffic[k]
            st["dram_frac"] = traffic[k] / (ms / 1e3) / 1e9 / hbm
        iw = ISSUE_WORK.get((k, w["roi"], w["ntests"]))
        if iw:
            per_unit, unit = iw
            ips = per_unit * units[k] / (ms / 1e3)
            st.update(issue_frac=ips / issue_peak, warp_instructions_per_s=ips,
                      warp_instructions_per_unit=per_unit, unit_of_work=unit)
        stages[k] = st
    dom = max(stage_ms_mean, key=stage_ms_mean.get)
    d = stages[dom]
    hbm_part = {"achieved": d["achieved_gbs"], "peak": hbm, "unit": "GB/s", "frac": d["hbm_frac"],
                "peak_source": f"{src} (hbm_gbs)" if src == "measured" else "fallback 6800 GB/s"}
    if "issue_frac" in d:
        line = {"kernel": dom, "bound": "sm_issue",
                "achieved": d["warp_instructions_per_s"] / 1e12, "peak": issue_peak / 1e12,
                "unit": "T warp-instructions/s", "frac": d["issue_frac"],
                "traffic": traffic.get(dom),
                "peak_source": f"{sms} SMs x {ISSUE_SLOTS_PER_SM} issue slots x {mhz:.0f} MHz "
                               "(median SM clock of the timed region)",
                "warp_instructions_per_unit": d["warp_instructions_per_unit"],
                "unit_of_work": d["unit_of_work"], "hbm": hbm_part}
    else:
        line = {"kernel": dom, "bound": "hbm", "achieved": d["achieved_gbs"], "peak": hbm,
                "unit": "GB/s", "frac": d["hbm_frac"], "traffic": traffic.get(dom),
                "peak_source": hbm_part["peak_source"]}
        if "dram_frac" in d:
            line["dram_frac"] = d["dram_frac"]
    if dom in ROOFLINE_NOTES:
        line["note"] = ROOFLINE_NOTES[dom]
    work = {"vix_targets": units["vix"],
            "vix_targets_per_s": units["vix"] / (stage_ms_mean["vix"] / 1e3),
            "site_rounds": r.site_rounds, "site_picks": r.nusedsheds}
    return line, stages, work


def fullsize_parity(workload, obs, sel, res):
    """The job's outputs against the reference's own recorded outputs for
    this workload (the full-size golden fixture, generated by seqsite), when
    there is one: observers, selection, observer count and covered cells."""
    import hashlib

    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        cases = {c["name"]: c for c in json.load(f).get("fullsize", [])}
    c = cases.get(workload)
    if c is None:
        return None
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    checks = {"observers": sha(obs) == c["obs_sha256"],
              "selected": sha(sel) == c["selected_sha256"],
              "nusedsheds": res.nusedsheds == c["nused"],
              "cumarea": res.cumarea == c["cumarea"]}
    return {"against": "reference seqsite outputs recorded in the full-size golden fixture",
            "bit_exact": all(checks.values()), "checks": checks,
            "selected_disagreeing": int(np.count_nonzero(sel)) - c["nused"]
            if not checks["selected"] else 0}


# cusite (siting.cu) rebuilt for sm_103a, as a reported comparison.  Its
# FINDMAX kernel (siting.cu:164-224) starts thread t of a 256-thread CTA at
# point t*ceil(npoints/256) of its block; where that is past the block's
# points the thread reads other blocks' cells, and in the last block row
# cells past the end of the VIX array.  It is run only where every block keeps
# every thread inside the block, within its other fixed limits (a 500 000-entry
# candidate list, siting.cu:645; nr threads a CTA, siting.cu:672).
def cusite_runs_in_bounds(w, geo):
    nr = 2 * w["roi"] + 1
    if geo.nwanted > 499999 or nr > 1024:
        return False
    bs = np.float32(geo.blocksize)
    n = w["nrows"]
    edges = [min(int(bs * np.float32(b)), n) for b in range(geo.nblocks + 1)]
    sizes = [b - a for a, b in zip(edges, edges[1:])]
    for sx in set(sizes):
        for sy in set(sizes):
            npoints = sx * sy
            per = -(-npoints // 256)
            if 255 * per >= npoints:
                return False
    return True


def cusite_column(w, dem, geo):
    from oracle_bind import REF_CUSITE

    if not os.path.exists(REF_CUSITE):
        return {"skipped": "cusite not built here (the reference's siting.cu is not staged)"}
    if not cusite_runs_in_bounds(w, geo):
        return {"skipped": "with these parameters cusite's FINDMAX reads outside its blocks "
                           "(past the VIX array in the last block row); not run"}
    path = write_dem_file(dem)
    try:
        r = time_reference_program(REF_CUSITE, w, path, "GPU")
    finally:
        os.unlink(path)
    r.pop("threads", None)
    r.pop("cores", None)
    r["build"] = "siting.cu with its makefile's command, -arch=sm_35 -> " \
                 "-gencode arch=compute_103a,code=sm_103a"
    r["note"] = "its results differ from seqsite (float division, FMA contraction, racy " \
                "reductions), so it is a timing comparison only; its times include its own " \
                "CUDA context creation, allocations and host copies"
    return r


def reference_inputs(w):
    """The workload's DEM and block geometry from the CPU side alone (the
    oracle's own generator, byte-equal to the library's, and the geometry of
    siting.cpp:688-695): the reference arm never loads the library."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_bind import Oracle

    port = Oracle("port")
    dem = port.fbm_dem(w["nrows"], w["seed"], octaves=w["octaves"],
                       ridged_weight=w["ridged"], range_max=w["range_max"])
    return dem, port.geometry(w["nrows"], w["bw"], w["nwanted0"])


class _StdoutToStderr:
    """The reference's SITE prints its progress line on stdout: keep it off
    the bench's single JSON line."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        os.dup2(2, 1)

    def __exit__(self, *exc):
        import ctypes

        ctypes.CDLL(None).fflush(None)  # C and C++ buffered output goes to stderr too
        os.dup2(self.saved, 1)
        os.close(self.saved)


def time_reference_library(w, dem, geo, warmup, steps, budget_s):
    """The reference's own CPU code (siting.cpp built with OpenMP, library
    form) on the whole workload with every host thread: each step runs the
    four stages of main (siting.cpp:737-759) on the in-memory DEM, like the
    GPU arm's device-resident step.  Without the reference's sources the
    oracle port (same stages, deterministic) stands in and says so.  Steps
    stop early once `budget_s` of CPU time is spent (at least one)."""
    from oracle_bind import REF_OMP_SO, Oracle

    n, roi = w["nrows"], w["roi"]
    cores = os.cpu_count() or 1
    if os.path.exists(REF_OMP_SO):
        orc, kind = Oracle("reference_omp"), "reference_omp"
    else:
        orc, kind = Oracle("port"), "port"
    threads = orc.set_threads(cores)
    nr = 2 * roi + 1
    nwpr = (nr + 63) // 64
    vix = np.empty(n * n, np.uint8)
    obs = np.empty(geo.nwanted, np.int32)
    sheds = np.empty(geo.nwanted * nr * nwpr, np.uint64)
    sel = np.empty(geo.nwanted, np.uint8)
    lib = orc.lib
    h = w["height"]

    def step():
        t = [time.perf_counter()]
        if kind == "port":
            sheds.fill(0)  # the reference's calc_sheds zeroes its own output
            lib.oracle_calc_vix(n, dem, roi, h, h, w["ntests"], vix)
            t.append(time.perf_counter())
            lib.oracle_find_max(n, vix, geo.blocksize, geo.nblocks, geo.nwantedperblock, obs)
            t.append(time.perf_counter())
            lib.oracle_calc_sheds(n, dem, roi, h, h, geo.nwanted, obs, sheds)
            t.append(time.perf_counter())
            cum = __import__("ctypes").c_longlong()
            lib.oracle_site_it(n, roi, w["intervis"], geo.nwanted, obs, sheds, sel,
                               __import__("ctypes").byref(cum), None)
        else:
            lib.ref_calc_vix(n, dem, roi, h, h, w["ntests"], vix)
            t.append(time.perf_counter())
            lib.ref_find_max(n, vix, geo.blocksize, geo.nwanted, geo.nblocks,
                             geo.nwantedperblock, obs)
            t.append(time.perf_counter())
            lib.ref_calc_sheds(n, dem, roi, h, h, geo.nwanted, obs, sheds)
            t.append(time.perf_counter())
            lib.ref_site_it(n, roi, w["intervis"], geo.nwanted, obs, sheds, sel)
        t.append(time.perf_counter())
        return [b - a for a, b in zip(t, t[1:])]

    spent, warm, runs = 0.0, 0, []
    with _StdoutToStderr():
        for i in range(warmup + steps):
            st = step()
            spent += sum(st)
            if i < warmup:
                warm += 1
            else:
                runs.append(st)
            if spent >= budget_s and runs:
                break
            if i < warmup and spent >= budget_s / 2:  # no more warm-up than half the budget
                warmup = i + 1
    mean = sum(sum(r) for r in runs) / len(runs)
    stages = {k: sum(r[j] for r in runs) / len(runs)
              for j, k in enumerate(("vix", "findmax", "viewshed", "site"))}
    return {"kind": kind, "value": n * n / mean, "unit": "cells/s", "cores": cores,
            "threads": threads, "seconds_per_step": mean, "steps": len(runs), "warmup": warm,
            "stages_s": stages, "nusedsheds": int(sel.sum()),
            "sample": f"the whole {n}x{n} job (no sampling), DEM in host memory, "
                      f"{len(runs)} timed run(s); "
                      + ("the reference's siting.cpp compiled with OpenMP in library form, "
                         f"omp_set_num_threads({threads})" if kind != "port" else
                         "oracle port (reference sources not staged on this machine)")}


_TIMING_KEYS = ("input", "vix", "findmax", "viewshed", "site", "output", "total")


def _parse_timing_line(text):
    """The reference programs' stdout line `input:.. vix:.. ... total:..`."""
    import re

    out = {}
    for k, v in re.findall(r"([a-z]+):([-+0-9.eE]+)", text):
        out[k] = float(v)
    return out


def time_reference_program(exe, w, dem_path, threads_note):
    """One run of a reference program (ompsite as its makefile builds it, or
    cusite rebuilt for sm_103a) through its own command line on the
    workload's DEM file: its own stage-timing line, plus the wall clock."""
    import tempfile

    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "observers.txt")
        cmd = [exe, str(w["nrows"]), str(w["roi"]), str(w["height"]), str(w["ntests"]),
               str(w["bw"]), str(w["nwanted0"]), str(w["intervis"]), dem_path, out]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"error": f"exit {r.returncode}: {(r.stdout + r.stderr).strip()[-200:]}"}
        tl = _parse_timing_line(r.stdout)
        nobs = sum(1 for _ in open(out))
    total = tl.get("total", wall)
    return {"value": w["nrows"] ** 2 / total, "unit": "cells/s", "seconds": total,
            "wall_s": wall, "stages_s": {k: tl[k] for k in _TIMING_KEYS if k in tl},
            "nusedsheds": int(tl.get("nusedsheds", nobs)), "coverage": tl.get("coverage"),
            "observers": nobs, "threads": threads_note, "cores": os.cpu_count() or 1,
            "command": " ".join([os.path.basename(exe)] + cmd[1:8] + ["dem.raw", "observers.txt"])}


def write_dem_file(dem):
    import tempfile

    fd, path = tempfile.mkstemp(suffix=".raw")
    with os.fdopen(fd, "wb") as f:
        f.write(np.ascontiguousarray(dem, np.uint16).tobytes())
    return path


def run_reference_arm(args, w):
    """`--impl reference`: the reference's own CPU implementation on the same
    workload and parameters as the GPU arm, no library code on the path."""
    dem, geo = reference_inputs(w)
    cb = time_reference_library(w, dem, geo, warmup=min(args.warmup, 1), steps=args.steps,
                                budget_s=args.reference_budget_s)
    from oracle_bind import REF_OMPSITE

    shipped = None
    if os.path.exists(REF_OMPSITE):
        path = write_dem_file(dem)
        try:
            shipped = time_reference_program(REF_OMPSITE, w, path,
                                             "50 (hard-coded, siting.cpp:633-636)")
        finally:
            os.unlink(path)
    config = workload_config(args, w, args.gpus, geo.nwanted)
    line = {"metric": METRIC, "value": cb["value"], "unit": "cells/s", "n_gpus": args.gpus,
            "steps": cb["steps"], "warmup": cb["warmup"], "steps_requested": args.steps,
            "warmup_requested": args.warmup,
            "ms_per_step": cb["seconds_per_step"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/u64", "data": "synthetic",
            "config": config, "impl": "reference",
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "threads", "kind",
                                                "sample")},
            "e2e": {"value": cb["value"], "unit": "cells/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "stages_s": cb["stages_s"], "nusedsheds": cb["nusedsheds"],
            "note": f"each step is one whole job; steps stop after "
                    f"{args.reference_budget_s:.0f} s of CPU time (at least one)"}
    if shipped is not None:
        line["ompsite_as_shipped"] = shipped
    print(json.dumps(line))


def run_batch_workload(args):
    """Batched form vs one plain job after another, same GPU, same inputs."""
    import torch

    import siting_gb300 as sg

    torch.cuda.set_device(0)
    jobs = batch_jobs(args.batch_jobs)
    params = [p for p, _ in jobs]
    dems = [sg.fbm_dem(p.nrows, d["seed"], octaves=8, range_max=d["range_max"]) for p, d in jobs]
    geos = [sg.block_geometry(p.nrows, p.bw, p.nwanted0) for p in params]
    cells = sum(p.nrows ** 2 for p in params)
    d_dems = [torch.from_numpy(d.view(np.int16)).cuda() for d in dems]
    obs_b = [torch.empty(g.nwanted, dtype=torch.int32, device="cuda") for g in geos]
    sel_b = [torch.empty(g.nwanted, dtype=torch.uint8, device="cuda") for g in geos]
    obs_p = [torch.empty(g.nwanted, dtype=torch.int32, device="cuda") for g in geos]
    sel_p = [torch.empty(g.nwanted, dtype=torch.uint8, device="cuda") for g in geos]
    cb, cp = sg.Context(0), sg.Context(0)
    sb, spl = torch.cuda.ExternalStream(cb.stream), torch.cuda.ExternalStream(cp.stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def timed(stream, fn):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), r

    batched = lambda: cb.run_batch_dev(params, d_dems, obs_b, sel_b)  # noqa: E731
    plain = lambda: [cp.run_dev(p, d, o, s) for p, d, o, s in zip(params, d_dems, obs_p, sel_p)]  # noqa: E731
    if args.batch_mode is not None:
        cb.set_batch_mode(args.batch_mode)
    if args.batch_only:  # the batched form alone (a launch list of its kernels)
        for _ in range(args.warmup):
            timed(sb, batched)
        tb = [timed(sb, batched)[0] for _ in range(args.steps)]
        cb.close()
        cp.close()
        return {"metric": METRIC + " (batched)", "value": cells / (sum(tb) / len(tb) / 1e3),
                "unit": "cells/s", "ms_per_step": sum(tb) / len(tb), "steps": args.steps,
                "warmup": args.warmup, "config": {"workload": f"batch{len(jobs)}_512_2048",
                                                  "batch_mode": args.batch_mode}}
    for _ in range(args.warmup):
        timed(sb, batched)
        timed(spl, plain)
    tb = [timed(sb, batched)[0] for _ in range(args.steps)]
    tp = [timed(spl, plain)[0] for _ in range(args.steps)]
    rb = batched()
    rp = plain()
    torch.cuda.synchronize()
    same = all(torch.equal(a, b) for a, b in zip(obs_b, obs_p)) and \
        all(torch.equal(a, b) for a, b in zip(sel_b, sel_p)) and \
        all((x.nusedsheds, x.cumarea) == (y.nusedsheds, y.cumarea) for x, y in zip(rb, rp))
    mb, mp = sum(tb) / len(tb), sum(tp) / len(tp)
    graph_stats = cb.batch_graph_stats()
    # the launch forms of the batch's VIX and FINDMAX (siting_ctx_set_batch_mode:
    # 1 = grids over many jobs' items, 2 = one launch per job), the merged form
    # also captured as a CUDA graph and replayed
    forms = {}
    for name, mode, graphs in (("merged_grids_graph", 1, True), ("merged_grids_direct", 1, False),
                               ("per_job_direct", 2, False)):
        cb.set_batch_mode(mode)
        cb.set_batch_graphs(graphs)
        for _ in range(2):
            timed(sb, batched)
        ts = [timed(sb, batched)[0] for _ in range(3)]
        forms[name] = sum(ts) / len(ts)
    cb.set_batch_mode(0)
    cb.set_batch_graphs(True)
    cb.close()
    cp.close()
    out = {"metric": METRIC + " (batched)", "value": cells / (mb / 1e3), "unit": "cells/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": mb,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/u64",
           "data": "synthetic",
           "config": {"workload": f"batch{len(jobs)}_512_2048", "jobs": len(jobs), "cells": cells,
                      "l2": "flushed (512 MiB write) between steps"},
           "plain": {"value": cells / (mp / 1e3), "unit": "cells/s", "ms_per_step": mp},
           "speedup_vs_plain": mp / mb, "bit_identical_to_plain": bool(same),
           "batch_phase_ms": {"upload": rb[0].ms_h2d,
                              "vix_findmax_viewshed": rb[0].ms_vix,
                              "site_after_them": rb[0].ms_site},
           "site_rounds_max": max(r.site_rounds for r in rb),
           "graph": {"captures": graph_stats[0], "replays": graph_stats[1]},
           "launch_forms_ms": forms,
           # where the floor is: each job's stage times when it runs alone
           # (the plain runs); VIX, FINDMAX and VIEWSHED already fill the GPU
           # one job at a time, so their sum bounds any batching from below
           "plain_stage_ms_sum": {k: float(sum(getattr(r, "ms_" + k) for r in rp))
                                  for k in ("vix", "findmax", "viewshed", "site")}}
    st_sum = out["plain_stage_ms_sum"]
    out["floor_ms"] = st_sum["vix"] + st_sum["findmax"] + st_sum["viewshed"]
    out["speedup_bound_vs_plain"] = mp / out["floor_ms"]
    return out


# The serving workload: a Poisson stream of requests, sides log-uniform in
# [256, 4096], roi U[20,200], height U[20,300], targets U[32,128],
# bw in {8,16,32}, nwanted = n^2/128, intervis Bernoulli(0.5), served under a
# 150 GB HBM budget.  Each request's DEM is a window of one of six 4096^2 fBm
# rasters (submitted with its row pitch, no copy).
def serve_jobs(nreq, seed=5):
    import siting_gb300 as sg

    rng = np.random.default_rng(seed)
    jobs = []
    for _ in range(nreq):
        n = int(np.exp(rng.uniform(np.log(256), np.log(4096))))
        p = sg.Params(nrows=n, roi=int(rng.integers(20, 201)), height=int(rng.integers(20, 301)),
                      ntests=int(rng.integers(32, 129)), bw=int(rng.choice([8, 16, 32])),
                      nwanted0=max(1, n * n // 128), intervis=int(rng.random() < 0.5))
        src = int(rng.integers(0, 6))
        x0, y0 = (int(v) for v in rng.integers(0, 4096 - n + 1, size=2))
        jobs.append((p, src, x0, y0))
    return jobs


def serve_rasters():
    import siting_gb300 as sg

    return [sg.fbm_dem(4096, 4096 * 7 + i, octaves=10, ridged_weight=0.3 * (i % 2),
                       range_max=int(2000 + 5600 * i)).reshape(4096, 4096) for i in range(6)]


def serve_at_rate(args, jobs, rasters, rate, seed=11):
    """One Poisson arrival stream through a fresh server: per-request latency
    (submission to results in host memory), throughput, admissions."""
    import queue

    import siting_gb300 as sg

    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(jobs))
    budget = int(args.serve_budget_gb * (1 << 30))
    srv = sg.Server(0, hbm_budget=budget, max_batch_jobs=args.batch_jobs, reserve=True)
    # warm-up: a few requests before the clock starts
    for p, src, x0, y0 in jobs[:3]:
        srv.wait(srv.submit(p, rasters[src][x0:x0 + p.nrows, y0:y0 + p.nrows]))
    infos, refused, pending = {}, 0, []
    q = queue.Queue()

    def waiter():  # collects completions in submission order
        while (t := q.get()) is not None:
            infos[t.id] = srv.wait(t)[2]

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    due = t0
    arrivals = []
    for (p, src, x0, y0), gap in zip(jobs, gaps):
        due += gap
        dt = due - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        arrivals.append(due - t0)
        try:
            t = srv.submit(p, rasters[src][x0:x0 + p.nrows, y0:y0 + p.nrows])
        except sg.SitingError:
            refused += 1
            continue
        pending.append(t)
        q.put(t)
    q.put(None)
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    served = [(t, infos[t.id]) for t in pending]
    lat = np.array([i.latency_s for _, i in served]) * 1e3
    cells = sum(t.params.nrows ** 2 for t, _ in served)
    span = max(i.t_done for _, i in served) - min(i.t_submit for _, i in served)
    return {"rate_per_s": rate, "requests": len(jobs), "value": cells / span, "unit": "cells/s",
            "latency_ms": {"p50": float(np.percentile(lat, 50)),
                           "p90": float(np.percentile(lat, 90)),
                           "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
            "served": len(served), "refused": refused, "wall_s": wall,
            "requests_per_s": len(served) / span,
            "admissions": st["batches"],
            "mean_in_flight_at_admission": float(np.mean([i.batch_jobs for _, i in served])),
            "gpu_busy_frac": st["busy_s"] / max(span, 1e-9),
            "peak_workspace_gb": st["peak_workspace"] / (1 << 30),
            "_served": served, "_arrivals": np.array(arrivals)}


def plain_service_times(jobs, rasters, check=None):
    """The plain loop: each request alone through siting_run (host buffers,
    upload and readback included), one after another.  Returns the service
    time of each, and whether the listed served requests' outputs equal it."""
    import siting_gb300 as sg

    ctx = sg.Context(0)
    times, same = [], True
    check = check or {}
    for i, (p, src, x0, y0) in enumerate(jobs):
        dem = np.ascontiguousarray(rasters[src][x0:x0 + p.nrows, y0:y0 + p.nrows]).ravel()
        t0 = time.perf_counter()
        o, s_, _r = ctx.run(p, dem)
        times.append(time.perf_counter() - t0)
        if i in check:
            t = check[i]
            same &= bool(np.array_equal(o, t.obs) and np.array_equal(s_, t.selected))
    ctx.close()
    return np.array(times), same


def fifo_latencies_ms(arrivals, service):
    """Latency of each request in a one-at-a-time FIFO loop with these
    arrivals (s) and service times (s)."""
    done, out = 0.0, []
    for a, sv in zip(arrivals, service):
        done = max(done, a) + sv
        out.append(done - a)
    return np.array(out) * 1e3


def run_serve_workload(args):
    """Serving loop under a Poisson arrival stream: latency percentiles and
    throughput against the plain one-request-at-a-time loop (the same
    requests run alone one after another: its throughput, and its latencies
    under the same arrivals from the measured service times); served
    requests are compared with their solo runs bit for bit."""
    rasters = serve_rasters()
    rates = args.serve_sweep or [args.serve_rate]
    per_rate = []
    for rate in rates:
        n = args.serve_requests if not args.serve_sweep else \
            min(args.serve_requests, max(200, int(rate * 30)))
        jobs = serve_jobs(n)
        r = serve_at_rate(args, jobs, rasters, rate)
        served = r.pop("_served")
        arrivals = r.pop("_arrivals")
        # the plain loop on the same requests (a prefix of them outside a sweep)
        k = len(jobs) if args.serve_sweep else min(len(jobs), args.serve_plain)
        check = {i: served[i][0] for i in range(min(args.serve_check, len(served)))}
        svc, same = plain_service_times(jobs[:k], rasters, check)
        cells_k = sum(p.nrows ** 2 for p, *_ in jobs[:k])
        plain = {"value": cells_k / svc.sum(), "unit": "cells/s", "requests_timed": k}
        if k == len(jobs):
            fl = fifo_latencies_ms(arrivals, svc)
            plain["latency_ms"] = {"p50": float(np.percentile(fl, 50)),
                                   "p99": float(np.percentile(fl, 99))}
        r["plain_loop"] = plain
        # below saturation the served throughput is the offered load, so the
        # like-for-like comparison is latency under the same arrivals; the
        # throughput ratio is against the plain loop's back-to-back capacity
        r["throughput_vs_plain_capacity"] = r["value"] / plain["value"]
        if "latency_ms" in plain:
            r["latency_vs_plain"] = {
                q: plain["latency_ms"][q] / r["latency_ms"][q] for q in ("p50", "p99")}
        r["checked_alone"] = len(check)
        r["bit_identical_alone"] = same
        per_rate.append(r)
    head = per_rate[0] if len(per_rate) == 1 else max(per_rate, key=lambda x: x["value"])
    out = {"metric": "DEM cells/s served", "value": head["value"], "unit": "cells/s",
           "n_gpus": 1, "steps": head["served"], "warmup": 3,
           "ms_per_step": 1e3 / head["requests_per_s"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/u64",
           "data": "synthetic",
           "config": {"workload": "serve_poisson", "rate_per_s": head["rate_per_s"],
                      "requests": head["requests"], "hbm_budget_gb": args.serve_budget_gb,
                      "max_in_flight": args.batch_jobs, "sides": "log-U[256,4096]",
                      "roi": "U[20,200]", "nwanted": "n^2/128"}}
    out.update({k: v for k, v in head.items() if k not in ("value", "unit")})
    if len(per_rate) > 1:
        out["sweep"] = per_rate
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2_4096",
                    choices=sorted(WORKLOADS) + ["c3_batch", "c5_serve"])
    ap.add_argument("--reference-budget-s", type=float, default=90.0,
                    help="CPU seconds after which the reference arm stops timing more steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline job only: no batched or serving measurements")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--batch-only", action="store_true",
                    help="batched workload: time the batched form alone (no plain runs)")
    ap.add_argument("--batch-mode", type=int, default=None, choices=[0, 1, 2],
                    help="batched workload: VIX/FINDMAX launch form (siting_ctx_set_batch_mode)")
    ap.add_argument("--autotune", action="store_true",
                    help="time the launch plans on a corner of the DEM first (siting_autotune)")
    ap.add_argument("--autotune-rows", type=int, default=1024)
    ap.add_argument("--shed-plan", type=int, default=None, choices=[0, 1, 2],
                    help="VIEWSHED window form (siting_autotune_set): 1 half windows, "
                         "2 the whole window, 0 the whole window through L1")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--serve-rate", type=float, default=100.0, help="mean arrivals per second")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-check", type=int, default=8,
                    help="requests re-run alone and compared bit for bit")
    ap.add_argument("--serve-plain", type=int, default=2000,
                    help="requests timed through the plain one-at-a-time loop (no sweep); "
                         "all of them give its latencies under the same arrivals")
    ap.add_argument("--serve-sweep", type=float, nargs="*", default=None,
                    help="arrival rates to sweep (requests: min(serve-requests, 30 s worth))")
    ap.add_argument("--site-ctas", type=int, default=0,
                    help="CTAs of the SITE kernel (0 = library default)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.workload == "c5_serve":
        if args.impl == "gb300" and rank == 0:
            print(json.dumps(run_serve_workload(args)))
        return
    if args.workload == "c3_batch":
        if args.impl == "gb300" and rank == 0:
            print(json.dumps(run_batch_workload(args)))
        return
    w = WORKLOADS[args.workload]

    if args.impl == "reference":
        if rank == 0:  # under torchrun the other ranks exit without work
            run_reference_arm(args, w)
        return

    out, state, stage_ms = run_gpu(args, w)
    if rank != 0:
        return
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        with open(pp) as f:
            peaks = json.load(f)
    line, stages, work = roofline(out, w, state, peaks, stage_ms)
    out["roofline"] = line
    out["roofline_stages"] = stages
    out["stage_work"] = work
    par = fullsize_parity(args.workload, state[1].cpu().numpy(), state[2].cpu().numpy(), state[3])
    if par is not None:
        out["parity"] = par
    if not args.no_cpu_baseline and int(os.environ.get("WORLD_SIZE", "1")) == 1:
        # one whole job of the reference's OpenMP code on the host cores
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from oracle_bind import Oracle

        geo = Oracle("port").geometry(w["nrows"], w["bw"], w["nwanted0"])
        cb = time_reference_library(w, state[0], geo, warmup=0, steps=1, budget_s=0)
        out["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "threads", "kind",
                                                  "sample")}
        out["cusite_baseline"] = cusite_column(w, state[0], geo)
    if args.workload == "c2_4096" and not args.no_extras and \
            int(os.environ.get("WORLD_SIZE", "1")) == 1:
        # the batched and serving forms, measured in the same run (after the
        # headline's timed region, with their own timing)
        ctx = state[4]
        del state
        ctx.close()
        import torch

        torch.cuda.empty_cache()
        b = run_batch_workload(argparse.Namespace(**{**vars(args), "steps": min(args.steps, 5),
                                                     "warmup": min(args.warmup, 3)}))
        out["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "steps", "warmup",
                                             "plain", "speedup_vs_plain",
                                             "bit_identical_to_plain", "batch_phase_ms",
                                             "plain_stage_ms_sum", "floor_ms",
                                             "speedup_bound_vs_plain", "graph",
                                             "launch_forms_ms", "config")}
        sv = run_serve_workload(args)
        out["serving"] = {k: sv[k] for k in ("value", "unit", "latency_ms", "served", "refused",
                                             "requests_per_s", "gpu_busy_frac", "config",
                                             "mean_in_flight_at_admission", "plain_loop",
                                             "latency_vs_plain",
                                             "throughput_vs_plain_capacity", "checked_alone",
                                             "bit_identical_alone")
                          if k in sv}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
