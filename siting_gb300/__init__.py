"""GB300 observer siting: VIX -> FINDMAX -> VIEWSHED -> SITE.

Python mirror of the library's C ABI (include/siting.h).  The stage functions
keep the reference's names, argument order and meaning (wenlili/siting:
calc_vix siting.cpp:192, find_max siting.cpp:235, calc_sheds siting.cpp:349,
site_it siting.cpp:501); errors raise ``SitingError`` carrying the library's
status and message instead of the reference's exit(1).

All compute runs in the CUDA kernels of ``libsiting_gb300.so``.  There is no
CPU fallback: importing works without the library (for building), but every
call that needs it raises if it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

__all__ = [
    "SitingError", "Params", "Geometry", "Result", "Context", "load", "block_geometry",
    "validate", "fbm_dem", "read_dem", "write_observers", "observers_text", "LIB_PATH",
    "CLI_PATH", "shed_words", "Plan",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libsiting_gb300.so")
CLI_PATH = os.path.join(_PKG, "cusite")

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, EIO, EDEVICE = range(7)


class SitingError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


class _ParamsC(C.Structure):
    _fields_ = [("nrows", C.c_int), ("roi", C.c_int), ("oht", C.c_int), ("tht", C.c_int),
                ("ntests", C.c_int), ("bw", C.c_int), ("nwanted0", C.c_int),
                ("intervis", C.c_int)]


class _GeometryC(C.Structure):
    _fields_ = [("blocksize", C.c_float), ("nblocks", C.c_int), ("nwantedperblock", C.c_int),
                ("nwanted", C.c_int)]


class _ResultC(C.Structure):
    _fields_ = [("nusedsheds", C.c_int), ("cumarea", C.c_longlong), ("coverage", C.c_double),
                ("nwanted", C.c_int), ("ms_vix", C.c_float), ("ms_findmax", C.c_float),
                ("ms_viewshed", C.c_float), ("ms_site", C.c_float), ("ms_h2d", C.c_float),
                ("ms_d2h", C.c_float), ("site_rounds", C.c_int)]


class _PlanC(C.Structure):
    _fields_ = [("vix_tile", C.c_int), ("vix_smem", C.c_int), ("shed_smem", C.c_int),
                ("site_ctas", C.c_int)]


@dataclass
class Plan:
    """Launch plan of one job; 0 / -1 take the library default."""
    vix_tile: int = 0
    vix_smem: int = -1
    shed_smem: int = -1
    site_ctas: int = 0

    def c(self) -> _PlanC:
        return _PlanC(self.vix_tile, self.vix_smem, self.shed_smem, self.site_ctas)


@dataclass
class Params:
    """One job: the CLI's nine arguments minus the file names."""
    nrows: int
    roi: int
    height: int = 0
    ntests: int = 50
    bw: int = 10
    nwanted0: int = 10000
    intervis: int = 0
    oht: int | None = None
    tht: int | None = None

    def c(self) -> _ParamsC:
        oht = self.height if self.oht is None else self.oht
        tht = self.height if self.tht is None else self.tht
        return _ParamsC(self.nrows, self.roi, oht, tht, self.ntests, self.bw, self.nwanted0,
                        self.intervis)


@dataclass
class Geometry:
    blocksize: float
    nblocks: int
    nwantedperblock: int
    nwanted: int


@dataclass
class Result:
    nusedsheds: int
    cumarea: int
    coverage: float
    nwanted: int
    ms_vix: float
    ms_findmax: float
    ms_viewshed: float
    ms_site: float
    ms_h2d: float
    ms_d2h: float
    site_rounds: int

    @staticmethod
    def of(r: _ResultC) -> "Result":
        return Result(*(getattr(r, f) for f, _ in _ResultC._fields_))


class _JobInfoC(C.Structure):
    _fields_ = [("status", C.c_int), ("result", _ResultC), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double), ("batch_id", C.c_int),
                ("batch_jobs", C.c_int), ("error", C.c_char * 160)]


class _ServerStatsC(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong),
                ("refused", C.c_longlong), ("batches", C.c_longlong), ("pending", C.c_longlong),
                ("peak_workspace", C.c_size_t), ("busy_s", C.c_double)]


_lib = None
_P = C.c_void_p


def load() -> C.CDLL:
    """Loads libsiting_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SitingError(EDEVICE, f"{LIB_PATH} is missing: run siting_gb300.build.build() first")
    lib = C.CDLL(LIB_PATH)
    i, f, ll, sz = C.c_int, C.c_float, C.c_longlong, C.c_size_t
    sig = {
        "siting_status_string": ([i], C.c_char_p),
        "siting_last_error": ([_P], C.c_char_p),
        "siting_validate": ([C.POINTER(_ParamsC), i, C.c_char_p, sz], i),
        "siting_block_geometry": ([i, i, i, C.POINTER(_GeometryC)], i),
        "siting_ctx_create": ([i, sz, C.POINTER(_P)], i),
        "siting_ctx_destroy": ([_P], i),
        "siting_ctx_sync": ([_P], i),
        "siting_ctx_stream": ([_P], _P),
        "siting_ctx_workspace_bytes": ([_P], sz),
        "siting_ctx_trim": ([_P], i),
        "siting_ctx_set_site_ctas": ([_P, i], i),
        "siting_ctx_set_batch_mode": ([_P, i], i),
        "siting_ctx_set_batch_graphs": ([_P, i], i),
        "siting_ctx_batch_graph_stats": ([_P, C.POINTER(ll), C.POINTER(ll)], i),
        "siting_pinned_alloc": ([sz, C.POINTER(_P)], i),
        "siting_pinned_free": ([_P], i),
        "siting_calc_vix": ([_P, i, _P, i, i, i, i, _P], i),
        "siting_calc_vix_dev": ([_P, i, _P, i, i, i, i, _P], i),
        "siting_find_max": ([_P, i, _P, f, i, i, i, _P], i),
        "siting_find_max_dev": ([_P, i, _P, f, i, i, i, _P], i),
        "siting_calc_sheds": ([_P, i, _P, i, i, i, i, _P, _P], i),
        "siting_calc_sheds_dev": ([_P, i, _P, i, i, i, i, _P, _P], i),
        "siting_site_it": ([_P, i, i, i, i, _P, _P, _P, C.POINTER(_ResultC)], i),
        "siting_site_it_dev": ([_P, i, i, i, i, _P, _P, _P, C.POINTER(_ResultC)], i),
        "siting_site_it_noalloc": ([i, i, i, i, _P, _P, _P, _P, C.POINTER(_ResultC)], i),
        "siting_run": ([_P, C.POINTER(_ParamsC), _P, _P, _P, C.POINTER(_ResultC)], i),
        "siting_run_dev": ([_P, C.POINTER(_ParamsC), _P, _P, _P, C.POINTER(_ResultC)], i),
        "siting_last_pick_order": ([_P, _P, i, C.POINTER(C.c_int)], i),
        "siting_last_site_phase_cycles": ([_P, _P, i], i),
        "siting_run_batch": ([_P, i, _P, _P, _P, _P, _P, _P], i),
        "siting_run_batch_dev": ([_P, i, _P, _P, _P, _P, _P, _P], i),
        "siting_batch_workspace_bytes": ([_P, i, _P, _P, C.POINTER(sz)], i),
        "siting_autotune": ([_P, C.POINTER(_ParamsC), _P, i, C.POINTER(_PlanC)], i),
        "siting_autotune_set": ([_P, i, i, C.POINTER(_PlanC)], i),
        "siting_autotune_clear": ([_P], i),
        "siting_selftest_wait": ([_P, i, ll], i),
        "siting_server_create": ([i, sz, i, i, C.POINTER(_P)], i),
        "siting_server_destroy": ([_P], i),
        "siting_server_submit": ([_P, C.POINTER(_ParamsC), _P, i, _P, _P, C.POINTER(ll)], i),
        "siting_server_wait": ([_P, ll, C.c_double, C.POINTER(_JobInfoC)], i),
        "siting_server_stats_get": ([_P, C.POINTER(_ServerStatsC)], i),
        "siting_read_dem": ([C.c_char_p, i, _P], i),
        "siting_write_observers": ([C.c_char_p, i, i, _P, _P], i),
        "siting_fbm_dem": ([_P, i, C.c_uint64, i, C.c_double, C.c_double, C.c_double,
                            C.c_double, i], i),
    }
    for name, (argt, rest) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = argt
        fn.restype = rest
    _lib = lib
    return lib


def shed_words(roi: int) -> int:
    """uint64 words per viewshed: (2roi+1) * ceil((2roi+1)/64)."""
    nr = 2 * roi + 1
    return nr * ((nr + 63) // 64)


def _ptr(a) -> int:
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a)


def block_geometry(nrows: int, bw: int, nwanted0: int) -> Geometry:
    g = _GeometryC()
    rc = load().siting_block_geometry(nrows, bw, nwanted0, C.byref(g))
    if rc:
        raise SitingError(rc, "The last block is too small for nwantedperblock.")
    return Geometry(g.blocksize, g.nblocks, g.nwantedperblock, g.nwanted)


def validate(p: Params, lib_form: bool = True) -> str | None:
    """Returns None if p is acceptable, else the reference's message."""
    buf = C.create_string_buffer(256)
    pc = p.c()
    rc = load().siting_validate(C.byref(pc), 1 if lib_form else 0, buf, 256)
    return None if rc == OK else buf.value.decode()


def fbm_dem(nrows: int, seed: int, octaves: int = 8, persistence: float = 0.5,
            lacunarity: float = 2.0, base_wavelength: float = 256.0, ridged_weight: float = 0.0,
            range_max: int = 10000) -> np.ndarray:
    """Seeded fBm terrain, uint16[nrows*nrows] row-major."""
    out = np.empty(nrows * nrows, np.uint16)
    rc = load().siting_fbm_dem(out.ctypes.data, nrows, seed, octaves, persistence, lacunarity,
                               base_wavelength, ridged_weight, range_max)
    if rc:
        raise SitingError(rc, "fbm_dem: invalid arguments")
    return out


def read_dem(path: str, nrows: int) -> np.ndarray:
    out = np.empty(nrows * nrows, np.uint16)
    rc = load().siting_read_dem(path.encode(), nrows, out.ctypes.data)
    if rc:
        raise SitingError(rc, "Input failed")
    return out


def write_observers(path: str, nrows: int, obs: np.ndarray, selected: np.ndarray) -> None:
    obs = np.ascontiguousarray(obs, np.int32)
    selected = np.ascontiguousarray(selected, np.uint8)
    rc = load().siting_write_observers(path.encode(), nrows, len(obs), obs.ctypes.data,
                                       selected.ctypes.data)
    if rc:
        raise SitingError(rc, "Output failed")


def observers_text(obs: np.ndarray, selected: np.ndarray, nrows: int) -> bytes:
    """The observers file's bytes: 'x,y\\n' per selected index in index order."""
    idx = np.nonzero(np.asarray(selected))[0]
    o = np.asarray(obs)[idx]
    return "".join(f"{v // nrows},{v % nrows}\n" for v in o.tolist()).encode()


class Context:
    """A device context: CUDA stream + resident workspace (HBM budget)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._lib = load()
        h = _P()
        rc = self._lib.siting_ctx_create(device, hbm_budget, C.byref(h))
        if rc:
            raise SitingError(rc, f"siting_ctx_create(device={device}) failed: "
                                  f"{self._lib.siting_status_string(rc).decode()}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._lib.siting_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc:
            raise SitingError(rc, self._lib.siting_last_error(self.h).decode())

    @property
    def stream(self) -> int:
        return self._lib.siting_ctx_stream(self.h) or 0

    def sync(self):
        self._check(self._lib.siting_ctx_sync(self.h))

    def workspace_bytes(self) -> int:
        return self._lib.siting_ctx_workspace_bytes(self.h)

    def trim(self):
        self._check(self._lib.siting_ctx_trim(self.h))

    def set_site_ctas(self, n: int):
        self._check(self._lib.siting_ctx_set_site_ctas(self.h, n))

    def set_batch_mode(self, mode: int):
        """How batches run VIX and FINDMAX: 0 automatic, 1 one queued launch per
        SITE launch (FINDMAX fused), 2 one launch per stage and job."""
        self._check(self._lib.siting_ctx_set_batch_mode(self.h, mode))

    def set_batch_graphs(self, on: bool):
        """Device-resident batches captured and replayed as CUDA graphs (default on)."""
        self._check(self._lib.siting_ctx_set_batch_graphs(self.h, int(bool(on))))

    def batch_graph_stats(self) -> tuple[int, int]:
        """(graphs captured, graphs replayed) by this context's batches."""
        c, r = C.c_longlong(), C.c_longlong()
        self._check(self._lib.siting_ctx_batch_graph_stats(self.h, C.byref(c), C.byref(r)))
        return c.value, r.value

    # ---- stages on host arrays (reference signatures) -----------------------
    def calc_vix(self, nrows, elevs, roi, oht, tht, ntests) -> np.ndarray:
        elevs = np.ascontiguousarray(elevs, np.uint16).ravel()
        vix = np.empty(nrows * nrows, np.uint8)
        self._check(self._lib.siting_calc_vix(self.h, nrows, elevs.ctypes.data, roi, oht, tht,
                                              ntests, vix.ctypes.data))
        return vix

    def find_max(self, nrows, vix, blocksize, nwanted, nblocks, nwantedperblock) -> np.ndarray:
        """Returns obs; `vix` (uint8 numpy, modified in place as the reference does)."""
        assert vix.dtype == np.uint8 and vix.flags.c_contiguous
        obs = np.empty(nwanted, np.int32)
        self._check(self._lib.siting_find_max(self.h, nrows, vix.ctypes.data, blocksize, nwanted,
                                              nblocks, nwantedperblock, obs.ctypes.data))
        return obs

    def calc_sheds(self, nrows, elevs, roi, oht, tht, obs) -> np.ndarray:
        elevs = np.ascontiguousarray(elevs, np.uint16).ravel()
        obs = np.ascontiguousarray(obs, np.int32)
        sheds = np.empty(len(obs) * shed_words(roi), np.uint64)
        self._check(self._lib.siting_calc_sheds(self.h, nrows, elevs.ctypes.data, roi, oht, tht,
                                                len(obs), obs.ctypes.data, sheds.ctypes.data))
        return sheds

    def site_it(self, nrows, roi, intervis, obs, sheds):
        """Returns (selected uint8[nsheds], Result)."""
        obs = np.ascontiguousarray(obs, np.int32)
        sheds = np.ascontiguousarray(sheds, np.uint64)
        sel = np.empty(len(obs), np.uint8)
        r = _ResultC()
        self._check(self._lib.siting_site_it(self.h, nrows, roi, intervis, len(obs),
                                             obs.ctypes.data, sheds.ctypes.data, sel.ctypes.data,
                                             C.byref(r)))
        return sel, Result.of(r)

    # ---- stages on device buffers (pointers or torch tensors) ----------------
    def calc_vix_dev(self, nrows, d_elevs, roi, oht, tht, ntests, d_vix):
        self._check(self._lib.siting_calc_vix_dev(self.h, nrows, _ptr(d_elevs), roi, oht, tht,
                                                  ntests, _ptr(d_vix)))

    def find_max_dev(self, nrows, d_vix, blocksize, nwanted, nblocks, npb, d_obs):
        self._check(self._lib.siting_find_max_dev(self.h, nrows, _ptr(d_vix), blocksize, nwanted,
                                                  nblocks, npb, _ptr(d_obs)))

    def calc_sheds_dev(self, nrows, d_elevs, roi, oht, tht, nsheds, d_obs, d_sheds):
        self._check(self._lib.siting_calc_sheds_dev(self.h, nrows, _ptr(d_elevs), roi, oht, tht,
                                                    nsheds, _ptr(d_obs), _ptr(d_sheds)))

    def site_it_dev(self, nrows, roi, intervis, nsheds, d_obs, d_sheds, d_selected) -> Result:
        r = _ResultC()
        self._check(self._lib.siting_site_it_dev(self.h, nrows, roi, intervis, nsheds, _ptr(d_obs),
                                                 _ptr(d_sheds), _ptr(d_selected), C.byref(r)))
        return Result.of(r)

    def last_pick_order(self, cap: int) -> np.ndarray:
        """Candidate indices of the last SITE run, in pick order."""
        out = np.empty(max(cap, 0), np.int32)
        cnt = C.c_int()
        self._check(self._lib.siting_last_pick_order(self.h, out.ctypes.data, cap, C.byref(cnt)))
        return out[:cnt.value]

    def last_site_phase_cycles(self) -> list:
        """Device cycles per SITE phase (CTA 0) of the last run."""
        out = (C.c_longlong * 13)()
        self._check(self._lib.siting_last_site_phase_cycles(self.h, out, 13))
        return list(out)

    # ---- whole pipeline ---------------------------------------------------------
    def run(self, p: Params, elevs):
        """Host DEM in, (obs, selected, Result) out."""
        elevs = np.ascontiguousarray(elevs, np.uint16).ravel() if isinstance(elevs, np.ndarray) \
            else elevs
        g = block_geometry(p.nrows, p.bw, p.nwanted0)
        obs = np.empty(g.nwanted, np.int32)
        sel = np.empty(g.nwanted, np.uint8)
        r = _ResultC()
        pc = p.c()
        self._check(self._lib.siting_run(self.h, C.byref(pc), _ptr(elevs), obs.ctypes.data,
                                         sel.ctypes.data, C.byref(r)))
        return obs, sel, Result.of(r)

    def run_into(self, p: Params, elevs_ptr, obs_ptr, sel_ptr) -> Result:
        """Host pointers (e.g. pinned buffers) in and out."""
        r = _ResultC()
        pc = p.c()
        self._check(self._lib.siting_run(self.h, C.byref(pc), _ptr(elevs_ptr), _ptr(obs_ptr),
                                         _ptr(sel_ptr), C.byref(r)))
        return Result.of(r)

    def run_dev(self, p: Params, d_elevs, d_obs, d_selected) -> Result:
        r = _ResultC()
        pc = p.c()
        self._check(self._lib.siting_run_dev(self.h, C.byref(pc), _ptr(d_elevs), _ptr(d_obs),
                                             _ptr(d_selected), C.byref(r)))
        return Result.of(r)

    # ---- batched form ---------------------------------------------------------
    def _batch(self, fn, params, dems, obs, sels, plans):
        nj = len(params)
        pa = (_ParamsC * nj)(*[p.c() for p in params])
        dp = (C.c_void_p * nj)(*[_ptr(d) for d in dems])
        op = (C.c_void_p * nj)(*[_ptr(o) for o in obs])
        sp = (C.c_void_p * nj)(*[_ptr(x) for x in sels])
        res = (_ResultC * nj)()
        pl = (_PlanC * nj)(*[q.c() for q in plans]) if plans is not None else None
        self._check(fn(self.h, nj, pa, dp, op, sp, res, pl))
        return [Result.of(r) for r in res]

    def run_batch(self, params, dems, plans=None):
        """Host DEMs in; per job (obs, selected, Result)."""
        dems = [np.ascontiguousarray(d, np.uint16).ravel() for d in dems]
        geos = [block_geometry(p.nrows, p.bw, p.nwanted0) for p in params]
        obs = [np.empty(g.nwanted, np.int32) for g in geos]
        sels = [np.empty(g.nwanted, np.uint8) for g in geos]
        res = self._batch(self._lib.siting_run_batch, params, dems, obs, sels, plans)
        return list(zip(obs, sels, res))

    def run_batch_dev(self, params, d_dems, d_obs, d_sels, plans=None):
        """Device buffers (pointers or tensors) in and out; per job Result."""
        return self._batch(self._lib.siting_run_batch_dev, params, d_dems, d_obs, d_sels, plans)

    def autotune(self, p: Params, dem: np.ndarray, sample_rows: int = 1024) -> Plan:
        """Times the stages' launch plans on a corner of dem and keeps the
        fastest for (roi, ntests) in this context; returns it."""
        dem = np.ascontiguousarray(dem, np.uint16).ravel()
        pc = p.c()
        out = _PlanC()
        self._check(self._lib.siting_autotune(self.h, C.byref(pc), dem.ctypes.data, sample_rows,
                                              C.byref(out)))
        return Plan(out.vix_tile, out.vix_smem, out.shed_smem, out.site_ctas)

    def selftest_wait(self, which: int, max_cycles: int = 1 << 22) -> int:
        """Status of a bounded device wait run against a condition never met
        (0: SITE group barrier, 1: TMA mbarrier): ETIMEOUT when it expired as
        designed.  Does not raise."""
        return self._lib.siting_selftest_wait(self.h, which, max_cycles)

    def autotune_set(self, roi: int, ntests: int, plan: Plan):
        """Keep `plan` for jobs with this (roi, ntests), as a tuned plan."""
        pc = plan.c()
        self._check(self._lib.siting_autotune_set(self.h, roi, ntests, C.byref(pc)))

    def autotune_clear(self):
        self._check(self._lib.siting_autotune_clear(self.h))

    def batch_workspace_bytes(self, params, plans=None) -> int:
        """Device workspace run_batch would take for these jobs (no device work)."""
        nj = len(params)
        pa = (_ParamsC * nj)(*[p.c() for p in params])
        pl = (_PlanC * nj)(*[q.c() for q in plans]) if plans is not None else None
        out = C.c_size_t()
        self._check(self._lib.siting_batch_workspace_bytes(self.h, nj, pa, pl, C.byref(out)))
        return out.value


@dataclass
class JobInfo:
    """Outcome of one served job; times in seconds since the server started."""
    status: int
    result: Result
    t_submit: float
    t_start: float
    t_done: float
    batch_id: int
    batch_jobs: int
    error: str

    @property
    def latency_s(self) -> float:
        return self.t_done - self.t_submit


@dataclass
class Ticket:
    id: int
    params: Params
    obs: np.ndarray
    selected: np.ndarray
    dem: np.ndarray  # kept alive until the job is waited for


class Server:
    """Serving loop: submitted jobs are admitted to the GPU while others are
    in flight, as memory and slots free up, under an HBM budget
    (siting_server_* in the library; one worker thread owns the GPU)."""

    def __init__(self, device: int = 0, hbm_budget: int = 8 << 30, max_batch_jobs: int = 64,
                 reserve: bool = False):
        self._lib = load()
        h = _P()
        rc = self._lib.siting_server_create(device, hbm_budget, max_batch_jobs, int(reserve),
                                            C.byref(h))
        if rc:
            raise SitingError(rc, f"siting_server_create(device={device}) failed: "
                                  f"{self._lib.siting_status_string(rc).decode()}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._lib.siting_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def submit(self, p: Params, dem: np.ndarray) -> Ticket:
        """Queues one job.  dem: uint16, either nrows*nrows contiguous or a 2-D
        window (row stride in whole elements) of a larger raster."""
        if dem.dtype != np.uint16:
            raise SitingError(EINVAL, "dem must be uint16")
        pitch = 0
        if dem.ndim == 2:
            if dem.strides[1] != 2 or dem.strides[0] % 2 or dem.shape != (p.nrows, p.nrows):
                raise SitingError(EINVAL, "dem window must be nrows x nrows with unit column stride")
            pitch = dem.strides[0] // 2
        elif not dem.flags.c_contiguous or dem.size != p.nrows * p.nrows:
            raise SitingError(EINVAL, "dem must hold nrows*nrows contiguous elements")
        g = block_geometry(p.nrows, p.bw, p.nwanted0)
        obs = np.empty(g.nwanted, np.int32)
        sel = np.empty(g.nwanted, np.uint8)
        pc = p.c()
        tid = C.c_longlong()
        rc = self._lib.siting_server_submit(self.h, C.byref(pc), dem.ctypes.data, pitch,
                                            obs.ctypes.data, sel.ctypes.data, C.byref(tid))
        if rc:
            raise SitingError(rc, f"submit refused: {self._lib.siting_status_string(rc).decode()}")
        return Ticket(tid.value, p, obs, sel, dem)

    def wait(self, t: Ticket, timeout: float | None = None):
        """(obs, selected, JobInfo) once the job is done; TimeoutError if it is
        not done within timeout seconds."""
        info = _JobInfoC()
        rc = self._lib.siting_server_wait(self.h, t.id, -1.0 if timeout is None else timeout,
                                          C.byref(info))
        if rc == ETIMEOUT:
            raise TimeoutError(f"job {t.id} not done within {timeout} s")
        if rc:
            raise SitingError(rc, f"wait({t.id}) failed")
        ji = JobInfo(info.status, Result.of(info.result), info.t_submit, info.t_start,
                     info.t_done, info.batch_id, info.batch_jobs, info.error.decode())
        if ji.status:
            raise SitingError(ji.status, ji.error)
        return t.obs, t.selected, ji

    def stats(self) -> dict:
        st = _ServerStatsC()
        rc = self._lib.siting_server_stats_get(self.h, C.byref(st))
        if rc:
            raise SitingError(rc, "stats failed")
        return {f: getattr(st, f) for f, _ in _ServerStatsC._fields_}
