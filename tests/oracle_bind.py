"""ctypes bindings to the CPU oracle (test infrastructure only).

Two CPU implementations share one Python interface:

* ``Oracle("port")``: the C restatement ``oracle/siting_oracle.c`` (seqsite
  semantics, OpenMP), built by ``oracle/Makefile`` on any machine.
* ``Oracle("reference")``: the reference's own ``siting.cpp`` compiled with
  ``-DSEQ`` from its sources (``oracle/_ref/libsitingref.so``); present only
  where those sources were available to build it (a reference checkout, or
  the git-ignored copy ``make -C oracle stage`` puts in ``oracle/_ref/src``).
* ``Oracle("reference_omp")``: the same source built with OpenMP (ompsite in
  library form), for timing only.

Only tests, the smoke check and the bench's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
import threading

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
PORT_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_DIR = os.path.join(ORACLE_DIR, "_ref")
# the reference's own files, staged from a reference checkout by
# `make -C oracle stage` (git-ignored; travels with the working tree)
REF_SRC = os.environ.get("SITING_REFERENCE_SRC", os.path.join(REF_DIR, "src"))
REF_SO = os.path.join(REF_DIR, "libsitingref.so")
REF_OMP_SO = os.path.join(REF_DIR, "libsitingref_omp.so")
REF_OMPSITE = os.path.join(REF_DIR, "ompsite")
REF_CUSITE = os.path.join(REF_DIR, "cusite_sm103a")

_lock = threading.Lock()
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


def build_port() -> str:
    """Build liboracle.so with make if it is missing or stale."""
    with _lock:
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"], check=True)
    return PORT_SO


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def ref_dem_bin() -> str | None:
    """The reference's sample DEM (dem.bin), if it is staged here."""
    p = os.path.join(REF_SRC, "dem.bin")
    return p if os.path.exists(p) else None


def _load(path: str) -> C.CDLL:
    return C.CDLL(path, mode=C.RTLD_LOCAL)


class Geometry:
    """Block geometry of siting.cpp:688-695."""

    def __init__(self, bs, nb, npb, nwanted, too_small):
        self.blocksize = bs
        self.nblocks = nb
        self.nwantedperblock = npb
        self.nwanted = nwanted
        self.too_small = bool(too_small)

    def __repr__(self):
        return (f"Geometry(bs={self.blocksize}, nb={self.nblocks}, "
                f"npb={self.nwantedperblock}, nwanted={self.nwanted})")


class Oracle:
    """Stage-level CPU pipeline with the reference's semantics."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            lib = _load(build_port() if not os.path.exists(PORT_SO) else PORT_SO)
            lib.oracle_geometry.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float),
                                            C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
            lib.oracle_calc_vix.argtypes = [C.c_int, _u16p, C.c_int, C.c_int, C.c_int, C.c_int, _u8p]
            lib.oracle_find_max.argtypes = [C.c_int, _u8p, C.c_float, C.c_int, C.c_int, _i32p]
            lib.oracle_calc_sheds.argtypes = [C.c_int, _u16p, C.c_int, C.c_int, C.c_int, C.c_int,
                                              _i32p, _u64p]
            lib.oracle_site_it.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _u64p, _u8p,
                                           C.POINTER(C.c_longlong), C.c_void_p]
            lib.oracle_site_it.restype = C.c_int
            lib.oracle_union_count.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _u64p, _u8p]
            lib.oracle_union_count.restype = C.c_longlong
            lib.oracle_vix_work.argtypes = [C.c_int, _u16p, C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
            lib.oracle_vix_cells.argtypes = [C.c_int, _u16p, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_void_p, C.c_int, _u8p]
            lib.oracle_threads.restype = C.c_int
            lib.oracle_set_threads.argtypes = [C.c_int]
            lib.oracle_fbm_dem.argtypes = [_u16p, C.c_int, C.c_uint64, C.c_int, C.c_double,
                                           C.c_double, C.c_double, C.c_double, C.c_int]
            lib.oracle_fbm_dem.restype = C.c_int
        elif kind in ("reference", "reference_omp"):
            path = REF_SO if kind == "reference" else REF_OMP_SO
            if not os.path.exists(path):
                raise FileNotFoundError(f"{path} not built (needs the reference sources)")
            lib = _load(path)
            lib.ref_geometry.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float),
                                         C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
            lib.ref_calc_vix.argtypes = [C.c_int, _u16p, C.c_int, C.c_int, C.c_int, C.c_int, _u8p]
            lib.ref_find_max.argtypes = [C.c_int, _u8p, C.c_float, C.c_int, C.c_int, C.c_int, _i32p]
            lib.ref_calc_sheds.argtypes = [C.c_int, _u16p, C.c_int, C.c_int, C.c_int, C.c_int,
                                           _i32p, _u64p]
            lib.ref_site_it.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _i32p, _u64p, _u8p]
            lib.ref_set_threads.argtypes = [C.c_int]
            lib.ref_set_threads.restype = C.c_int
        else:
            raise ValueError(kind)
        self.lib = lib

    def set_threads(self, n: int) -> int:
        """OpenMP threads of the parallel loops; returns the count in force."""
        if self.kind == "port":
            self.lib.oracle_set_threads(n)
            return int(self.lib.oracle_threads())
        return int(self.lib.ref_set_threads(n))

    def fbm_dem(self, nrows: int, seed: int, octaves: int = 8, persistence: float = 0.5,
                lacunarity: float = 2.0, base_wavelength: float = 256.0,
                ridged_weight: float = 0.0, range_max: int = 10000) -> np.ndarray:
        """Seeded fBm DEM (port only): the same bytes as the library's
        generator for the same arguments, without loading the library."""
        port = self if self.kind == "port" else Oracle("port")
        out = np.empty(nrows * nrows, np.uint16)
        rc = port.lib.oracle_fbm_dem(out, nrows, seed, octaves, persistence, lacunarity,
                                     base_wavelength, ridged_weight, range_max)
        if rc:
            raise ValueError(f"oracle_fbm_dem: status {rc}")
        return out

    # -- stages ------------------------------------------------------------
    def geometry(self, nrows: int, bw: int, nwanted0: int) -> Geometry:
        bs = C.c_float()
        nb, npb, nw = C.c_int(), C.c_int(), C.c_int()
        fn = self.lib.oracle_geometry if self.kind == "port" else self.lib.ref_geometry
        bad = fn(nrows, bw, nwanted0, C.byref(bs), C.byref(nb), C.byref(npb), C.byref(nw))
        return Geometry(bs.value, nb.value, npb.value, nw.value, bad)

    def vix(self, dem: np.ndarray, nrows: int, roi: int, oht: int, tht: int, ntests: int):
        out = np.zeros(nrows * nrows, np.uint8)
        dem = np.ascontiguousarray(dem, np.uint16).ravel()
        fn = self.lib.oracle_calc_vix if self.kind == "port" else self.lib.ref_calc_vix
        fn(nrows, dem, roi, oht, tht, ntests, out)
        return out

    def vix_cells(self, dem: np.ndarray, nrows: int, roi: int, oht: int, tht: int, ntests: int,
                  cells: np.ndarray) -> np.ndarray:
        """VIX of the listed cells only (port only)."""
        cells = np.ascontiguousarray(cells, np.int64)
        out = np.zeros(len(cells), np.uint8)
        dem = np.ascontiguousarray(dem, np.uint16).ravel()
        self.lib.oracle_vix_cells(nrows, dem, roi, oht, tht, ntests, cells.ctypes.data,
                                  len(cells), out)
        return out

    def find_max(self, vix: np.ndarray, nrows: int, geo: Geometry):
        """Returns (obs, vix_after); the input array is not modified."""
        v = np.array(vix, np.uint8, copy=True).ravel()
        obs = np.zeros(geo.nwanted, np.int32)
        if self.kind == "port":
            self.lib.oracle_find_max(nrows, v, geo.blocksize, geo.nblocks, geo.nwantedperblock, obs)
        else:
            self.lib.ref_find_max(nrows, v, geo.blocksize, geo.nwanted, geo.nblocks,
                                  geo.nwantedperblock, obs)
        return obs, v

    def sheds(self, dem: np.ndarray, nrows: int, roi: int, oht: int, tht: int, obs: np.ndarray):
        nr = 2 * roi + 1
        nwpr = (nr + 63) // 64
        out = np.zeros(len(obs) * nr * nwpr, np.uint64)
        dem = np.ascontiguousarray(dem, np.uint16).ravel()
        obs = np.ascontiguousarray(obs, np.int32)
        fn = self.lib.oracle_calc_sheds if self.kind == "port" else self.lib.ref_calc_sheds
        fn(nrows, dem, roi, oht, tht, len(obs), obs, out)
        return out

    def site(self, nrows: int, roi: int, intervis: int, obs: np.ndarray, sheds: np.ndarray,
             want_order: bool = False):
        """Returns (selected u8[nsheds], nused, cumarea[, pick order])."""
        obs = np.ascontiguousarray(obs, np.int32)
        sheds = np.ascontiguousarray(sheds, np.uint64)
        sel = np.zeros(len(obs), np.uint8)
        if self.kind == "port":
            cum = C.c_longlong()
            order = np.zeros(len(obs), np.int32) if want_order else None
            nused = self.lib.oracle_site_it(nrows, roi, intervis, len(obs), obs, sheds, sel,
                                            C.byref(cum),
                                            order.ctypes.data if want_order else None)
            cumarea = cum.value
        else:
            sys.stdout.flush()
            self.lib.ref_site_it(nrows, roi, intervis, len(obs), obs, sheds, sel)
            nused = int(sel.sum())
            cumarea = None
            order = None
        if want_order:
            return sel, nused, cumarea, (order[:nused] if order is not None else None)
        return sel, nused, cumarea

    def union_count(self, nrows, roi, obs, sheds, selected) -> int:
        port = self if self.kind == "port" else Oracle("port")
        return int(port.lib.oracle_union_count(nrows, roi, len(obs), np.ascontiguousarray(obs, np.int32),
                                               np.ascontiguousarray(sheds, np.uint64),
                                               np.ascontiguousarray(selected, np.uint8)))

    def vix_work(self, dem, nrows, roi, oht, tht, ntests):
        a, b = C.c_longlong(), C.c_longlong()
        self.lib.oracle_vix_work(nrows, np.ascontiguousarray(dem, np.uint16).ravel(), roi, oht, tht,
                                 ntests, C.byref(a), C.byref(b))
        return a.value, b.value

    def run(self, dem, nrows, roi, height, ntests, bw, nwanted0, intervis):
        """Whole pipeline; returns a dict of every stage's output."""
        geo = self.geometry(nrows, bw, nwanted0)
        vix = self.vix(dem, nrows, roi, height, height, ntests)
        obs, vix_after = self.find_max(vix, nrows, geo)
        sheds = self.sheds(dem, nrows, roi, height, height, obs)
        sel, nused, cumarea = self.site(nrows, roi, intervis, obs, sheds)
        if cumarea is None:
            cumarea = self.union_count(nrows, roi, obs, sheds, sel)
        return dict(geo=geo, vix=vix, vix_after=vix_after, obs=obs, sheds=sheds,
                    selected=sel, nused=nused, cumarea=cumarea)


def observers_text(obs: np.ndarray, selected: np.ndarray, nrows: int) -> bytes:
    """Observers file of siting.cpp:761-765: 'x,y\\n' per selected index."""
    idx = np.nonzero(np.asarray(selected))[0]
    o = np.asarray(obs)[idx]
    return "".join(f"{v // nrows},{v % nrows}\n" for v in o.tolist()).encode()


def fnv1a64(a: np.ndarray) -> str:
    """FNV-1a 64 over the raw bytes of an array (hex)."""
    data = np.ascontiguousarray(a).view(np.uint8)
    h = 0xcbf29ce484222325
    # vectorised in chunks is not possible for FNV; use python over bytes for
    # small arrays and a C-speed fallback via numpy for large ones
    prime = 0x100000001b3
    mask = 0xFFFFFFFFFFFFFFFF
    for b in data.tobytes():
        h = ((h ^ b) * prime) & mask
    return f"{h:016x}"
