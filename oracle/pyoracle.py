"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes bindings of the two CPU oracles (see oracle/README.md).  Imported by
tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
as the checker; the product never imports it.

  build()            compile oracle/_build/liboracle.so (always) and
                     oracle/_ref/libmcfl_ref.so (only where the reference
                     checkout is present)
  Oracle             the restatement (port.cpp)
  RefOracle          the reference's own transport built for the host
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PORT = os.path.join(HERE, "_build", "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libmcfl_ref.so")

u64p = ctypes.POINTER(ctypes.c_ulonglong)
f64p = ctypes.POINTER(ctypes.c_double)


class CResult(ctypes.Structure):
    _fields_ = [
        ("grid", ctypes.c_int * 3),
        ("image", ctypes.c_int * 2),
        ("number_of_photons", ctypes.c_ulonglong),
        ("photons_exc", ctypes.c_ulonglong),
        ("photons_fl", ctypes.c_ulonglong),
        ("fl_voxels", ctypes.c_long),
        ("failed_voxels", ctypes.c_long),
        ("Rd", u64p),
        ("Tt", u64p),
        ("fhd", u64p),
        ("flR", f64p),
        ("flT", f64p),
        ("flR128", u64p),
        ("flT128", u64p),
        ("balance", ctypes.c_ulonglong * 6),
        ("steps_exc", ctypes.c_ulonglong),
        ("steps_fl", ctypes.c_ulonglong),
        ("time_xyt", u64p),
        ("time_size", ctypes.c_long),
        ("seconds_exc", ctypes.c_double),
        ("seconds_fl", ctypes.c_double),
    ]


MAX_BULKS = 100


class CBulk(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("mutr", "mua", "g", "n", "flc", "muaf", "eY", "albedof", "mus")]


MAX_LAYERS = 100


class CLayer(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("z_min", "z_max", "mutr", "mua", "g", "n", "flc", "muaf", "eY",
                                              "albedof")]


class CInclusion(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("x", "y", "z", "r", "mutr", "mua", "g", "n", "flc", "muaf", "eY",
                                              "albedof")]


class CSim(ctypes.Structure):
    _fields_ = [
        ("number_of_photons", ctypes.c_ulonglong),
        ("number_of_photons_per_voxel", ctypes.c_uint),
        ("n_bulks", ctypes.c_uint),
        ("start_weight", ctypes.c_uint),
        ("grid_size", ctypes.c_int),
        ("esp", ctypes.c_float),
        ("xi", ctypes.c_float),
        ("yi", ctypes.c_float),
        ("zi", ctypes.c_float),
        ("dir", ctypes.c_float),
        ("fhd_activated", ctypes.c_int),
        ("do_fl_sim", ctypes.c_int),
        ("bulk_method", ctypes.c_int),
        ("det_dx", ctypes.c_float),
        ("det_dy", ctypes.c_float),
        ("det_nx", ctypes.c_int),
        ("det_ny", ctypes.c_int),
        ("det_x0", ctypes.c_float),
        ("det_y0", ctypes.c_float),
        ("bulks", CBulk * (MAX_BULKS + 2)),
        ("bulk_info", ctypes.POINTER(ctypes.c_short)),
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("nz", ctypes.c_int),
        ("half_x", ctypes.c_float),
        ("half_y", ctypes.c_float),
        ("vox_per_cm", ctypes.c_float * 3),
        ("fluor_map", ctypes.POINTER(ctypes.c_float)),
        ("max_fl_voxels", ctypes.c_long),
        ("launch_rng_reuse", ctypes.c_int),
        ("do_temp_sim", ctypes.c_int),
        ("tdet_x0", ctypes.c_float),
        ("tdet_y0", ctypes.c_float),
        ("tdet_nx", ctypes.c_int),
        ("tdet_ny", ctypes.c_int),
        ("tdet_sep_x", ctypes.c_float),
        ("tdet_sep_y", ctypes.c_float),
        ("tdet_r", ctypes.c_float),
        ("tdet_face", ctypes.c_int),
        ("tdet_bins", ctypes.c_long),
        ("tdet_max", ctypes.c_ulonglong),
        ("n_layers", ctypes.c_int),
        ("layers", CLayer * (MAX_LAYERS + 2)),
        ("inclusion", CInclusion),
        ("photon_offset", ctypes.c_ulonglong),
        ("exact_stepping", ctypes.c_int),
    ]


@dataclass
class Result:
    grid: tuple
    image: tuple
    number_of_photons: int
    photons_exc: int
    photons_fl: int
    fl_voxels: int
    failed_voxels: int
    Rd: np.ndarray  # uint64, nx + nx*ny
    Tt: np.ndarray
    fhd: np.ndarray  # uint64, grid
    flR: np.ndarray  # float64, nx + nx*ny
    flT: np.ndarray
    flR128: np.ndarray | None  # uint64 (n, 2): lo, hi
    flT128: np.ndarray | None
    balance: tuple
    steps_exc: int
    steps_fl: int
    time_xyt: np.ndarray | None = None  # uint64, index ix + nx*(iy + ny*bin)
    seconds_exc: float = 0.0  # reference streams: wall-clock of the excitation phase
    seconds_fl: float = 0.0   # reference streams: wall-clock of the emission phase


def _to_result(lib, r: CResult) -> Result:
    nx, ny = r.image[0], r.image[1]
    xy = nx + nx * ny
    nvox = r.grid[0] * r.grid[1] * r.grid[2]

    def arr(ptr, n, dt):
        if not ptr or n <= 0:
            return None
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)

    out = Result(
        grid=tuple(r.grid), image=(nx, ny), number_of_photons=r.number_of_photons,
        photons_exc=r.photons_exc, photons_fl=r.photons_fl, fl_voxels=r.fl_voxels,
        failed_voxels=r.failed_voxels,
        Rd=arr(r.Rd, xy, np.uint64), Tt=arr(r.Tt, xy, np.uint64), fhd=arr(r.fhd, nvox, np.uint64),
        flR=arr(r.flR, xy, np.float64), flT=arr(r.flT, xy, np.float64),
        flR128=None if not r.flR128 else arr(r.flR128, 2 * xy, np.uint64).reshape(xy, 2),
        flT128=None if not r.flT128 else arr(r.flT128, 2 * xy, np.uint64).reshape(xy, 2),
        balance=tuple(r.balance), steps_exc=r.steps_exc, steps_fl=r.steps_fl,
        time_xyt=arr(r.time_xyt, r.time_size, np.uint64), seconds_exc=r.seconds_exc, seconds_fl=r.seconds_fl,
    )
    lib.oracle_free_result(ctypes.byref(r))
    return out


def build(reference_dir: str | None = None, quiet: bool = True) -> None:
    """Build the restatement, and the reference build where its sources exist."""
    kw = dict(cwd=HERE, check=True)
    if quiet:
        kw.update(stdout=subprocess.DEVNULL, stderr=subprocess.PIPE)
    subprocess.run(["make", "-s", "all"], **kw)
    args = ["make", "-s", "ref"]
    if reference_dir:
        args.append(f"REFERENCE_DIR={reference_dir}")
    subprocess.run(args, **kw)


def reference_dir() -> str:
    """The reference checkout the host build of the reference compiles from:
    REFERENCE_DIR of the environment, else the Makefile's default."""
    env = os.environ.get("REFERENCE_DIR")
    if env:
        return env
    r = subprocess.run(["make", "-s", "refdir"], cwd=HERE, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                       text=True)
    return r.stdout.strip()


def _load(path):
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = ctypes.CDLL(path)
    lib.oracle_free_result.argtypes = [ctypes.POINTER(CResult)]
    return lib


class Oracle:
    """The CPU restatement (port.cpp)."""

    def __init__(self, path: str = LIB_PORT):
        self.lib = _load(path)
        L = self.lib
        L.oracle_run_refstream.argtypes = [ctypes.POINTER(CSim), ctypes.c_char_p, ctypes.c_ulonglong,
                                           ctypes.c_ulonglong, ctypes.c_int, ctypes.c_int, ctypes.POINTER(CResult)]
        L.oracle_run_photon.argtypes = [ctypes.POINTER(CSim), ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint,
                                        ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(CResult)]
        L.oracle_safeprime_multipliers.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int]
        L.oracle_write_safeprimes.argtypes = [ctypes.c_char_p, ctypes.c_int]

    def multipliers(self, count: int = 32769) -> np.ndarray:
        out = np.zeros(count, dtype=np.uint32)
        n = self.lib.oracle_safeprime_multipliers(out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), count)
        if n != count:
            raise RuntimeError("multiplier search exhausted")
        return out

    def write_safeprimes(self, path: str, count: int = 32769) -> None:
        if self.lib.oracle_write_safeprimes(path.encode(), count) != 0:
            raise RuntimeError("could not write " + path)

    def run_refstream(self, sim: "CSim", safeprimes: str, seed_exc: int, seed_fl: int, libm: bool = True,
                      nthreads: int = 1) -> Result:
        r = CResult()
        rc = self.lib.oracle_run_refstream(ctypes.byref(sim), safeprimes.encode(), seed_exc, seed_fl,
                                           1 if libm else 0, nthreads, ctypes.byref(r))
        if rc != 0:
            raise RuntimeError(f"oracle_run_refstream failed ({rc})")
        return _to_result(self.lib, r)

    def run_photon(self, sim: "CSim", table32768: np.ndarray, seed_exc: int, seed_fl: int,
                   libm: bool = False, nthreads: int = 0) -> Result:
        """nthreads 0: all host cores; the result does not depend on it."""
        nthreads = nthreads or (os.cpu_count() or 1)
        t = np.ascontiguousarray(table32768, dtype=np.uint32)
        assert t.size == 32768
        r = CResult()
        rc = self.lib.oracle_run_photon(ctypes.byref(sim), t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                        t.size, seed_exc, seed_fl, 1 if libm else 0, nthreads, ctypes.byref(r))
        if rc != 0:
            raise RuntimeError(f"oracle_run_photon failed ({rc})")
        return _to_result(self.lib, r)


class RefOracle:
    """The reference's own transport, compiled for the host (oracle/_ref)."""

    def __init__(self, path: str = LIB_REF):
        self.lib = _load(path)
        L = self.lib
        L.ref_run_mci.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_ulonglong, ctypes.c_ulonglong,
                                  ctypes.c_int, ctypes.c_int, ctypes.POINTER(CResult)]
        L.ref_parse_mci.argtypes = [ctypes.c_char_p, ctypes.POINTER(CSim)]

    @staticmethod
    def available(path: str = LIB_REF) -> bool:
        return os.path.exists(path)

    def run_mci(self, mci: str, safeprimes: str, seed_exc: int, seed_fl: int, nthreads: int = 1,
                write_files: bool = False) -> Result:
        """Runs in the .mci file's directory (the reference opens the bulk
        file and writes its outputs relative to the working directory)."""
        r = CResult()
        cwd = os.getcwd()
        d = os.path.dirname(os.path.abspath(mci))
        try:
            os.chdir(d)
            rc = self.lib.ref_run_mci(os.path.basename(mci).encode(), os.path.abspath(safeprimes).encode(),
                                      seed_exc, seed_fl, nthreads, 1 if write_files else 0, ctypes.byref(r))
        finally:
            os.chdir(cwd)
        if rc != 0:
            raise RuntimeError(f"ref_run_mci failed ({rc})")
        return _to_result(self.lib, r)

    def parse_mci(self, mci: str) -> "CSim":
        s = CSim()
        cwd = os.getcwd()
        try:
            os.chdir(os.path.dirname(os.path.abspath(mci)))
            rc = self.lib.ref_parse_mci(os.path.basename(mci).encode(), ctypes.byref(s))
        finally:
            os.chdir(cwd)
        if rc != 0:
            raise RuntimeError(f"ref_parse_mci failed ({rc})")
        return s


def sim_from_fields(labels: np.ndarray, bulks: list[dict], *, esp: float, grid_size: int, photons: int,
                    photons_per_voxel: int, det: tuple, source: tuple, do_fl: int = 1, dir_: float = 1.0,
                    n_out: float = 1.0) -> tuple["CSim", np.ndarray]:
    """Builds a method-2 simulation the way the reference's parser would
    (CUDAMCFLio.cu:528-652).  bulks: one dict per label 1..n with keys
    n, mua, mus, flc, absc_exi, absc_emi, eY, g (the .mci columns)."""
    s = CSim()
    s.bulk_method = 2
    s.number_of_photons = photons
    s.number_of_photons_per_voxel = photons_per_voxel
    s.grid_size = grid_size
    s.esp = esp
    s.do_fl_sim = do_fl
    s.fhd_activated = 1 if do_fl in (1, 2) else 0
    (s.det_dx, s.det_dy, s.det_nx, s.det_ny, s.det_x0, s.det_y0) = det
    s.xi, s.yi, s.zi = source
    s.dir = dir_
    n = len(bulks)
    s.n_bulks = n
    f32 = np.float32
    s.bulks[0] = CBulk(float(np.finfo(np.float32).max), 0.0, 1.0, n_out, 0.0, 0.0, 0.0, 0.0)
    s.bulks[n + 1] = CBulk(float(np.finfo(np.float32).max), 0.0, 1.0, n_out, 0.0, 0.0, 0.0, 0.0)
    for i, b in enumerate(bulks, start=1):
        mua, mus, flc = f32(b["mua"]), f32(b["mus"]), f32(b["flc"])
        ax, am = f32(b["absc_exi"]), f32(b["absc_emi"])
        mutr = f32(np.finfo(np.float32).max) if mus == 0 else f32(f32(1.0) / f32(mua + mus))
        s.bulks[i] = CBulk(mutr, f32(mua + flc * ax), f32(b["g"]), f32(b["n"]), flc, f32(mua + flc * am),
                           f32(b["eY"]), f32(mus / f32(flc * ax + mus)), mus)
    r = (np.float64(n_out) - np.float64(f32(bulks[0]["n"]))) / (np.float64(n_out) + np.float64(f32(bulks[0]["n"])))
    s.start_weight = int(np.float64(0xFFFFFFFF) * (1 - r * r))
    lab = np.ascontiguousarray(labels, dtype=np.int16)
    s.bulk_info = lab.ctypes.data_as(ctypes.POINTER(ctypes.c_short))
    return s, lab


def sim_from_arrays(labels: np.ndarray, bulks, *, half_x: float, half_y: float, thickness: float, vox_per_cm,
                    photons: int, per_voxel: int, det: tuple, source=(0.0, 0.0, 0.0), start_weight: int = 0,
                    fluor_map: np.ndarray | None = None, do_fl: int = 1) -> "CSim":
    """A general-geometry simulation over (nz, ny, nx) labels with the same
    floats the engine uses for its medium.  bulks: objects with the fields of
    mcfl_bulk (mutr, mua, g, n, flc, muaf, eY, albedof), n+2 entries.  The
    returned structure keeps its arrays alive."""
    s = CSim()
    s.bulk_method = 2
    s.number_of_photons = photons
    s.number_of_photons_per_voxel = per_voxel
    s.esp = thickness
    s.grid_size = 0
    s.do_fl_sim = do_fl
    s.fhd_activated = 1 if do_fl in (1, 2) else 0
    s.det_dx, s.det_dy, s.det_nx, s.det_ny, s.det_x0, s.det_y0 = det
    s.xi, s.yi, s.zi = source
    s.dir = 1.0
    s.n_bulks = len(bulks) - 2
    for i, b in enumerate(bulks):
        s.bulks[i] = CBulk(b.mutr, b.mua, b.g, b.n, b.flc, b.muaf, b.eY, b.albedof, b.mus)
    if start_weight == 0:
        n1, n2 = np.float64(np.float32(bulks[0].n)), np.float64(np.float32(bulks[1].n))
        r = (n1 - n2) / (n1 + n2)
        start_weight = int(np.float64(0xFFFFFFFF) * (1 - r * r))
    s.start_weight = start_weight
    lab = np.ascontiguousarray(labels.astype(np.int16))
    s.bulk_info = lab.ctypes.data_as(ctypes.POINTER(ctypes.c_short))
    s.nz, s.ny, s.nx = lab.shape
    s.half_x, s.half_y = half_x, half_y
    s.vox_per_cm[:] = list(vox_per_cm)
    keep = [lab]
    if fluor_map is not None:
        fm = np.ascontiguousarray(fluor_map, dtype=np.float32)
        s.fluor_map = fm.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        keep.append(fm)
    s._keep = keep
    return s
