"""GB300 photon-transport engine for voxelized fluorescent turbid media.

Python view of the C ABI in ``include/mcfl.h`` (libmcfl.so, built in-tree by
``cudamcfl_gb300.build``).  The transport runs only in the CUDA library: when
the library is missing, importing :data:`lib` raises instead of falling back
to anything else.

    ctx = Context()                      # one GPU
    med = ctx.medium(labels, bulks, voxel_cm=(0.02, 0.02, 0.02))
    res = ctx.run(med, photons=10**6, photons_per_voxel=1000,
                  source=(0.0, 0.0, 0.0), det=Detector(0, 0, 0.04, 0.04, 100, 100))
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

MATH_EXACT = 0
MATH_FAST = 1
MATH_F64 = 2  # the same kernel in double precision (precision study)
SOURCE_GAUSS_BEAM = 1
SOURCE_WIDEFIELD = 3
NSTATS = 9
STAT_NAMES = ("done", "steps", "absorbed", "exit_top", "exit_bottom", "roulette_loss", "roulette_gain",
              "zero_drop_loss", "capped")
STR_LEN = 500
MAX_BULKS = 253

OK, E_ARG, E_CUDA, E_IO, E_PARSE, E_NOMEM, E_STATE, E_RANGE, E_BUSY, E_TIMEOUT, E_CAPPED = (
    0, -1, -2, -3, -4, -5, -6, -7, -8, -9, -10)


class McflError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


# ----------------------------------------------------------------- structs

class Bulk(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("mutr", "mua", "g", "n", "flc", "muaf", "eY", "albedof", "mus")]


class Layer(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("z_min", "z_max", "mutr", "mua", "g", "n", "flc", "muaf", "eY",
                                              "albedof")]


class Inclusion(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("x", "y", "z", "r", "mutr", "mua", "g", "n", "flc", "muaf", "eY",
                                              "albedof")]


class Det(ctypes.Structure):
    _fields_ = [("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("x0", ctypes.c_float), ("y0", ctypes.c_float), ("sep", ctypes.c_float),
                ("x0_temp_det", ctypes.c_float), ("y0_temp_det", ctypes.c_float),
                ("x_temp_numdets", ctypes.c_uint), ("y_temp_numdets", ctypes.c_uint),
                ("x_temp_sepdets", ctypes.c_float), ("y_temp_sepdets", ctypes.c_float),
                ("temp_det_r", ctypes.c_float), ("temp_rort", ctypes.c_uint),
                ("temp_bins", ctypes.c_ulong), ("max_temp", ctypes.c_ulong)]


class Simulation(ctypes.Structure):
    _fields_ = [("number_of_photons", ctypes.c_ulonglong), ("number_of_photons_per_voxel", ctypes.c_uint),
                ("n_layers", ctypes.c_uint), ("n_bulks", ctypes.c_uint), ("start_weight", ctypes.c_uint),
                ("outp_filename", ctypes.c_char * STR_LEN), ("inp_filename", ctypes.c_char * STR_LEN),
                ("begin", ctypes.c_long), ("end", ctypes.c_long), ("AorB", ctypes.c_char),
                ("det", Det), ("layers", ctypes.POINTER(Layer)), ("bulks", ctypes.POINTER(Bulk)),
                ("inclusion", Inclusion), ("grid_size", ctypes.c_int), ("esp", ctypes.c_float),
                ("xi", ctypes.c_float), ("yi", ctypes.c_float), ("zi", ctypes.c_float), ("dir", ctypes.c_float),
                ("n_down", ctypes.c_float), ("fhd_activated", ctypes.c_int), ("do_fl_sim", ctypes.c_int),
                ("bulk_method", ctypes.c_int), ("bulk_info", ctypes.POINTER(ctypes.c_ubyte)),
                ("bulkinfo_filename", ctypes.c_char * STR_LEN), ("do_temp_sim", ctypes.c_int),
                ("num_x", ctypes.c_int), ("num_y", ctypes.c_int), ("num_z", ctypes.c_int),
                ("bulk_values_read", ctypes.c_longlong)]


class Source(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float),
                ("width", ctypes.c_float), ("height", ctypes.c_float)]


class MediumDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("half_x", ctypes.c_float), ("half_y", ctypes.c_float), ("thickness", ctypes.c_float),
                ("vox_per_cm", ctypes.c_float * 3), ("labels", ctypes.POINTER(ctypes.c_ubyte)),
                ("fluor_map", ctypes.POINTER(ctypes.c_float)), ("n_bulks", ctypes.c_int),
                ("bulks", ctypes.POINTER(Bulk))]


class LayeredDesc(ctypes.Structure):
    _fields_ = [("n_layers", ctypes.c_int), ("layers", ctypes.POINTER(Layer)), ("inclusion", Inclusion),
                ("grid_size", ctypes.c_int)]


class Detector(ctypes.Structure):
    _fields_ = [("x0", ctypes.c_float), ("y0", ctypes.c_float), ("dx", ctypes.c_float), ("dy", ctypes.c_float),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int)]


class TimeDetectors(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("x0", ctypes.c_float), ("y0", ctypes.c_float),
                ("sep_x", ctypes.c_float), ("sep_y", ctypes.c_float), ("radius", ctypes.c_float),
                ("face", ctypes.c_int), ("bins", ctypes.c_int), ("max_fs", ctypes.c_ulonglong)]


class RunDesc(ctypes.Structure):
    _fields_ = [("photons", ctypes.c_ulonglong), ("photons_per_voxel", ctypes.c_uint), ("fluence", ctypes.c_int),
                ("seed_exc", ctypes.c_ulonglong), ("seed_fl", ctypes.c_ulonglong), ("start_weight", ctypes.c_uint),
                ("source", Source), ("det", Detector), ("launch_rng_reuse", ctypes.c_int),
                ("tdet", TimeDetectors), ("photon_offset", ctypes.c_ulonglong), ("exact_stepping", ctypes.c_int)]


_u64p = ctypes.POINTER(ctypes.c_ulonglong)
_f64p = ctypes.POINTER(ctypes.c_double)


class RunOut(ctypes.Structure):
    _fields_ = [("Rd", _u64p), ("Tt", _u64p), ("R", _f64p), ("T", _f64p), ("fhd", _u64p), ("phd", _f64p),
                ("flR", _f64p), ("flT", _f64p), ("flR128", _u64p), ("flT128", _u64p),
                ("stats_exc", ctypes.c_ulonglong * NSTATS), ("stats_fl", ctypes.c_ulonglong * NSTATS),
                ("photons_fl", ctypes.c_ulonglong), ("fl_voxels", ctypes.c_longlong),
                ("energy_exc", ctypes.c_double * 4), ("ms_exc", ctypes.c_float), ("ms_fl", ctypes.c_float),
                ("time_xyt", _u64p)]


SCHEDULE_BATCHED = 0
SCHEDULE_PLAIN = 1


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_ulonglong), ("max_jobs", ctypes.c_uint),
                ("slice_passes", ctypes.c_uint), ("express_period", ctypes.c_uint), ("express_ratio", ctypes.c_uint),
                ("slice_us", ctypes.c_uint)]


class ServerMetrics(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_ulonglong), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("photons", ctypes.c_ulonglong), ("slices", ctypes.c_ulonglong),
                ("busy_s", ctypes.c_double), ("span_s", ctypes.c_double), ("mean_inflight", ctypes.c_double),
                ("max_inflight", ctypes.c_ulonglong), ("hbm_used", ctypes.c_ulonglong),
                ("hbm_budget", ctypes.c_ulonglong), ("upload_s", ctypes.c_double), ("finish_s", ctypes.c_double),
                ("kernel_s", ctypes.c_double)]


# ----------------------------------------------------------------- loading

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads libmcfl.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"libmcfl.so not built ({path}); run cudamcfl_gb300.build.build()")
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    vp = ctypes.c_void_p
    sig = {
        "mcfl_last_error": (ctypes.c_char_p, []),
        "mcfl_create": (ctypes.c_int, [ctypes.c_int, P(vp)]),
        "mcfl_destroy": (None, [vp]),
        "mcfl_set_option": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_longlong]),
        "mcfl_get_option": (ctypes.c_longlong, [vp, ctypes.c_char_p]),
        "mcfl_set_stream": (ctypes.c_int, [vp, vp]),
        "mcfl_medium_create": (ctypes.c_int, [vp, P(MediumDesc), P(vp)]),
        "mcfl_medium_free": (None, [vp]),
        "mcfl_medium_bytes": (ctypes.c_size_t, [vp]),
        "mcfl_medium_from_simulation": (ctypes.c_int, [vp, P(Simulation), P(vp)]),
        "mcfl_medium_create_layered": (ctypes.c_int, [vp, P(LayeredDesc), P(vp)]),
        "mcfl_run": (ctypes.c_int, [vp, vp, P(RunDesc), P(RunOut)]),
        "mcfl_autotune": (ctypes.c_int, [vp, vp, P(RunDesc), ctypes.c_ulonglong, P(ctypes.c_int),
                                         P(ctypes.c_double)]),
        "mcfl_run_desc_from_simulation": (ctypes.c_int, [P(Simulation), ctypes.c_ulonglong, P(RunDesc)]),
        "mcfl_launch_count": (ctypes.c_ulonglong, [vp]),
        "mcfl_read_simulation_data": (ctypes.c_int, [ctypes.c_char_p, P(P(Simulation)), ctypes.c_int]),
        "mcfl_free_simulation_struct": (None, [P(Simulation), ctypes.c_int]),
        "mcfl_interpret_arg": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_char_p), P(ctypes.c_ulonglong),
                                              P(ctypes.c_int)]),
        "mcfl_init_RNG": (ctypes.c_int, [P(ctypes.c_ulonglong), P(ctypes.c_uint), ctypes.c_uint, ctypes.c_char_p,
                                         ctypes.c_ulonglong]),
        "mcfl_write_safeprimes": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint]),
        "mcfl_DoOneSimulation": (ctypes.c_ulonglong, [P(Simulation), ctypes.c_ulonglong, _f64p, _u64p, _u64p]),
        "mcfl_DoOneSimulationFl": (ctypes.c_ulonglong, [P(Simulation), ctypes.c_ulonglong, _u64p, _u64p]),
        "mcfl_Write_Simulation_Results": (ctypes.c_int, [P(Simulation), _u64p, _u64p, ctypes.c_double]),
        "mcfl_write_phd": (ctypes.c_int, [P(Simulation), _f64p]),
        "mcfl_write_time": (ctypes.c_int, [P(Simulation), _u64p]),
        "mcfl_write_fl_images": (ctypes.c_int, [P(Simulation), _f64p, _f64p]),
        "mcfl_run_mci": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_ulonglong]),
        "mcfl_batch_run": (ctypes.c_int, [vp, vp, P(RunDesc), ctypes.c_int, ctypes.c_int, P(RunOut),
                                          P(ctypes.c_float)]),
        "mcfl_batch_run_media": (ctypes.c_int, [vp, P(vp), P(RunDesc), ctypes.c_int, ctypes.c_int, P(RunOut),
                                                P(ctypes.c_float)]),
        "mcfl_run_plain": (ctypes.c_int, [vp, vp, P(RunDesc), ctypes.c_longlong, P(RunOut)]),
        "mcfl_server_create": (ctypes.c_int, [vp, P(ServerOpts), P(vp)]),
        "mcfl_server_submit": (ctypes.c_int, [vp, P(MediumDesc), P(RunDesc), P(ctypes.c_ulonglong)]),
        "mcfl_server_wait": (ctypes.c_int, [vp, ctypes.c_ulonglong, ctypes.c_int]),
        "mcfl_server_result": (ctypes.c_int, [vp, ctypes.c_ulonglong, P(RunOut), P(ctypes.c_double)]),
        "mcfl_server_metrics": (ctypes.c_int, [vp, P(ServerMetrics)]),
        "mcfl_server_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return (load().mcfl_last_error() or b"").decode()


def check(code: int) -> None:
    if code != OK:
        raise McflError(code, last_error())


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def f64ptr(a: np.ndarray):
    return a.ctypes.data_as(_f64p)


# ----------------------------------------------------------------- helpers

def bulk_from_mci_columns(n: float, mua: float, mus: float, flc: float = 0.0, absc_exi: float = 0.0,
                          absc_emi: float = 0.0, eY: float = 0.0, g: float = 0.9) -> Bulk:
    """One bulk descriptor from the .mci columns (n mua mus flc AbsCExi AbsCEmi
    eY g), derived as the reference's parser does (CUDAMCFLio.cu:557-568),
    in single precision."""
    f = np.float32
    n, mua, mus, flc, ax, am, eY, g = (f(v) for v in (n, mua, mus, flc, absc_exi, absc_emi, eY, g))
    mutr = f(np.finfo(np.float32).max) if mus == 0 else f(f(1.0) / f(mua + mus))
    with np.errstate(invalid="ignore", divide="ignore"):  # mus = flc = 0 gives 0/0 = NaN, as in the reference
        albedof = f(mus / f(f(flc * ax) + mus))
    return Bulk(mutr, f(mua + f(flc * ax)), g, n, flc, f(mua + f(flc * am)), eY, albedof, mus)


def outer_bulk(n: float = 1.0) -> Bulk:
    return Bulk(float(np.finfo(np.float32).max), 0.0, 1.0, n, 0.0, 0.0, 0.0, 0.0, 0.0)


def layers_from_mci_columns(n_up: float, slabs, n_down: float) -> list:
    """The layer table of a layered medium (bulk method 1) from the .mci
    columns of its slabs (n mua mus flc AbsCExi AbsCEmi eY g thickness),
    derived as the reference's parser does (CUDAMCFLio.cu:437-477), in single
    precision: n_slabs + 2 entries, the outer media carrying only n."""
    f = np.float32
    out = [Layer(0, 0, 0, 0, 0, f(n_up), 0, 0, 0, 0)]
    dtot = f(0.0)
    for n, mua, mus, flc, ax, am, eY, g, thick in slabs:
        n, mua, mus, flc, ax, am, eY, g, thick = (f(v) for v in (n, mua, mus, flc, ax, am, eY, g, thick))
        z_min = dtot
        dtot = f(dtot + thick)
        mutr = f(np.finfo(np.float32).max) if mus == 0 else f(f(1.0) / f(mua + mus))
        with np.errstate(invalid="ignore", divide="ignore"):
            albedof = f(mus / f(f(flc * ax) + mus))
        out.append(Layer(z_min, dtot, mutr, f(mua + f(flc * ax)), g, n, flc, f(mua + f(flc * am)), eY, albedof))
    out.append(Layer(0, 0, 0, 0, 0, f(n_down), 0, 0, 0, 0))
    return out


def inclusion_from_mci_columns(x, y, z, r, n, mua, mus, flc=0.0, absc_exi=0.0, absc_emi=0.0, eY=0.0,
                               g=0.9) -> "Inclusion":
    """The spherical inclusion of a layered medium from its .mci columns
    (x y z r n mua mus flc AbsCExi AbsCEmi eY g, CUDAMCFLio.cu:484-500)."""
    f = np.float32
    x, y, z, r, n, mua, mus, flc, ax, am, eY, g = (f(v) for v in (x, y, z, r, n, mua, mus, flc, absc_exi, absc_emi,
                                                                 eY, g))
    mutr = f(np.finfo(np.float32).max) if mus == 0 else f(f(1.0) / f(mua + mus))
    with np.errstate(invalid="ignore", divide="ignore"):
        albedof = f(mus / f(f(flc * ax) + mus))
    return Inclusion(x, y, z, r, mutr, f(mua + f(flc * ax)), g, n, flc, f(mua + f(flc * am)), eY, albedof)


@dataclass
class RunResult:
    Rd: np.ndarray
    Tt: np.ndarray
    R: np.ndarray | None
    T: np.ndarray | None
    fhd: np.ndarray | None
    phd: np.ndarray | None
    flR: np.ndarray | None
    flT: np.ndarray | None
    flR128: np.ndarray | None
    flT128: np.ndarray | None
    stats_exc: dict
    stats_fl: dict
    photons_fl: int
    fl_voxels: int
    energy_exc: tuple
    ms_exc: float
    ms_fl: float
    time_xyt: np.ndarray | None = None  # uint64 (bins, ny, nx) raw time-resolved tallies


class Medium:
    """A device-resident medium.  It is freed by free(), by garbage
    collection, or by closing its context, whichever comes first."""

    def __init__(self, ctx: "Context", handle: int, shape: tuple, keep: list):
        self.ctx = ctx
        self.handle = handle
        self.shape = shape  # (nz, ny, nx)
        self._keep = keep
        ctx._media.add(self)

    @property
    def nbytes(self) -> int:
        return int(load().mcfl_medium_bytes(self.handle))

    def free(self) -> None:
        if self.handle and self.ctx is not None and self.ctx.handle:
            load().mcfl_medium_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One GPU context of the engine."""

    def __init__(self, device: int = -1, math: int = MATH_EXACT, **options):
        import weakref
        L = load()
        h = ctypes.c_void_p()
        self.handle = None
        self._media = weakref.WeakSet()
        check(L.mcfl_create(device, ctypes.byref(h)))
        self.handle = h
        self.set_option("math", math)
        for k, v in options.items():
            self.set_option(k, v)

    def set_option(self, key: str, value: int) -> None:
        check(load().mcfl_set_option(self.handle, key.encode(), int(value)))

    def get_option(self, key: str) -> int:
        return int(load().mcfl_get_option(self.handle, key.encode()))

    def set_stream(self, stream_handle: int | None) -> None:
        check(load().mcfl_set_stream(self.handle, stream_handle))

    def autotune(self, medium: "Medium", rd: RunDesc, sample_photons: int = 2_000_000) -> tuple[int, float]:
        """Times every kernel variant (with and without the L2 window, with
        each form of the photon-hitting-density tally when `rd` tallies it) on
        a sample of `rd` and keeps the fastest; returns (variant, photons/s)."""
        v = ctypes.c_int(0)
        rate = ctypes.c_double(0.0)
        check(load().mcfl_autotune(self.handle, medium.handle, ctypes.byref(rd), int(sample_photons),
                                   ctypes.byref(v), ctypes.byref(rate)))
        return v.value, rate.value

    @property
    def launches(self) -> int:
        return int(load().mcfl_launch_count(self.handle))

    def close(self) -> None:
        if self.handle:
            for m in list(self._media):
                m.free()  # media go before their context (mcfl_medium_free needs it)
            load().mcfl_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def medium(self, labels: np.ndarray, bulks: list, *, voxel_cm=None, vox_per_cm=None, half_x=None, half_y=None,
               thickness=None, fluor_map: np.ndarray | None = None) -> Medium:
        """labels: uint8 array (nz, ny, nx), x fastest in memory; bulks: the
        n+2 Bulk entries (0 above, n+1 below).  The grid is centred on x=y=0
        and spans 0 <= z < thickness."""
        lab = np.ascontiguousarray(labels, dtype=np.uint8)
        nz, ny, nx = lab.shape
        if vox_per_cm is None:
            vc = np.asarray(voxel_cm, dtype=np.float64)
            vox_per_cm = tuple(float(np.float32(1.0 / v)) for v in vc)
            if half_x is None:
                half_x = float(np.float32(nx * vc[0] / 2))
                half_y = float(np.float32(ny * vc[1] / 2))
                thickness = float(np.float32(nz * vc[2]))
        d = MediumDesc()
        d.nx, d.ny, d.nz = nx, ny, nz
        d.half_x, d.half_y, d.thickness = half_x, half_y, thickness
        d.vox_per_cm[:] = list(vox_per_cm)
        d.labels = lab.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))
        fm = None
        if fluor_map is not None:
            fm = np.ascontiguousarray(fluor_map, dtype=np.float32)
            assert fm.shape == lab.shape
            d.fluor_map = fm.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        barr = (Bulk * len(bulks))(*bulks)
        d.n_bulks = len(bulks) - 2
        d.bulks = barr
        h = ctypes.c_void_p()
        check(load().mcfl_medium_create(self.handle, ctypes.byref(d), ctypes.byref(h)))
        return Medium(self, h, lab.shape, [])

    def medium_layered(self, layers: list, inclusion: "Inclusion", grid_size: int) -> Medium:
        """A layered medium with one spherical inclusion (bulk method 1):
        layers as layers_from_mci_columns returns them."""
        arr = (Layer * len(layers))(*layers)
        d = LayeredDesc(len(layers) - 2, ctypes.cast(arr, ctypes.POINTER(Layer)), inclusion, int(grid_size))
        h = ctypes.c_void_p()
        check(load().mcfl_medium_create_layered(self.handle, ctypes.byref(d), ctypes.byref(h)))
        esp = np.float32(layers[-2].z_max)
        g = np.float32(grid_size)
        n = int(np.float32(np.float32(4) * esp) * g)
        return Medium(self, h, (int(esp * g), n, n), [arr])

    def medium_from_simulation(self, sim: Simulation) -> Medium:
        h = ctypes.c_void_p()
        check(load().mcfl_medium_from_simulation(self.handle, ctypes.byref(sim), ctypes.byref(h)))
        return Medium(self, h, (sim.num_z, sim.num_y, sim.num_x), [])

    def run(self, medium: Medium, rd: RunDesc, *, images: bool = True, raw: bool = True, fluence: bool = True,
            emission128: bool = True) -> RunResult:
        """Runs one two-phase simulation and returns numpy copies."""
        det = rd.det
        xy = det.nx + det.nx * det.ny
        nz, ny, nx = medium.shape
        nv = nx * ny * nz
        em = rd.photons_per_voxel > 0
        fl_on = em or rd.fluence
        out = RunOut()
        keep = {}

        def alloc(name, n, dt, ptrf):
            a = np.zeros(n, dtype=dt)
            keep[name] = a
            setattr(out, name, ptrf(a))

        alloc("Rd", xy, np.uint64, u64ptr)
        alloc("Tt", xy, np.uint64, u64ptr)
        if images:
            alloc("R", xy, np.float64, f64ptr)
            alloc("T", xy, np.float64, f64ptr)
        if fl_on and fluence:
            if raw:
                alloc("fhd", nv, np.uint64, u64ptr)
            alloc("phd", nv, np.float64, f64ptr)
        if em:
            alloc("flR", xy, np.float64, f64ptr)
            alloc("flT", xy, np.float64, f64ptr)
            if emission128:
                alloc("flR128", 2 * xy, np.uint64, u64ptr)
                alloc("flT128", 2 * xy, np.uint64, u64ptr)
        td = rd.tdet
        if td.nx > 0:
            alloc("time_xyt", td.nx * td.ny * td.bins, np.uint64, u64ptr)
        rc = load().mcfl_run(self.handle, medium.handle, ctypes.byref(rd), ctypes.byref(out))
        check(rc)
        g = keep.get
        return RunResult(
            Rd=g("Rd"), Tt=g("Tt"), R=g("R"), T=g("T"), fhd=g("fhd"), phd=g("phd"), flR=g("flR"), flT=g("flT"),
            flR128=None if g("flR128") is None else g("flR128").reshape(xy, 2),
            flT128=None if g("flT128") is None else g("flT128").reshape(xy, 2),
            stats_exc=dict(zip(STAT_NAMES, list(out.stats_exc))), stats_fl=dict(zip(STAT_NAMES, list(out.stats_fl))),
            photons_fl=int(out.photons_fl), fl_voxels=int(out.fl_voxels), energy_exc=tuple(out.energy_exc),
            ms_exc=float(out.ms_exc), ms_fl=float(out.ms_fl),
            time_xyt=None if g("time_xyt") is None else g("time_xyt").reshape(td.bins, td.ny, td.nx))


def _medium_desc(labels, bulks, voxel_cm, fluor_map=None):
    """MediumDesc over numpy arrays (kept alive by the returned tuple)."""
    lab = np.ascontiguousarray(labels, dtype=np.uint8)
    nz, ny, nx = lab.shape
    vc = np.asarray(voxel_cm, dtype=np.float64)
    d = MediumDesc()
    d.nx, d.ny, d.nz = nx, ny, nz
    d.half_x = float(np.float32(nx * vc[0] / 2))
    d.half_y = float(np.float32(ny * vc[1] / 2))
    d.thickness = float(np.float32(nz * vc[2]))
    d.vox_per_cm[:] = [float(np.float32(1.0 / v)) for v in vc]
    d.labels = lab.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))
    fm = None
    if fluor_map is not None:
        fm = np.ascontiguousarray(fluor_map, dtype=np.float32)
        d.fluor_map = fm.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    barr = (Bulk * len(bulks))(*bulks)
    d.n_bulks = len(bulks) - 2
    d.bulks = barr
    return d, (lab, fm, barr)


def _alloc_out(xy, nv=0, images=True, fluence=False):
    out = RunOut()
    keep = {}
    for name, n, dt, pf in (("Rd", xy, np.uint64, u64ptr), ("Tt", xy, np.uint64, u64ptr)):
        a = np.zeros(n, dtype=dt)
        keep[name] = a
        setattr(out, name, pf(a))
    if images:
        for name in ("R", "T"):
            a = np.zeros(xy, dtype=np.float64)
            keep[name] = a
            setattr(out, name, f64ptr(a))
    if fluence:
        a = np.zeros(nv, dtype=np.uint64)
        keep["fhd"] = a
        out.fhd = u64ptr(a)
    return out, keep


def batch_run(ctx: "Context", medium, runs: list, schedule: int = SCHEDULE_BATCHED,
              images: bool = True):
    """Runs excitation-only simulations on one medium, or on a medium each
    when `medium` is a list (one per run).  Returns (list of dicts with Rd,
    Tt, R, T, stats, and time_xyt for runs with time-resolved detectors;
    GPU ms)."""
    n = len(runs)
    arr = (RunDesc * n)(*runs)
    outs = (RunOut * n)()
    keeps = []
    for i, r in enumerate(runs):
        xy = r.det.nx + r.det.nx * r.det.ny
        o, k = _alloc_out(xy, images=images)
        if r.tdet.nx:
            t = np.zeros(r.tdet.nx * r.tdet.ny * r.tdet.bins, dtype=np.uint64)
            o.time_xyt = u64ptr(t)
            k["time_xyt"] = t
        outs[i] = o
        keeps.append(k)
    ms = ctypes.c_float()
    if isinstance(medium, (list, tuple)):
        assert len(medium) == n
        handles = (ctypes.c_void_p * n)(*[m.handle for m in medium])
        check(load().mcfl_batch_run_media(ctx.handle, handles, arr, n, schedule, outs, ctypes.byref(ms)))
    else:
        check(load().mcfl_batch_run(ctx.handle, medium.handle, arr, n, schedule, outs, ctypes.byref(ms)))
    res = []
    for i in range(n):
        d = dict(keeps[i])
        d["stats"] = dict(zip(STAT_NAMES, list(outs[i].stats_exc)))
        res.append(d)
    return res, float(ms.value)


def run_plain(ctx: "Context", medium: "Medium", rd: RunDesc, max_voxels: int = 0):
    """Two-phase run with one emission launch per voxel."""
    xy = rd.det.nx + rd.det.nx * rd.det.ny
    out = RunOut()
    keep = {}
    for name, n in (("Rd", xy), ("Tt", xy), ("flR128", 2 * xy), ("flT128", 2 * xy)):
        a = np.zeros(n, dtype=np.uint64)
        keep[name] = a
        setattr(out, name, u64ptr(a))
    check(load().mcfl_run_plain(ctx.handle, medium.handle, ctypes.byref(rd), max_voxels, ctypes.byref(out)))
    keep["flR128"] = keep["flR128"].reshape(xy, 2)
    keep["flT128"] = keep["flT128"].reshape(xy, 2)
    keep.update(stats_exc=dict(zip(STAT_NAMES, list(out.stats_exc))),
                stats_fl=dict(zip(STAT_NAMES, list(out.stats_fl))), fl_voxels=int(out.fl_voxels),
                photons_fl=int(out.photons_fl), ms_exc=float(out.ms_exc), ms_fl=float(out.ms_fl))
    return keep


class Server:
    """Continuous-batching server over one context."""

    def __init__(self, ctx: "Context", hbm_budget_bytes: int = 0, max_jobs: int = 0, slice_passes: int = 0,
                 express_period: int = 0, express_ratio: int = 0, slice_us: int = 0):
        o = ServerOpts(hbm_budget_bytes, max_jobs, slice_passes, express_period, express_ratio, slice_us)
        h = ctypes.c_void_p()
        check(load().mcfl_server_create(ctx.handle, ctypes.byref(o), ctypes.byref(h)))
        self.handle = h
        self._keep = {}
        self._shape = {}

    def submit(self, labels, bulks, voxel_cm, rd: RunDesc, fluor_map=None) -> int:
        d, keep = _medium_desc(labels, bulks, voxel_cm, fluor_map)
        rid = ctypes.c_ulonglong()
        check(load().mcfl_server_submit(self.handle, ctypes.byref(d), ctypes.byref(rd), ctypes.byref(rid)))
        self._keep[rid.value] = (d, keep, rd)
        self._shape[rid.value] = (rd.det.nx + rd.det.nx * rd.det.ny, int(np.prod(np.shape(labels))),
                                  bool(rd.fluence), rd.tdet.nx * rd.tdet.ny * rd.tdet.bins if rd.tdet.nx else 0)
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1) -> int:
        return int(load().mcfl_server_wait(self.handle, rid, timeout_ms))

    def result(self, rid: int):
        xy, nv, fl, tsize = self._shape[rid]
        out, keep = _alloc_out(xy, nv, images=False, fluence=fl)
        if tsize:
            keep["time_xyt"] = np.zeros(tsize, dtype=np.uint64)
            out.time_xyt = u64ptr(keep["time_xyt"])
        lat = ctypes.c_double()
        check(load().mcfl_server_result(self.handle, rid, ctypes.byref(out), ctypes.byref(lat)))
        self._keep.pop(rid, None)
        keep["stats"] = dict(zip(STAT_NAMES, list(out.stats_exc)))
        keep["latency_ms"] = float(lat.value)
        return keep

    def metrics(self) -> dict:
        m = ServerMetrics()
        check(load().mcfl_server_metrics(self.handle, ctypes.byref(m)))
        return {k: getattr(m, k) for k, _ in ServerMetrics._fields_}

    def close(self) -> None:
        if self.handle:
            load().mcfl_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_desc(photons: int, *, source=(0.0, 0.0, 0.0), det: Detector, photons_per_voxel: int = 0, fluence: int = 0,
             seed_exc: int = 1, seed_fl: int = 2, start_weight: int = 0, kind: int = SOURCE_GAUSS_BEAM,
             width: float = 0.0, height: float = 0.0, launch_rng_reuse: int = 0, tdet: tuple | None = None,
             exact_stepping: int = 0) -> RunDesc:
    """tdet: time-resolved detectors (x0, y0, nx, ny, sep_x, sep_y, radius,
    face, bins, max_fs), or None.  exact_stepping: 1 for voxel-boundary
    stepping (mu_t spent voxel by voxel, Fresnel with each face's normal),
    0 for the reference's stepping."""
    r = RunDesc()
    r.photons = photons
    r.photons_per_voxel = photons_per_voxel
    r.fluence = fluence
    r.seed_exc = seed_exc
    r.seed_fl = seed_fl
    r.start_weight = start_weight
    r.source = Source(kind, *[float(v) for v in source], width, height)
    r.det = det
    r.launch_rng_reuse = launch_rng_reuse
    r.exact_stepping = exact_stepping
    if tdet:
        x0, y0, tnx, tny, sx, sy, rad, face, bins, tmax = tdet
        r.tdet = TimeDetectors(tnx, tny, x0, y0, sx, sy, rad, face, bins, tmax)
    return r


def read_simulation_data(path: str):
    """read_simulation_data: returns (array pointer, count); free with
    free_simulations."""
    L = load()
    p = ctypes.POINTER(Simulation)()
    n = L.mcfl_read_simulation_data(path.encode(), ctypes.byref(p), 0)
    if n <= 0:
        raise McflError(E_PARSE, last_error())
    return p, n


def free_simulations(p, n: int) -> None:
    load().mcfl_free_simulation_struct(p, n)
