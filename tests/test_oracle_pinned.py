"""Pins the CPU oracle to the reference.

The restatement in oracle/port.cpp, run with the reference's RNG streams and
schedule and C-library math, must reproduce the reference's own transport
(compiled for the host from its sources, oracle/_ref) bit for bit:
  - against golden fixtures made by that build (tests/golden/, runs anywhere);
  - live against the build itself where the reference checkout is present.
The product's parser, writers and init_RNG are checked against the
reference's own functions the same way.
"""
import ctypes
import os
import tempfile

import numpy as np
import pytest

from tests import cases

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
FIXTURES = {"tiny": dict(photons=40000, per_voxel=33000), "mismatch": dict(photons=36000, per_voxel=33000),
            "glass": dict(photons=36000, per_voxel=33000), "mismatch_timed": dict(photons=36000, per_voxel=33000),
            "glass_timed_exit": dict(photons=36000, per_voxel=33000), "layered": dict(photons=36000, per_voxel=33000),
            "layered_timed_exit": dict(photons=36000, per_voxel=33000)}
BUILDERS = {**cases.ALL, **cases.LAYERED}


def _same(a, b):
    assert a.shape == b.shape
    return np.array_equal(a, b)


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_port_reproduces_reference_golden(name, oracle, safeprimes_file, tmp_path):
    g = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    case = BUILDERS[name](**FIXTURES[name])
    # the fixture was made from the .mci this case writes
    mci = case.write_mci(str(tmp_path))
    assert open(mci).read() == str(g["mci"])
    s1, s2 = (int(v) for v in g["seeds"])
    r = oracle.run_refstream(case.oracle_sim(), safeprimes_file, s1, s2, libm=True)
    assert r.photons_exc == int(g["photons_exc"]) and r.photons_fl == int(g["photons_fl"])
    assert r.fl_voxels == int(g["fl_voxels"])
    for k in ("Rd", "Tt", "fhd", "flR", "flT"):
        assert _same(getattr(r, k), g[k]), k
    if "time_xyt" in g:
        assert g["time_xyt"].sum() > 0
        assert _same(r.time_xyt, g["time_xyt"])
    else:
        assert r.time_xyt is None


@pytest.mark.parametrize("name", ["tiny", "glass", "glass_timed_exit", "layered_timed_exit"])
def test_port_reproduces_reference_build_live(name, oracle, ref_oracle, safeprimes_file, tmp_path):
    case = BUILDERS[name](photons=34000, per_voxel=32800)
    mci = case.write_mci(str(tmp_path))
    sim = ref_oracle.parse_mci(mci)
    a = ref_oracle.run_mci(mci, safeprimes_file, 4242, 99)
    b = oracle.run_refstream(sim, safeprimes_file, 4242, 99, libm=True)
    for k in ("Rd", "Tt", "fhd", "flR", "flT"):
        assert _same(getattr(a, k), getattr(b, k)), k
    if case.temporal:
        assert _same(a.time_xyt, b.time_xyt)


def _sim_fields(s):
    out = {k: getattr(s, k) for k, _ in s._fields_ if k not in ("bulks", "bulk_info", "vox_per_cm", "fluor_map")}
    # mus is not a BulkStruct field (the reference's parser keeps only mutr):
    # only voxel-boundary stepping reads it
    out["bulks"] = [tuple(np.float32(getattr(s.bulks[i], f)).tobytes() for f, _ in s.bulks[i]._fields_ if f != "mus")
                    for i in range(s.n_bulks + 2)]
    return out


@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_case_builder_matches_reference_parser(name, ref_oracle, tmp_path):
    """tests/cases.py builds the oracle input with the same floats the
    reference's parser derives from the .mci text."""
    case = cases.ALL[name]()
    mci = case.write_mci(str(tmp_path))
    parsed = ref_oracle.parse_mci(mci)
    built = case.oracle_sim()
    a, b = _sim_fields(parsed), _sim_fields(built)
    for k in ("number_of_photons", "number_of_photons_per_voxel", "n_bulks", "start_weight", "grid_size", "esp",
              "xi", "yi", "zi", "dir", "fhd_activated", "do_fl_sim", "det_dx", "det_dy", "det_nx", "det_ny",
              "det_x0", "det_y0", "bulks") + (TEMPORAL if case.temporal else ("do_temp_sim",)):
        assert a[k] == b[k], k
    n = int(np.prod(case.labels.shape))
    pa = np.ctypeslib.as_array(parsed.bulk_info, shape=(n,))
    assert np.array_equal(pa, case.labels.ravel().astype(np.int16))


TEMPORAL = ("do_temp_sim", "tdet_x0", "tdet_y0", "tdet_nx", "tdet_ny", "tdet_sep_x", "tdet_sep_y", "tdet_r",
            "tdet_face", "tdet_bins", "tdet_max")


def _floats(st):
    return [np.float32(getattr(st, f)).tobytes() for f, _ in st._fields_]


@pytest.mark.parametrize("name", sorted(cases.LAYERED))
def test_layered_case_builder_matches_reference_parser(name, ref_oracle, tmp_path):
    """Layered media: the layer table, the inclusion and the temporal
    detectors built in Python equal what the reference's parser reads from
    the .mci text (outer media: n only, the parser leaves the rest unset)."""
    case = cases.LAYERED[name]()
    mci = case.write_mci(str(tmp_path))
    parsed = ref_oracle.parse_mci(mci)
    built = case.oracle_sim()
    for k in ("number_of_photons", "start_weight", "grid_size", "esp", "xi", "yi", "zi", "dir", "fhd_activated",
              "do_fl_sim", "det_dx", "det_dy", "det_nx", "det_ny", "det_x0", "det_y0", "n_layers") + \
            (TEMPORAL if case.temporal else ("do_temp_sim",)):
        assert getattr(parsed, k) == getattr(built, k), k
    n = parsed.n_layers
    for i in range(1, n + 1):
        assert _floats(parsed.layers[i]) == _floats(built.layers[i]), i
    assert parsed.layers[0].n == built.layers[0].n and parsed.layers[n + 1].n == built.layers[n + 1].n
    assert _floats(parsed.inclusion) == _floats(built.inclusion)


def _product_parse(lib, mci):
    import cudamcfl_gb300 as mc
    cwd = os.getcwd()
    os.chdir(os.path.dirname(mci))
    try:
        p, n = mc.read_simulation_data(os.path.basename(mci))
    finally:
        os.chdir(cwd)
    return p, n


def _ref_sample(path):
    from oracle import pyoracle
    ref_dir = pyoracle.reference_dir()
    p = os.path.join(ref_dir, path) if ref_dir else ""
    if not os.path.exists(p):
        pytest.skip("reference checkout not present")
    return p


@pytest.mark.parametrize("src", ["case:tiny", "case:mismatch", "case:glass", "case:mismatch_timed", "lay:layered",
                                 "lay:layered_timed_exit", "ref:sample2.mci"])
def test_product_parser_matches_reference_parser(src, mcfl_lib, ref_oracle, tmp_path):
    import cudamcfl_gb300 as mc
    case = None
    if src.startswith("case:"):
        case = cases.ALL[src[5:]]()
        mci = case.write_mci(str(tmp_path))
    elif src.startswith("lay:"):
        mci = cases.LAYERED[src[4:]]().write_mci(str(tmp_path))
    else:
        mci = _ref_sample(src[4:])
    ref = ref_oracle.parse_mci(mci)
    p, n = _product_parse(mcfl_lib, mci)
    try:
        s = p[0]
        for k in ("number_of_photons", "number_of_photons_per_voxel", "n_bulks", "start_weight", "grid_size",
                  "do_fl_sim", "fhd_activated", "bulk_method"):
            assert getattr(s, k) == getattr(ref, k), k
        for k in ("esp", "xi", "yi", "zi", "dir"):
            assert np.float32(getattr(s, k)).tobytes() == np.float32(getattr(ref, k)).tobytes(), k
        for k, rk in (("dx", "det_dx"), ("dy", "det_dy"), ("x0", "det_x0"), ("y0", "det_y0")):
            assert np.float32(getattr(s.det, k)).tobytes() == np.float32(getattr(ref, rk)).tobytes(), k
        assert (s.det.nx, s.det.ny) == (ref.det_nx, ref.det_ny)
        if ref.do_temp_sim:
            for k, rk in (("x0_temp_det", "tdet_x0"), ("y0_temp_det", "tdet_y0"), ("x_temp_sepdets", "tdet_sep_x"),
                          ("y_temp_sepdets", "tdet_sep_y"), ("temp_det_r", "tdet_r")):
                assert np.float32(getattr(s.det, k)).tobytes() == np.float32(getattr(ref, rk)).tobytes(), k
            assert (s.det.x_temp_numdets, s.det.y_temp_numdets, s.det.temp_rort, s.det.temp_bins, s.det.max_temp) == \
                (ref.tdet_nx, ref.tdet_ny, ref.tdet_face, ref.tdet_bins, ref.tdet_max)
        if s.bulk_method == 1:
            assert s.n_layers == ref.n_layers
            for i in range(1, s.n_layers + 1):
                for f, _ in mc.Layer._fields_:
                    assert np.float32(getattr(s.layers[i], f)).tobytes() == \
                        np.float32(getattr(ref.layers[i], f)).tobytes(), (i, f)
            for i in (0, s.n_layers + 1):
                assert np.float32(s.layers[i].n) == np.float32(ref.layers[i].n)
            for f, _ in mc.Inclusion._fields_:
                assert np.float32(getattr(s.inclusion, f)).tobytes() == \
                    np.float32(getattr(ref.inclusion, f)).tobytes(), f
            return
        for i in range(s.n_bulks + 2):
            for f, _ in mc.Bulk._fields_:
                if f == "mus":  # not a BulkStruct field: the .mci column itself, 0 outside the slab
                    if i in (0, s.n_bulks + 1):
                        assert s.bulks[i].mus == 0.0, i
                    elif case is not None:
                        assert np.float32(s.bulks[i].mus) == np.float32(case.columns[i - 1][2]), i
                    continue
                assert np.float32(getattr(s.bulks[i], f)).tobytes() == \
                    np.float32(getattr(ref.bulks[i], f)).tobytes(), (i, f)
        nv = s.num_x * s.num_y * s.num_z
        a = np.ctypeslib.as_array(s.bulk_info, shape=(nv,)).astype(np.int16)
        b = np.ctypeslib.as_array(ref.bulk_info, shape=(nv,))
        assert np.array_equal(a, b)
    finally:
        mc.free_simulations(p, n)


def test_product_init_rng_matches_reference(mcfl_lib, ref_oracle, safeprimes_file):
    import cudamcfl_gb300 as mc
    n = 32768
    xa, aa = (ctypes.c_ulonglong * n)(), (ctypes.c_uint * n)()
    xb, ab = (ctypes.c_ulonglong * n)(), (ctypes.c_uint * n)()
    ref_oracle.lib.ref_init_rng.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint),
                                            ctypes.c_uint, ctypes.c_char_p, ctypes.c_ulonglong]
    for seed in (1, 12345, 2**40 + 7):
        assert mcfl_lib.mcfl_init_RNG(xa, aa, n, safeprimes_file.encode(), seed) == 0
        assert ref_oracle.lib.ref_init_rng(xb, ab, n, safeprimes_file.encode(), seed) == 0
        assert list(xa) == list(xb) and list(aa) == list(ab)
    assert mcfl_lib.mcfl_init_RNG(xa, aa, n, safeprimes_file.encode(), 0) == 1  # invalid seed, as the reference


def _strip_param(text):
    return [ln for ln in text.splitlines() if not ln.startswith("Compilation date") and "User time" not in ln]


def test_writers_match_reference(mcfl_lib, ref_oracle, safeprimes_file, tmp_path):
    """The product's writers format the reference's own tallies exactly as the
    reference's writers do (all six output files)."""
    import cudamcfl_gb300 as mc
    case = cases.tiny(photons=34000, per_voxel=32800)
    d1, d2 = tmp_path / "ref", tmp_path / "prod"
    d1.mkdir()
    d2.mkdir()
    mci1 = case.write_mci(str(d1))
    case.write_mci(str(d2))
    r = ref_oracle.run_mci(mci1, safeprimes_file, 5, 6, write_files=True)
    p, n = _product_parse(mcfl_lib, str(d2 / "tiny.mci"))
    cwd = os.getcwd()
    os.chdir(d2)
    try:
        sim = p[0]
        Rd, Tt = r.Rd.copy(), r.Tt.copy()
        assert mcfl_lib.mcfl_Write_Simulation_Results(p, mc.u64ptr(Rd), mc.u64ptr(Tt), 0.0) == 0
        phd = (r.fhd.astype(np.float64) / float(0xFFFFFFFF * r.photons_exc)).copy()
        assert mcfl_lib.mcfl_write_phd(p, mc.f64ptr(phd)) == 0
        flR, flT = r.flR.copy(), r.flT.copy()
        assert mcfl_lib.mcfl_write_fl_images(p, mc.f64ptr(flR), mc.f64ptr(flT)) == 0
    finally:
        os.chdir(cwd)
        mc.free_simulations(p, n)
    for suffix in ("_Refl.dat", "_Trans.dat", "_PHD-Ascii.dat", "_FlR.dat", "_FlT.dat"):
        a = open(d1 / f"tiny-out{suffix}").read()
        b = open(d2 / f"tiny-out{suffix}").read()
        assert a == b, suffix
    a = _strip_param(open(d1 / "tiny-out_param.dat").read())
    b = _strip_param(open(d2 / "tiny-out_param.dat").read())
    assert a == b


def test_time_writer_matches_reference(mcfl_lib, ref_oracle, safeprimes_file, tmp_path):
    """<out>_time.dat of the product's writer equals the reference's for the
    reference's own time-resolved tallies."""
    import cudamcfl_gb300 as mc
    case = cases.mismatch_timed(photons=34000, per_voxel=32800)
    case.do_fl = 0
    d1, d2 = tmp_path / "ref", tmp_path / "prod"
    d1.mkdir()
    d2.mkdir()
    mci1 = case.write_mci(str(d1))
    case.write_mci(str(d2))
    r = ref_oracle.run_mci(mci1, safeprimes_file, 5, 6, write_files=True)
    assert r.time_xyt is not None and r.time_xyt.sum() > 0
    p, n = _product_parse(mcfl_lib, str(d2 / f"{case.name}.mci"))
    cwd = os.getcwd()
    os.chdir(d2)
    try:
        t = r.time_xyt.copy()
        assert mcfl_lib.mcfl_write_time(p, mc.u64ptr(t)) == 0
    finally:
        os.chdir(cwd)
        mc.free_simulations(p, n)
    a = open(d1 / f"{case.name}-out_time.dat").read()
    b = open(d2 / f"{case.name}-out_time.dat").read()
    assert a == b
