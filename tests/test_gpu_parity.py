"""CUDA engine against the CPU oracle.

The exact-math kernel and the oracle's photon-indexed restatement perform the
same IEEE operations on the same random streams, so every tally must be
identical bit for bit: R/T images, photon hitting density, the 128-bit
emission accumulators and the per-job weight accounting.  The fast-math
kernel (hardware SFU intrinsics, the reference's own GPU numerics) is held to
the statistical gate instead (tests/test_gpu_statistics.py).
"""
import numpy as np
import pytest

import cudamcfl_gb300 as mc
from tests import cases

STAT_ORDER = ("absorbed", "exit_top", "exit_bottom", "roulette_loss", "roulette_gain", "zero_drop_loss")


def _compare(res, ref, emission=True):
    assert np.array_equal(res.Rd, ref.Rd)
    assert np.array_equal(res.Tt, ref.Tt)
    assert np.array_equal(res.fhd, ref.fhd)
    assert tuple(res.stats_exc[k] for k in STAT_ORDER) == tuple(ref.balance)
    assert res.stats_exc["done"] == ref.photons_exc
    assert res.stats_exc["steps"] == ref.steps_exc
    assert res.stats_exc["capped"] == 0
    if ref.time_xyt is not None:
        assert res.time_xyt is not None and res.time_xyt.ravel().sum() > 0
        assert np.array_equal(res.time_xyt.ravel(), ref.time_xyt)
    else:
        assert res.time_xyt is None
    if emission:
        assert res.fl_voxels == ref.fl_voxels
        assert res.photons_fl == ref.photons_fl
        assert res.stats_fl["steps"] == ref.steps_fl
        assert np.array_equal(res.flR128, ref.flR128)
        assert np.array_equal(res.flT128, ref.flT128)
        assert np.array_equal(res.flR, ref.flR)
        assert np.array_equal(res.flT, ref.flT)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.ALL))
def test_exact_kernel_bit_identical_to_oracle(name, gpu_ctx, oracle, table32768):
    case = cases.ALL[name](photons=20000, per_voxel=500)
    ref = oracle.run_photon(case.oracle_sim(), table32768, 11, 22, libm=False)
    med = case.engine_medium(gpu_ctx)
    res = gpu_ctx.run(med, case.run_desc(11, 22))
    _compare(res, ref)
    assert ref.fl_voxels > 0


@pytest.mark.gpu
def test_exact_kernel_launch_shape_does_not_change_tallies(gpu_ctx, oracle, table32768):
    """Photon-indexed streams: block size and grid size change which thread
    carries which photon, never the tallies."""
    case = cases.mismatch(photons=30000, per_voxel=300)
    ref = oracle.run_photon(case.oracle_sim(), table32768, 5, 6, libm=False)
    med = case.engine_medium(gpu_ctx)
    try:
        for block, bps in ((64, 1), (128, 2), (256, 0)):
            gpu_ctx.set_option("block", block)
            gpu_ctx.set_option("blocks_per_sm", bps)
            _compare(gpu_ctx.run(med, case.run_desc(5, 6)), ref)
        gpu_ctx.set_option("block", 256)
        gpu_ctx.set_option("blocks_per_sm", 0)
        # every occupancy variant, with and without the persisting-L2 window,
        # with each form of the photon-hitting-density tally (one add per
        # pass, register sums, warp sums) and either form of the pass
        # (SIMT-arranged, per-test branching)
        for variant, bound in ((0, 256), (1, 256), (2, 128)):
            for l2 in (0, 1):
                for agg, form in ((0, 0), (0, 1), (1, 0), (2, 0)):
                    gpu_ctx.set_option("variant", variant)
                    gpu_ctx.set_option("l2_window", l2)
                    gpu_ctx.set_option("phd_agg", agg)
                    gpu_ctx.set_option("pass_form", form)
                    assert gpu_ctx.get_option("launch_block") == bound
                    _compare(gpu_ctx.run(med, case.run_desc(5, 6)), ref)
        # free lanes waiting for others before they start new photons
        gpu_ctx.set_option("l2_window", 0)
        gpu_ctx.set_option("phd_agg", 0)
        gpu_ctx.set_option("pass_form", 0)
        for relaunch in (2, 7, 32):
            gpu_ctx.set_option("relaunch", relaunch)
            assert gpu_ctx.get_option("relaunch") == relaunch
            _compare(gpu_ctx.run(med, case.run_desc(5, 6)), ref)
    finally:
        gpu_ctx.set_option("relaunch", 1)
        gpu_ctx.set_option("block", 256)
        gpu_ctx.set_option("blocks_per_sm", 0)
        gpu_ctx.set_option("variant", 0)
        gpu_ctx.set_option("l2_window", 0)
        gpu_ctx.set_option("phd_agg", 0)
        gpu_ctx.set_option("pass_form", 0)


@pytest.mark.gpu
def test_autotune_keeps_a_variant_and_tallies(gpu_ctx, oracle, table32768):
    """The autotuner leaves one of the variants in the context; the run after
    it still equals the oracle bit for bit."""
    case = cases.sphere(photons=20000, per_voxel=200)
    ref = oracle.run_photon(case.oracle_sim(), table32768, 8, 9, libm=False)
    med = case.engine_medium(gpu_ctx)
    try:
        variant, rate = gpu_ctx.autotune(med, case.run_desc(8, 9), sample_photons=20000)
        assert variant in (0, 1, 2) and rate > 0
        assert gpu_ctx.get_option("variant") == variant
        assert gpu_ctx.get_option("phd_agg") in (0, 1, 2)
        assert gpu_ctx.get_option("pass_form") in (0, 1)
        assert gpu_ctx.get_option("relaunch") in (1, 2)
        _compare(gpu_ctx.run(med, case.run_desc(8, 9)), ref)
    finally:
        gpu_ctx.set_option("relaunch", 1)
        gpu_ctx.set_option("variant", 0)
        gpu_ctx.set_option("l2_window", 0)
        gpu_ctx.set_option("phd_agg", 0)
        gpu_ctx.set_option("pass_form", 0)


@pytest.mark.gpu
def test_excitation_only_and_no_fluence(gpu_ctx, oracle, table32768):
    case = cases.tiny(photons=25000, per_voxel=0)
    case.do_fl = 0
    ref = oracle.run_photon(case.oracle_sim(), table32768, 99, 100, libm=False)
    med = case.engine_medium(gpu_ctx)
    res = gpu_ctx.run(med, case.run_desc(99, 100))
    assert np.array_equal(res.Rd, ref.Rd) and np.array_equal(res.Tt, ref.Tt)
    assert res.fhd is None and res.flR is None


def _synthetic_sim(m, photons, per_voxel):
    from oracle import pyoracle
    nz, ny, nx = m.labels.shape
    vc = m.voxel_cm
    return pyoracle.sim_from_arrays(
        m.labels, m.bulks, half_x=float(np.float32(nx * vc[0] / 2)), half_y=float(np.float32(ny * vc[1] / 2)),
        thickness=float(np.float32(nz * vc[2])), vox_per_cm=[float(np.float32(1 / v)) for v in vc],
        photons=photons, per_voxel=per_voxel,
        det=(m.det.dx, m.det.dy, m.det.nx, m.det.ny, m.det.x0, m.det.y0), fluor_map=m.fluor_map)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", ["config1", "config2"])
def test_benchmark_media_bit_identical_to_oracle(cfg, gpu_ctx, oracle, table32768):
    """General geometry (anisotropic voxels, lateral extent 2 x thickness),
    8 labels, the fp32 fluorophore map: the workloads the benchmark runs."""
    from cudamcfl_gb300 import media
    m = getattr(media, cfg)()
    photons, per_voxel = (20000, 40) if cfg == "config1" else (6000, 2)
    ref = oracle.run_photon(_synthetic_sim(m, photons, per_voxel), table32768, 21, 22, libm=False)
    med = gpu_ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
    rd = mc.run_desc(photons, det=m.det, photons_per_voxel=per_voxel, fluence=1, seed_exc=21, seed_fl=22)
    res = gpu_ctx.run(med, rd)
    med.free()
    _compare(res, ref)


@pytest.mark.gpu
def test_launch_rng_reuse_bit_identical_to_oracle(gpu_ctx, oracle, table32768):
    case = cases.tiny(photons=40000, per_voxel=33000)
    sim = case.oracle_sim()
    sim.launch_rng_reuse = 1
    ref = oracle.run_photon(sim, table32768, 8, 9, libm=False)
    med = case.engine_medium(gpu_ctx)
    rd = case.run_desc(8, 9)
    rd.launch_rng_reuse = 1
    _compare(gpu_ctx.run(med, rd), ref)


@pytest.mark.gpu
def test_weight_is_conserved_exactly(gpu_ctx):
    """absorbed + left at both faces + roulette losses - roulette gains =
    photons x start weight, in integers (no photon wraps its weight here)."""
    from cudamcfl_gb300 import media
    m = media.config2()
    med = gpu_ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
    for kind in (mc.SOURCE_GAUSS_BEAM, mc.SOURCE_WIDEFIELD):
        rd = mc.run_desc(200_000, det=m.det, seed_exc=3, kind=kind, width=3.0, height=2.0)
        r = gpu_ctx.run(med, rd)
        s = r.stats_exc
        w0 = int(np.float64(0xFFFFFFFF) * (1 - ((1.0 - np.float64(np.float32(1.4))) /
                                               (1.0 + np.float64(np.float32(1.4)))) ** 2))
        lhs = s["absorbed"] + s["exit_top"] + s["exit_bottom"] + s["roulette_loss"] + s["zero_drop_loss"] - \
            s["roulette_gain"]
        assert lhs % 2**64 == (200_000 * w0) % 2**64
        assert abs(r.energy_exc[3]) < 1e-12
        assert s["done"] == 200_000 and s["capped"] == 0
    med.free()


@pytest.mark.gpu
def test_reference_host_routines_on_the_engine(mcfl_lib, oracle, table32768, tmp_path):
    """mcfl_DoOneSimulation / mcfl_DoOneSimulationFl / mcfl_run_mci: the
    drop-ins of DoOneSimulation, DoOneSimulationFl and cuda_fl's main."""
    import ctypes
    import os
    case = cases.tiny(photons=40000, per_voxel=33000)
    mci = case.write_mci(str(tmp_path))
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        p, n = mc.read_simulation_data("tiny.mci")
        sim = p[0]
        xy = sim.det.nx + sim.det.nx * sim.det.ny
        nv = sim.num_x * sim.num_y * sim.num_z
        Rd, Tt, fx = np.zeros(xy, np.uint64), np.zeros(xy, np.uint64), np.zeros(nv)
        got = mcfl_lib.mcfl_DoOneSimulation(p, 77, mc.f64ptr(fx), mc.u64ptr(Rd), mc.u64ptr(Tt))
        assert got == 40000 and Rd.sum() > 0 and fx.sum() > 0
        o = case.oracle_sim()
        o.do_fl_sim = 0
        # the .mci path turns the reference's launch-number reuse on
        o.launch_rng_reuse = 1
        ref = oracle.run_photon(o, table32768, 77, 78, libm=False)
        assert np.array_equal(Rd, ref.Rd) and np.array_equal(Tt, ref.Tt)
        # one emission run from the voxel at the source corner, emission absorption as the caller sets it
        for i in range(sim.n_bulks + 2):
            sim.bulks[i].mua = sim.bulks[i].muaf
        sim.xi, sim.yi, sim.zi = -0.25, -0.25, 0.0
        sim.number_of_photons = 33000
        R2, T2 = np.zeros(xy, np.uint64), np.zeros(xy, np.uint64)
        got = mcfl_lib.mcfl_DoOneSimulationFl(p, 5, mc.u64ptr(R2), mc.u64ptr(T2))
        assert got == 33000 and R2.sum() > 0
        mc.free_simulations(p, n)
        assert mcfl_lib.mcfl_run_mci(b"tiny.mci", ctypes.c_ulonglong(12345)) == 0
        for suffix in ("_param.dat", "_Refl.dat", "_Trans.dat", "_PHD-Ascii.dat", "_FlR.dat", "_FlT.dat"):
            assert os.path.getsize(f"tiny-out{suffix}") > 0
        img = np.loadtxt("tiny-out_FlR.dat")
        assert img.shape == (20, 20) and img.sum() > 0
    finally:
        os.chdir(cwd)


@pytest.mark.gpu
def test_bad_inputs_fail_with_status(gpu_ctx):
    case = cases.tiny()
    med = case.engine_medium(gpu_ctx)
    rd = case.run_desc(1, 2)
    rd.photons = 0
    with pytest.raises(mc.McflError) as e:
        gpu_ctx.run(med, rd)
    assert e.value.code == mc.E_ARG
    rd = case.run_desc(1, 2)
    rd.det.nx = 0
    with pytest.raises(mc.McflError):
        gpu_ctx.run(med, rd)
    lab = case.labels.copy()
    lab[0, 0, 0] = 9  # beyond n_bulks + 1
    with pytest.raises(mc.McflError) as e:
        gpu_ctx.medium(lab, case.bulks(), vox_per_cm=(4.0, 4.0, 4.0), half_x=1.0, half_y=1.0, thickness=0.5)
    assert e.value.code == mc.E_ARG
    for bad in (0, 33):
        with pytest.raises(mc.McflError) as e:
            gpu_ctx.set_option("relaunch", bad)
        assert e.value.code == mc.E_ARG
    gpu_ctx.set_option("step_cap", 50)  # photons live for hundreds of passes: the cap must report
    try:
        with pytest.raises(mc.McflError) as e:
            gpu_ctx.run(med, case.run_desc(1, 2, photons=2000))
        assert e.value.code == mc.E_CAPPED
    finally:
        gpu_ctx.set_option("step_cap", 1 << 24)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.LAYERED))
def test_layered_exact_kernel_bit_identical_to_oracle(name, gpu_ctx, oracle, table32768):
    """Layered media (the reference's bulk method 1): R/T images, photon
    hitting density, weight accounting and time-resolved tallies bit for bit."""
    case = cases.LAYERED[name](photons=30000)
    ref = oracle.run_photon(case.oracle_sim(), table32768, 13, 14, libm=False)
    med = case.engine_medium(gpu_ctx)
    res = gpu_ctx.run(med, case.run_desc(13, 14))
    med.free()
    assert res.fhd.size == ref.fhd.size and ref.Rd.sum() > 0
    _compare(res, ref, emission=False)


@pytest.mark.gpu
def test_run_mci_on_a_layered_medium(mcfl_lib, oracle, table32768, tmp_path):
    """A bulk-method-1 .mci through mcfl_run_mci: the reference's files, the
    excitation tallies equal to the oracle's (same photon streams, the .mci
    path's launch-number reuse), emission images of zeros as the reference
    writes them for layered media."""
    import ctypes
    import os
    case = cases.layered(photons=40000)
    case.do_fl = 1
    mci = case.write_mci(str(tmp_path))
    o = case.oracle_sim()
    o.launch_rng_reuse = 1
    ref = oracle.run_photon(o, table32768, 4321, 4322, libm=False)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        assert mcfl_lib.mcfl_run_mci(os.path.basename(mci).encode(), ctypes.c_ulonglong(4321)) == 0
        for suffix in ("_param.dat", "_Refl.dat", "_Trans.dat", "_PHD-Ascii.dat", "_FlR.dat", "_FlT.dat"):
            assert os.path.getsize(f"layered-out{suffix}") > 0
        assert not np.loadtxt("layered-out_FlR.dat").any()
        refl = np.loadtxt("layered-out_Refl.dat")
        scale = float(0xFFFFFFFF) * 40000 * np.float32(0.05) * np.float32(0.05)
        expect = ref.Rd[:40 * 40].reshape(40, 40).astype(np.float64) / scale
        assert np.allclose(refl, expect, rtol=1e-6, atol=0)
    finally:
        os.chdir(cwd)


@pytest.mark.gpu
def test_run_mci_runs_every_simulation_of_a_file(mcfl_lib, tmp_path):
    """A two-run .mci (voxelized, then layered): run i is seeded from
    seed + 2i and writes its own files, identical to running it alone."""
    import ctypes
    import os
    a = cases.tiny(photons=40000, per_voxel=33000)
    a.do_fl = 0
    b = cases.layered(photons=40000)
    b.do_fl = 0
    la = open(a.write_mci(str(tmp_path))).read().splitlines()
    lb = open(b.write_mci(str(tmp_path))).read().splitlines()
    (tmp_path / "multi.mci").write_text("\n".join(["# two runs", "1.0 # file version", "2 # runs"] + la[3:] +
                                                  lb[3:]) + "\n")
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        assert mcfl_lib.mcfl_run_mci(b"multi.mci", ctypes.c_ulonglong(9)) == 0
        both = {f: open(f).read() for f in ("tiny-out_Refl.dat", "tiny-out_Trans.dat", "layered-out_Refl.dat",
                                            "layered-out_Trans.dat")}
        assert mcfl_lib.mcfl_run_mci(b"tiny.mci", ctypes.c_ulonglong(9)) == 0
        assert mcfl_lib.mcfl_run_mci(b"layered.mci", ctypes.c_ulonglong(11)) == 0
        for f, text in both.items():
            assert open(f).read() == text, f
    finally:
        os.chdir(cwd)


@pytest.mark.gpu
@pytest.mark.parametrize("photons,per_voxel", [(1, 1), (31, 1), (33, 2), (1000, 3)])
def test_ragged_photon_counts_bit_identical(photons, per_voxel, gpu_ctx, oracle, table32768):
    """Budgets far below one photon per thread and not a multiple of a warp:
    one photon, a part of a warp, a warp and one."""
    case = cases.mismatch(photons=photons, per_voxel=per_voxel)
    ref = oracle.run_photon(case.oracle_sim(), table32768, 3, 4, libm=False)
    med = case.engine_medium(gpu_ctx)
    res = gpu_ctx.run(med, case.run_desc(3, 4))
    med.free()
    _compare(res, ref)
    assert res.stats_exc["done"] == photons


@pytest.mark.gpu
def test_hundred_labels_bit_identical(gpu_ctx, oracle, table32768):
    """100 bulk descriptors (the oracle's maximum; the engine's shared label
    table holds 256) scattered over the grid."""
    rng = np.random.default_rng(7)
    nz, ny, nx = 20, 40, 40
    lab = rng.integers(1, 101, size=(nz, ny, nx)).astype(np.uint8)
    bulks = [mc.outer_bulk(1.0)]
    for i in range(100):
        bulks.append(mc.bulk_from_mci_columns(1.3 + 0.002 * i, rng.uniform(0.05, 1.0), rng.uniform(20, 120),
                                              1.0 if i % 3 == 0 else 0.0, 0.05, 0.02, 0.1, rng.uniform(0.6, 0.95)))
    bulks.append(mc.outer_bulk(1.0))
    det = mc.Detector(0.0, 0.0, 0.05, 0.05, 32, 32)
    from oracle import pyoracle
    sim = pyoracle.sim_from_arrays(lab, bulks, half_x=1.0, half_y=1.0, thickness=0.5, vox_per_cm=[20.0, 20.0, 40.0],
                                   photons=20000, per_voxel=5, det=(0.05, 0.05, 32, 32, 0.0, 0.0))
    ref = oracle.run_photon(sim, table32768, 17, 18, libm=False)
    med = gpu_ctx.medium(lab, bulks, vox_per_cm=(20.0, 20.0, 40.0), half_x=1.0, half_y=1.0, thickness=0.5)
    res = gpu_ctx.run(med, mc.run_desc(20000, det=det, photons_per_voxel=5, fluence=1, seed_exc=17, seed_fl=18,
                                       start_weight=sim.start_weight))
    med.free()
    _compare(res, ref)
    assert ref.fl_voxels > 0


@pytest.mark.gpu
def test_large_grid_bit_identical(gpu_ctx, oracle, table32768):
    """A 1024 x 1024 x 64 grid (67M voxels): the index arithmetic at the
    sizes of the large precision-study medium."""
    nz, ny, nx = 64, 1024, 1024
    lab = np.ones((nz, ny, nx), dtype=np.uint8)
    lab[8:40, 400:600, 450:650] = 2
    bulks = [mc.outer_bulk(1.0), mc.bulk_from_mci_columns(1.4, 0.1, 30.0, g=0.9),
             mc.bulk_from_mci_columns(1.4, 0.3, 50.0, 1.0, 0.05, 0.02, 0.1, 0.85), mc.outer_bulk(1.0)]
    det = mc.Detector(0.0, 0.0, 0.1, 0.1, 50, 50)
    from oracle import pyoracle
    sim = pyoracle.sim_from_arrays(lab, bulks, half_x=2.56, half_y=2.56, thickness=0.64,
                                   vox_per_cm=[200.0, 200.0, 100.0], photons=4000, per_voxel=0,
                                   det=(0.1, 0.1, 50, 50, 0.0, 0.0), do_fl=2)
    ref = oracle.run_photon(sim, table32768, 5, 6, libm=False)
    med = gpu_ctx.medium(lab, bulks, vox_per_cm=(200.0, 200.0, 100.0), half_x=2.56, half_y=2.56, thickness=0.64)
    res = gpu_ctx.run(med, mc.run_desc(4000, det=det, fluence=1, seed_exc=5, seed_fl=6,
                                       start_weight=sim.start_weight))
    med.free()
    _compare(res, ref, emission=False)


@pytest.mark.gpu
def test_time_and_layer_inputs_fail_with_status(gpu_ctx):
    case = cases.mismatch_timed()
    med = case.engine_medium(gpu_ctx)
    rd = case.run_desc(1, 2)
    rd.tdet.bins = 0
    with pytest.raises(mc.McflError) as e:
        gpu_ctx.run(med, rd)
    assert e.value.code == mc.E_ARG
    rd = case.run_desc(1, 2)
    rd.tdet.face = 2
    with pytest.raises(mc.McflError):
        gpu_ctx.run(med, rd)
    med.free()
    lc = cases.layered()
    lm = lc.engine_medium(gpu_ctx)
    rd = lc.run_desc(1, 2)
    rd.source.z = 5.0  # below every slab
    with pytest.raises(mc.McflError) as e:
        gpu_ctx.run(lm, rd)
    assert e.value.code == mc.E_ARG
    rd = lc.run_desc(1, 2)
    rd.photons_per_voxel = 100  # no emission in layered media
    with pytest.raises(mc.McflError):
        gpu_ctx.run(lm, rd)
    lm.free()
    with pytest.raises(mc.McflError) as e:
        gpu_ctx.medium_layered(lc.layers()[:1] + lc.layers()[-1:], lc.incl(), 10)  # no slab
    assert e.value.code == mc.E_RANGE


@pytest.mark.gpu
@pytest.mark.parametrize("reuse", [0, 1])
def test_photon_offset_shards_sum_to_the_whole_run(reuse, gpu_ctx):
    """Runs over disjoint photon index ranges of one seed (photon_offset) sum
    to the run over their union, bit for bit: the decomposition a multi-GPU
    run would use; with the reference's first-photon reuse on, the reuse
    follows the index in the whole run (the first 32768 photons span both
    shards here)."""
    case = cases.mismatch(photons=40000, per_voxel=0)
    case.do_fl = 2
    med = case.engine_medium(gpu_ctx)
    rd = case.run_desc(7, 8)
    rd.launch_rng_reuse = reuse
    whole = gpu_ctx.run(med, rd)
    parts = []
    for off, n in ((0, 17000), (17000, 23000)):
        rd = case.run_desc(7, 8, photons=n)
        rd.photon_offset = off
        rd.launch_rng_reuse = reuse
        parts.append(gpu_ctx.run(med, rd))
    med.free()
    for k in ("Rd", "Tt", "fhd"):
        assert np.array_equal(getattr(parts[0], k) + getattr(parts[1], k), getattr(whole, k)), k
    for k in STAT_ORDER + ("steps", "done"):
        assert parts[0].stats_exc[k] + parts[1].stats_exc[k] == whole.stats_exc[k], k


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(cases.EXACT))
def test_voxel_boundary_stepping_bit_identical_to_oracle(name, gpu_ctx, oracle, table32768):
    """Voxel-boundary stepping (mu_t spent voxel by voxel, Fresnel with each
    face's normal, scattering-free voxels crossed): the exact-math kernel
    against the oracle's restatement, excitation and emission, bit for bit."""
    case = cases.EXACT[name](photons=20000, per_voxel=500)
    ref = oracle.run_photon(case.oracle_sim(), table32768, 11, 22, libm=False)
    med = case.engine_medium(gpu_ctx)
    res = gpu_ctx.run(med, case.run_desc(11, 22))
    med.free()
    _compare(res, ref)
    assert ref.fl_voxels > 0


@pytest.mark.gpu
def test_voxel_boundary_stepping_inputs_fail_with_status(gpu_ctx):
    """Exact stepping has no layered media; a batch shares one stepping."""
    med = cases.mismatch().engine_medium(gpu_ctx)
    a = cases.mismatch().run_desc(1, 2)
    a.photons_per_voxel, a.fluence = 0, 0
    b = cases.mismatch().run_desc(3, 4)
    b.photons_per_voxel, b.fluence = 0, 0
    b.exact_stepping = 1
    with pytest.raises(mc.McflError) as e:
        mc.batch_run(gpu_ctx, med, [a, b])
    assert e.value.code == mc.E_ARG
    med.free()
    lc = cases.layered()
    lm = lc.engine_medium(gpu_ctx)
    rd = lc.run_desc(1, 2)
    rd.exact_stepping = 1
    with pytest.raises(mc.McflError) as e:
        gpu_ctx.run(lm, rd)
    assert e.value.code == mc.E_ARG
    lm.free()


@pytest.mark.gpu
def test_voxel_boundary_stepping_batch_equals_alone(gpu_ctx):
    """Batched and plain schedules of exact-stepping runs equal each run
    alone, bit for bit."""
    case = cases.mismatch()
    med = case.engine_medium(gpu_ctx)
    dx, dy, nx, ny, x0, y0 = case.det
    det = mc.Detector(x0, y0, dx, dy, nx, ny)
    budgets = [5000, 17000, 1, 900]
    runs = [mc.run_desc(b, source=(0.1 * i - 0.15, 0.05, 0.0), det=det, seed_exc=40 + i,
                        start_weight=case.start_weight(), exact_stepping=1) for i, b in enumerate(budgets)]
    bat, _ = mc.batch_run(gpu_ctx, med, runs, mc.SCHEDULE_BATCHED)
    pla, _ = mc.batch_run(gpu_ctx, med, runs, mc.SCHEDULE_PLAIN)
    for i, rd in enumerate(runs):
        one = gpu_ctx.run(med, rd, images=True, raw=True)
        for r in (bat[i], pla[i]):
            assert np.array_equal(r["Rd"], one.Rd) and np.array_equal(r["Tt"], one.Tt)
            assert r["stats"]["done"] == budgets[i]
            assert r["stats"]["steps"] == one.stats_exc["steps"]
            assert r["stats"]["absorbed"] == one.stats_exc["absorbed"]
    med.free()
