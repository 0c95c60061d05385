"""Batching, the plain schedule, graph replay and the continuous-batching
server.  Every schedule must reproduce the tallies of the same simulation run
alone, bit for bit: photon k of a simulation always draws stream
(key, offset + k) and all tallies are integer sums."""
import numpy as np
import pytest

import cudamcfl_gb300 as mc
from cudamcfl_gb300 import media
from tests import cases


def _alone(ctx, med, rd):
    return ctx.run(med, rd, images=True, raw=True)


@pytest.mark.gpu
def test_batched_equals_plain_equals_alone(gpu_ctx):
    case = cases.sphere()
    med = case.engine_medium(gpu_ctx)
    dx, dy, nx, ny, x0, y0 = case.det
    det = mc.Detector(x0, y0, dx, dy, nx, ny)
    srcs = [(-0.3, 0.1), (0.0, 0.0), (0.25, -0.2), (0.5, 0.5), (-0.6, -0.4)]
    budgets = [3000, 20000, 7000, 12000, 500]
    runs = [mc.run_desc(b, source=(x, y, 0.0), det=det, seed_exc=100 + i, start_weight=case.start_weight())
            for i, ((x, y), b) in enumerate(zip(srcs, budgets))]
    bat, _ = mc.batch_run(gpu_ctx, med, runs, mc.SCHEDULE_BATCHED)
    pla, _ = mc.batch_run(gpu_ctx, med, runs, mc.SCHEDULE_PLAIN)
    for i, rd in enumerate(runs):
        one = _alone(gpu_ctx, med, rd)
        for r in (bat[i], pla[i]):
            assert np.array_equal(r["Rd"], one.Rd) and np.array_equal(r["Tt"], one.Tt)
            assert np.array_equal(r["R"], one.R) and np.array_equal(r["T"], one.T)
            assert r["stats"]["done"] == budgets[i]
            assert r["stats"]["absorbed"] == one.stats_exc["absorbed"]
    # replaying the recorded batch graph reproduces it
    bat2, _ = mc.batch_run(gpu_ctx, med, runs, mc.SCHEDULE_BATCHED)
    for a, b in zip(bat, bat2):
        assert np.array_equal(a["Rd"], b["Rd"]) and np.array_equal(a["Tt"], b["Tt"])


@pytest.mark.gpu
def test_batch_over_many_media_equals_alone(gpu_ctx):
    """Sources on four different media (voxelized, mismatched, glass and
    sphere) with uneven budgets in one launch of the mixed-media kernel, and
    in the plain schedule: each equals its run alone, bit for bit."""
    chosen = [cases.tiny(), cases.mismatch(), cases.glass(), cases.sphere()]
    meds = [c.engine_medium(gpu_ctx) for c in chosen]
    det = mc.Detector(0.0, 0.0, 0.1, 0.1, 20, 20)
    runs, media_of = [], []
    budgets = [4000, 25000, 900, 12000, 7000, 3000, 16000, 1]
    for i, b in enumerate(budgets):
        k = i % len(chosen)
        runs.append(mc.run_desc(b, source=(0.05 * k, -0.02 * k, 0.0), det=det, seed_exc=300 + i,
                                start_weight=chosen[k].start_weight()))
        media_of.append(meds[k])
    bat, _ = mc.batch_run(gpu_ctx, media_of, runs, mc.SCHEDULE_BATCHED)
    pla, _ = mc.batch_run(gpu_ctx, media_of, runs, mc.SCHEDULE_PLAIN)
    for i, rd in enumerate(runs):
        one = _alone(gpu_ctx, media_of[i], rd)
        for r in (bat[i], pla[i]):
            assert np.array_equal(r["Rd"], one.Rd) and np.array_equal(r["Tt"], one.Tt)
            assert r["stats"]["done"] == budgets[i]
            assert r["stats"]["absorbed"] == one.stats_exc["absorbed"]
            assert r["stats"]["steps"] == one.stats_exc["steps"]
    for m in meds:
        m.free()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny", "sphere"])
def test_plain_per_voxel_emission_equals_batched(name, gpu_ctx):
    case = cases.ALL[name](photons=20000, per_voxel=300)
    med = case.engine_medium(gpu_ctx)
    rd = case.run_desc(31, 32)
    bat = gpu_ctx.run(med, rd)
    pla = mc.run_plain(gpu_ctx, med, rd)
    assert pla["fl_voxels"] == bat.fl_voxels > 0
    assert np.array_equal(pla["Rd"], bat.Rd) and np.array_equal(pla["Tt"], bat.Tt)
    assert np.array_equal(pla["flR128"], bat.flR128) and np.array_equal(pla["flT128"], bat.flT128)
    assert pla["stats_fl"]["steps"] == bat.stats_fl["steps"]


@pytest.mark.gpu
def test_graph_replay_follows_new_seeds(gpu_ctx):
    case = cases.mismatch(photons=20000, per_voxel=100)
    med = case.engine_medium(gpu_ctx)
    a1 = gpu_ctx.run(med, case.run_desc(1, 2))
    b = gpu_ctx.run(med, case.run_desc(3, 4))
    a2 = gpu_ctx.run(med, case.run_desc(1, 2))
    assert np.array_equal(a1.Rd, a2.Rd) and np.array_equal(a1.flR128, a2.flR128)
    assert not np.array_equal(a1.Rd, b.Rd)
    gpu_ctx.set_option("graphs", 0)
    try:
        a3 = gpu_ctx.run(med, case.run_desc(1, 2))
    finally:
        gpu_ctx.set_option("graphs", 1)
    assert np.array_equal(a1.Rd, a3.Rd) and np.array_equal(a1.fhd, a3.fhd)


def _request_media(seed):
    rng = np.random.default_rng(seed)
    out = []
    for i, (nx, ny, nz) in enumerate([(32, 32, 16), (48, 40, 24), (64, 64, 32), (24, 24, 24)]):
        vox = (0.05, 0.05, 0.05)
        lab = np.ones((nz, ny, nx), dtype=np.uint8)
        media.add_sphere(lab, vox, (rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3), nz * 0.05 / 2), 0.3, 2)
        bulks = [mc.outer_bulk(1.0), mc.bulk_from_mci_columns(1.4, 0.1 + 0.05 * i, 80.0 + 10 * i, g=0.85),
                 mc.bulk_from_mci_columns(1.33, 0.5, 50.0, g=0.7), mc.outer_bulk(1.0)]
        out.append((lab, bulks, vox))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("slice_passes,slice_us,express_period,express_ratio,relaunch",
                         [(64, 0, 0, 0, 1), (4096, 0, 0, 0, 1), (64, 0, 2, 2, 8), (256, 0, 7, 1, 32),
                          (0, 200, 0, 0, 1), (0, 0, 0, 0, 2)])
def test_server_results_equal_alone(slice_passes, slice_us, express_period, express_ratio, relaunch, gpu_ctx):
    """Each served result equals the same request run alone, bit for bit, for
    slices ended by a pass cap or by the clock, any queue policy and any
    relaunch threshold."""
    meds = _request_media(7)
    det = mc.Detector(0.0, 0.0, 0.05, 0.05, 30, 30)
    reqs = []
    for i in range(10):
        lab, bulks, vox = meds[i % len(meds)]
        kind = mc.SOURCE_WIDEFIELD if i % 3 == 0 else mc.SOURCE_GAUSS_BEAM
        rd = mc.run_desc(2000 + 1500 * i, source=(0.05 * i - 0.2, 0.0, 0.0), det=det, fluence=i % 2,
                         seed_exc=500 + i, kind=kind, width=1.0, height=0.8)
        reqs.append((lab, bulks, vox, rd))
    ctx2 = mc.Context(math=mc.MATH_EXACT)
    ctx2.set_option("relaunch", relaunch)
    srv = mc.Server(ctx2, hbm_budget_bytes=64 << 20, max_jobs=4, slice_passes=slice_passes,
                    express_period=express_period, express_ratio=express_ratio, slice_us=slice_us)
    try:
        ids = [srv.submit(lab, bulks, vox, rd) for lab, bulks, vox, rd in reqs]
        results = []
        for rid in ids:
            assert srv.wait(rid, 120000) == 0
            results.append(srv.result(rid))
        m = srv.metrics()
        assert m["completed"] == len(reqs) and m["max_inflight"] > 1
    finally:
        srv.close()
        ctx2.close()
    for (lab, bulks, vox, rd), res in zip(reqs, results):
        med = gpu_ctx.medium(lab, bulks, voxel_cm=vox)
        one = gpu_ctx.run(med, rd)
        assert np.array_equal(res["Rd"], one.Rd) and np.array_equal(res["Tt"], one.Tt)
        assert res["stats"]["absorbed"] == one.stats_exc["absorbed"]
        assert res["stats"]["steps"] == one.stats_exc["steps"]
        if rd.fluence:
            assert np.array_equal(res["fhd"], one.fhd)
        med.free()


@pytest.mark.gpu
def test_server_rejects_request_above_budget(gpu_ctx):
    lab = np.ones((64, 64, 64), dtype=np.uint8)
    bulks = [mc.outer_bulk(1.0), mc.bulk_from_mci_columns(1.4, 0.1, 100.0), mc.outer_bulk(1.0)]
    det = mc.Detector(0.0, 0.0, 0.05, 0.05, 10, 10)
    ctx2 = mc.Context()
    srv = mc.Server(ctx2, hbm_budget_bytes=1 << 16, max_jobs=2)
    try:
        rid = srv.submit(lab, bulks, (0.05, 0.05, 0.05), mc.run_desc(1000, det=det))
        assert srv.wait(rid, 60000) == mc.E_RANGE
    finally:
        srv.close()
        ctx2.close()


@pytest.mark.gpu
def test_recorded_graph_follows_a_new_medium_at_a_reused_address(gpu_ctx, oracle, table32768):
    """Media freed and created in turn (the allocator may hand a new medium
    the old one's address; the label counts differ) never replay the previous
    medium's recorded graph: every run equals the oracle."""
    from tests.test_gpu_parity import _compare
    for make in (cases.tiny, cases.glass, cases.tiny, cases.mismatch, cases.glass):
        case = make(photons=3000, per_voxel=0)
        case.do_fl = 2
        ref = oracle.run_photon(case.oracle_sim(), table32768, 12, 13, libm=False)
        med = case.engine_medium(gpu_ctx)
        res = gpu_ctx.run(med, case.run_desc(12, 13))
        med.free()
        _compare(res, ref, emission=False)


def _same(res, one, timed=False):
    assert np.array_equal(res["Rd"], one.Rd) and np.array_equal(res["Tt"], one.Tt)
    for k in ("done", "steps", "absorbed", "exit_top", "exit_bottom"):
        assert res["stats"][k] == one.stats_exc[k], k
    if timed:
        assert np.array_equal(res["time_xyt"], one.time_xyt.ravel())
        assert one.time_xyt.sum() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [0, 1])
def test_batch_time_detectors_equal_alone(exact, gpu_ctx):
    """Runs with and without time-resolved detectors in one batch, over one
    medium (single-medium timed kernel) and over several (mixed-media timed
    kernel), with the reference's and with voxel-boundary stepping: each run's
    histograms, images and weight accounting equal the run alone."""
    base = [cases.timed(face=0), cases.timed(face=1, base=cases.glass), cases.timed(face=1)]
    meds = [c.engine_medium(gpu_ctx) for c in base]
    try:
        det = mc.Detector(0.0, 0.0, 0.1, 0.1, 20, 20)
        runs, media_of = [], []
        for i, b in enumerate([6000, 15000, 900, 9000, 4000, 1]):
            c = base[i % 3]
            runs.append(mc.run_desc(b, source=(0.02 * i, -0.03 * i, 0.0), det=det, seed_exc=700 + i,
                                    start_weight=c.start_weight(), tdet=c.temporal if i % 2 == 0 else None,
                                    exact_stepping=exact))
            media_of.append(meds[i % 3])
        for medium in (meds[0], media_of):  # one medium, then several
            for sched in (mc.SCHEDULE_BATCHED, mc.SCHEDULE_PLAIN):
                got, _ = mc.batch_run(gpu_ctx, medium, runs, sched)
                for i, rd in enumerate(runs):
                    m = medium if not isinstance(medium, list) else medium[i]
                    _same(got[i], gpu_ctx.run(m, rd, images=True, raw=True), timed=bool(rd.tdet.nx))
    finally:
        for m in meds:
            m.free()


@pytest.mark.gpu
def test_batch_voxel_boundary_stepping_over_several_media_equals_alone(gpu_ctx):
    """Voxel-boundary stepping over four media in one launch of the
    mixed-media kernel (each job carrying its medium's label + free-radius
    map): every run equals its run alone, bit for bit."""
    chosen = [cases.tiny(), cases.mismatch(), cases.glass(), cases.sparse()]
    meds = [c.engine_medium(gpu_ctx) for c in chosen]
    try:
        det = mc.Detector(0.0, 0.0, 0.1, 0.1, 20, 20)
        runs, media_of = [], []
        for i, b in enumerate([4000, 25000, 900, 12000, 7000, 3000, 16000, 1]):
            k = i % len(chosen)
            runs.append(mc.run_desc(b, source=(0.05 * k, -0.02 * k, 0.0), det=det, seed_exc=300 + i,
                                    start_weight=chosen[k].start_weight(), exact_stepping=1))
            media_of.append(meds[k])
        bat, _ = mc.batch_run(gpu_ctx, media_of, runs, mc.SCHEDULE_BATCHED)
        for i, rd in enumerate(runs):
            _same(bat[i], gpu_ctx.run(media_of[i], rd, images=True, raw=True))
    finally:
        for m in meds:
            m.free()


@pytest.mark.gpu
@pytest.mark.parametrize("slice_passes", [64, 4096, 0])
def test_server_time_detectors_and_stepping_equal_alone(slice_passes, gpu_ctx):
    """Requests of all four kinds (the reference's or voxel-boundary
    stepping, with or without time-resolved detectors) served together: the
    kinds take turns in slices, each with its own photons in flight, and
    every result equals the request run alone, bit for bit."""
    meds = _request_media(11)
    det = mc.Detector(0.0, 0.0, 0.05, 0.05, 30, 30)
    tdet = (0.0, 0.0, 2, 2, 0.3, 0.3, 0.2, 1, 24, 300000)
    reqs = []
    for i in range(12):
        lab, bulks, vox = meds[i % len(meds)]
        rd = mc.run_desc(1500 + 1300 * i, source=(0.04 * i - 0.2, 0.01 * i, 0.0), det=det, fluence=i % 2,
                         seed_exc=900 + i, tdet=tdet if (i // 2) % 2 else None, exact_stepping=i % 2)
        reqs.append((lab, bulks, vox, rd))
    ctx2 = mc.Context(math=mc.MATH_EXACT)
    srv = mc.Server(ctx2, hbm_budget_bytes=64 << 20, max_jobs=5, slice_passes=slice_passes)
    try:
        ids = [srv.submit(lab, bulks, vox, rd) for lab, bulks, vox, rd in reqs]
        results = []
        for rid in ids:
            assert srv.wait(rid, 120000) == 0
            results.append(srv.result(rid))
    finally:
        srv.close()
        ctx2.close()
    for (lab, bulks, vox, rd), res in zip(reqs, results):
        med = gpu_ctx.medium(lab, bulks, voxel_cm=vox)
        one = gpu_ctx.run(med, rd)
        _same(res, one, timed=bool(rd.tdet.nx))
        if rd.fluence:
            assert np.array_equal(res["fhd"], one.fhd)
        med.free()
