"""Statistical gates of the CUDA engine (3 sigma of the batch-means standard
error per pixel; integrated reflectance, transmittance and absorbed fraction
within 3 sigma and within 0.1 % where the photon budget resolves 0.1 %).

  fast-math kernel vs exact-math kernel: same physics, hardware SFU
  intrinsics vs the portable series (the exact kernel is bit-identical to the
  oracle's photon-indexed restatement);
  CUDA engine vs the reference's own RNG streams and schedule (the oracle's
  reference-stream restatement, bit-identical to the reference), with the
  reference's first-photon random-number reuse reproduced.
"""
import os

import numpy as np
import pytest

import cudamcfl_gb300 as mc
from tests import cases, stats

B = 16


def _run(ctx, med, case, b, photons=None, per_voxel=None, emission=True, seed0=0, reuse=0):
    rd = case.run_desc(seed0 + 11 + b, seed0 + 5011 + b, photons=photons)
    if per_voxel is not None:
        rd.photons_per_voxel = per_voxel
    if not emission:
        rd.photons_per_voxel = 0
    rd.launch_rng_reuse = reuse
    return ctx.run(med, rd)


def _fractions(results, w0):
    out = {}
    for k in ("absorbed", "exit_top", "exit_bottom"):
        out[k] = [r.stats_exc[k] / (r.stats_exc["done"] * w0) for r in results]
    return out


@pytest.mark.gpu
def test_fast_math_kernel_agrees_with_exact_kernel(gpu_ctx):
    case = cases.sphere()
    fast = mc.Context(math=mc.MATH_FAST)
    try:
        me, mf = case.engine_medium(gpu_ctx), case.engine_medium(fast)
        ex = [_run(gpu_ctx, me, case, b, photons=400_000, per_voxel=300) for b in range(B)]
        fa = [_run(fast, mf, case, b, photons=400_000, per_voxel=300, seed0=100) for b in range(B)]
        xy = case.det[2] * case.det[3]
        for k in ("Rd", "Tt", "fhd"):
            a = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in fa])
            b = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in ex])
            stats.gate(a, b, frac_max=0.02, min_rel=1e-2, shape=None if k == "fhd" else (case.det[3], case.det[2]))
        for k in ("flR", "flT"):
            stats.gate(np.stack([getattr(r, k)[:xy] for r in fa]), np.stack([getattr(r, k)[:xy] for r in ex]),
                       frac_max=0.02, min_rel=1e-2)
        # integrated, 1.6e8 photons per kernel: 0.1 %
        ex = [_run(gpu_ctx, me, case, b, photons=10_000_000, emission=False, seed0=7) for b in range(B)]
        fa = [_run(fast, mf, case, b, photons=10_000_000, emission=False, seed0=900) for b in range(B)]
        w0 = case.start_weight()
        fx, ff = _fractions(ex, w0), _fractions(fa, w0)
        for k in fx:
            stats.scalar_gate(ff[k], fx[k], rel_tol=1e-3)
    finally:
        fast.close()


@pytest.mark.gpu
@pytest.mark.parametrize("math", [mc.MATH_EXACT, mc.MATH_FAST])
def test_engine_agrees_with_reference_streams(math, oracle, safeprimes_file):
    """tiny medium, fluorescent voxels at the beam entry; the reference side is
    the reference-stream restatement on all host cores."""
    nthreads = os.cpu_count() or 1
    case = cases.tiny(photons=250_000, per_voxel=33000)
    sim = case.oracle_sim()
    ref = [oracle.run_refstream(sim, safeprimes_file, 1000 + b, 2000 + b, libm=True, nthreads=nthreads)
           for b in range(B)]
    ctx = mc.Context(math=math)
    med = case.engine_medium(ctx)
    eng = [_run(ctx, med, case, b, reuse=1, seed0=300) for b in range(B)]
    med.free()
    xy = case.det[2] * case.det[3]
    for k in ("Rd", "Tt", "fhd"):
        a = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in eng])
        b = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in ref])
        stats.gate(a, b, frac_max=0.02, min_rel=1e-2, shape=None if k == "fhd" else (case.det[3], case.det[2]))
    for k in ("flR", "flT"):
        stats.gate(np.stack([getattr(r, k)[:xy] for r in eng]), np.stack([getattr(r, k)[:xy] for r in ref]),
                   frac_max=0.02, min_rel=1e-2)
    w0 = case.start_weight()
    fe = _fractions(eng, w0)
    for i, k in enumerate(("absorbed", "exit_top", "exit_bottom")):
        stats.scalar_gate(fe[k], [r.balance[i] / (r.photons_exc * w0) for r in ref])
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("math", [mc.MATH_EXACT, mc.MATH_FAST])
@pytest.mark.parametrize("face", [0, 1])
def test_time_resolved_detectors_agree_with_reference_streams(math, face, oracle, safeprimes_file):
    """Time-of-flight histograms of the disc detectors on the entry or exit
    face, engine against the reference-stream restatement (excitation only),
    per detector and time bin within 3 sigma."""
    nthreads = os.cpu_count() or 1
    case = cases.timed(photons=200_000, per_voxel=0, face=face)
    case.do_fl = 0
    sim = case.oracle_sim()
    ref = [oracle.run_refstream(sim, safeprimes_file, 4000 + b, 1, libm=True, nthreads=nthreads) for b in range(B)]
    ctx = mc.Context(math=math)
    med = case.engine_medium(ctx)
    eng = [_run(ctx, med, case, b, emission=False, reuse=1, seed0=700) for b in range(B)]
    med.free()
    ctx.close()
    a = np.stack([r.time_xyt.ravel().astype(float) for r in eng])
    b = np.stack([r.time_xyt.astype(float) for r in ref])
    assert b.sum() > 0
    stats.gate(a, b, frac_max=0.02, min_rel=1e-2)


@pytest.mark.gpu
@pytest.mark.parametrize("math", [mc.MATH_EXACT, mc.MATH_FAST])
def test_layered_medium_agrees_with_reference_streams(math, oracle, safeprimes_file):
    """Layered medium (bulk method 1) with time-resolved detectors: engine
    against the reference-stream restatement, R/T, fluence and time bins
    within 3 sigma."""
    nthreads = os.cpu_count() or 1
    case = cases.layered_timed_exit(photons=150_000)
    sim = case.oracle_sim()
    ref = [oracle.run_refstream(sim, safeprimes_file, 6000 + b, 1, libm=True, nthreads=nthreads) for b in range(B)]
    ctx = mc.Context(math=math)
    med = case.engine_medium(ctx)
    eng = []
    for b in range(B):
        rd = case.run_desc(900 + b, 1)
        rd.launch_rng_reuse = 1
        eng.append(ctx.run(med, rd))
    med.free()
    ctx.close()
    xy = case.det[2] * case.det[3]
    for k in ("Rd", "Tt", "fhd"):
        a = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in eng])
        b = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in ref])
        stats.gate(a, b, frac_max=0.02, min_rel=1e-2, shape=None if k == "fhd" else (case.det[3], case.det[2]))
    stats.gate(np.stack([r.time_xyt.ravel().astype(float) for r in eng]),
               np.stack([r.time_xyt.astype(float) for r in ref]), frac_max=0.02, min_rel=1e-2)
    w0 = case.start_weight()
    fe = _fractions(eng, w0)
    for i, k in enumerate(("absorbed", "exit_top", "exit_bottom")):
        stats.scalar_gate(fe[k], [r.balance[i] / (r.photons_exc * w0) for r in ref])


@pytest.mark.gpu
def test_integrated_within_0p1_percent_of_reference_streams(oracle, safeprimes_file):
    """Integrated R, T and absorbed fraction of the fast kernel against the
    reference streams on 1.6e7 reference photons: within 3 sigma and 0.1 %
    with the reference's first-photon reuse reproduced; within 0.1 % without
    it (the reuse biases the reference's own reflectance by a few 1e-4 at this
    budget, 3.3 % first photons)."""
    nthreads = os.cpu_count() or 1
    case = cases.tiny(photons=1_000_000, per_voxel=0)
    case.do_fl = 0
    sim = case.oracle_sim()
    ref = [oracle.run_refstream(sim, safeprimes_file, 70_000 + b, 1, libm=True, nthreads=nthreads)
           for b in range(B)]
    ctx = mc.Context(math=mc.MATH_FAST)
    med = case.engine_medium(ctx)
    w0 = case.start_weight()
    for reuse in (1, 0):
        if reuse:
            runs = [_run(ctx, med, case, b, photons=1_000_000, emission=False, reuse=1, seed0=5000 + 37 * b)
                    for b in range(B)]
        else:
            runs = [_run(ctx, med, case, b, photons=20_000_000, emission=False, reuse=0, seed0=9000)
                    for b in range(B)]
        fe = _fractions(runs, w0)
        for i, k in enumerate(("absorbed", "exit_top", "exit_bottom")):
            r = [x.balance[i] / (x.photons_exc * w0) for x in ref]
            if reuse:
                out = stats.scalar_gate(fe[k], r, rel_tol=None)
            else:
                a, b = np.mean(fe[k]), np.mean(r)
                out = {"a": a, "b": b, "rel_diff": abs(a - b) / b}
            assert out["rel_diff"] < 1e-3, (reuse, k, out)
    med.free()
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("math", [mc.MATH_EXACT, mc.MATH_FAST])
def test_voxel_boundary_stepping_agrees_with_independent_slab_mc(math):
    """Two index-mismatched slabs as a laterally wide voxel grid: the engine's
    voxel-boundary stepping gives the reflectance, transmittance and absorbed
    fraction of the independent layered-slab Monte Carlo (tests/slab_mc.py)
    within 3 sigma."""
    from tests import slab_mc
    layers = [(0.04, 1.0, 100.0, 0.9, 1.37), (0.06, 0.5, 80.0, 0.8, 1.5)]
    lab = np.ones((10, 8, 8), np.uint8)
    lab[4:] = 2
    bulks = [mc.outer_bulk(1.0)] + [mc.bulk_from_mci_columns(l[4], l[1], l[2], g=l[3]) for l in layers] + \
        [mc.outer_bulk(1.0)]
    ctx = mc.Context(math=math)
    try:
        med = ctx.medium(lab, bulks, vox_per_cm=(0.1, 0.1, 100.0), half_x=40.0, half_y=40.0, thickness=0.1)
        det = mc.Detector(0.0, 0.0, 0.1, 0.1, 10, 10)
        runs = [mc.run_desc(200_000, det=det, seed_exc=77 + b, exact_stepping=1) for b in range(B)]
        res, _ = mc.batch_run(ctx, med, runs)
        med.free()
    finally:
        ctx.close()
    n1, n2 = np.float64(np.float32(1.0)), np.float64(np.float32(1.37))
    w0 = int(np.float64(0xFFFFFFFF) * (1 - ((n1 - n2) / (n1 + n2)) ** 2))
    eng = np.array([[r["stats"][k] / (200_000 * w0) for k in ("exit_top", "exit_bottom", "absorbed")] for r in res])
    ref = np.array([slab_mc.run(layers, 1.0, 1.0, 20000, 4100 + b) for b in range(B)])
    for i in range(3):
        stats.scalar_gate(eng[:, i], ref[:, i])
