"""The double-precision build of the transport kernel (MATH_F64) and the
single- vs double-precision study.

  F64 vs the exact single-precision kernel on independent seeds: the same
  physics, so per-pixel 3-sigma agreement (batch means) and integrated
  fractions within 3 sigma;
  F64 keeps the exact integer weight accounting;
  the paired study (identical seeds in every build) on the quarter-resolution
  precision medium: integrated R/T/A of both single-precision builds within
  a few paired standard errors of FP64 and the same mean passes per photon.
"""
import numpy as np
import pytest

import cudamcfl_gb300 as mc
from cudamcfl_gb300 import media, precision
from tests import cases, stats

B = 12


def _fractions(results, w0):
    return {k: [r.stats_exc[k] / (r.stats_exc["done"] * w0) for r in results]
            for k in ("absorbed", "exit_top", "exit_bottom")}


@pytest.mark.gpu
def test_f64_kernel_agrees_with_exact_kernel(gpu_ctx):
    case = cases.sphere(per_voxel=300)
    f64 = mc.Context(math=mc.MATH_F64)
    try:
        me, md = case.engine_medium(gpu_ctx), case.engine_medium(f64)
        ex = [gpu_ctx.run(me, case.run_desc(11 + b, 5011 + b, photons=300_000)) for b in range(B)]
        dp = [f64.run(md, case.run_desc(811 + b, 9011 + b, photons=300_000)) for b in range(B)]
        xy = case.det[2] * case.det[3]
        for k in ("Rd", "Tt", "fhd"):
            a = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in dp])
            b = np.stack([getattr(r, k)[:xy if k != "fhd" else None].astype(float) for r in ex])
            stats.gate(a, b, frac_max=0.02, min_rel=1e-2, shape=None if k == "fhd" else (case.det[3], case.det[2]))
        for k in ("flR", "flT"):
            stats.gate(np.stack([getattr(r, k)[:xy] for r in dp]), np.stack([getattr(r, k)[:xy] for r in ex]),
                       frac_max=0.02, min_rel=1e-2)
        w0 = case.start_weight()
        fx, fd = _fractions(ex, w0), _fractions(dp, w0)
        for k in fx:
            stats.scalar_gate(fd[k], fx[k])
    finally:
        f64.close()


@pytest.mark.gpu
def test_f64_kernel_conserves_weight_exactly():
    m = media.config2()
    ctx = mc.Context(math=mc.MATH_F64)
    try:
        med = ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
        rd = mc.run_desc(100_000, det=m.det, seed_exc=3, kind=mc.SOURCE_WIDEFIELD, width=3.0, height=2.0)
        s = ctx.run(med, rd).stats_exc
        w0 = int(np.float64(0xFFFFFFFF) * (1 - ((1.0 - np.float64(np.float32(1.4))) /
                                               (1.0 + np.float64(np.float32(1.4)))) ** 2))
        lhs = s["absorbed"] + s["exit_top"] + s["exit_bottom"] + s["roulette_loss"] + s["zero_drop_loss"] - \
            s["roulette_gain"]
        assert lhs % 2**64 == (100_000 * w0) % 2**64
        assert s["done"] == 100_000 and s["capped"] == 0
        med.free()
        # the server parks photons in single precision: refused for this build
        with pytest.raises(mc.McflError):
            mc.Server(ctx)
    finally:
        ctx.close()


@pytest.mark.gpu
def test_paired_precision_study_quarter_resolution():
    m = media.config5(shape=(64, 128, 128), voxel=0.04)
    ctx = mc.Context()
    try:
        med = ctx.medium(m.labels, m.bulks, voxel_cm=m.voxel_cm, fluor_map=m.fluor_map)
        w, h = m.info["widefield"]

        det = mc.Detector(0.0, 0.0, w / 32, h / 32, 32, 32)  # ~100 photons per pixel and batch

        def rd_for_seed(seed):
            return mc.run_desc(100_000, det=det, fluence=1, seed_exc=seed, seed_fl=seed + 1,
                               kind=mc.SOURCE_WIDEFIELD, width=w, height=h)

        res = precision.study(ctx, med, rd_for_seed, 6)
        s = precision.summarize(res)
        for mode in ("fast", "exact"):
            for k in ("R_total", "T_total", "absorbed"):
                # transmittance through 2.56 cm at mu_s' = 20/cm is ~1e-6: its
                # relative difference is noise, held by the paired z alone
                assert abs(s[mode][k]["z"]) < 5.0, (mode, k, s[mode][k])
                assert abs(s[mode][k]["rel_diff"]) < max(5e-3, 5 * s[mode][k]["paired_se_rel"]), (mode, k, s[mode][k])
            assert abs(s[mode]["steps_ratio"] - 1.0) < 5e-3, s[mode]
            assert s[mode]["R_image"]["entries"] > 500
            assert s[mode]["R_image"]["beyond_3se"] < 0.05, s[mode]["R_image"]
        assert ctx.get_option("math") == mc.MATH_EXACT
        med.free()
    finally:
        ctx.close()
