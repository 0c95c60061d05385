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
    finally:
        gpu_ctx.set_option("block", 256)
        gpu_ctx.set_option("blocks_per_sm", 0)


@pytest.mark.gpu
def test_excitation_only_and_no_fluence(gpu_ctx, oracle, table32768):
    case = cases.tiny(photons=25000, per_voxel=0)
    case.do_fl = 0
    ref = oracle.run_photon(case.oracle_sim(), table32768, 99, 100, libm=False)
    med = case.engine_medium(gpu_ctx)
    res = gpu_ctx.run(med, case.run_desc(99, 100))
    assert np.array_equal(res.Rd, ref.Rd) and np.array_equal(res.Tt, ref.Tt)
    assert res.fhd is None and res.flR is None
