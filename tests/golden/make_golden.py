"""Generates the golden fixtures of tests/test_oracle_pinned.py by running the
reference's own transport (the host build oracle/_ref/libmcfl_ref.so, compiled
from the reference checkout) on the small media of tests/cases.py.

    python tests/golden/make_golden.py          (needs the reference checkout)

Each fixture holds the raw excitation R/T images, the raw photon hitting
density, the emission images and (for the media with time-resolved
detectors) the raw time-resolved tallies of one two-phase run, with the seeds and the
.mci inputs needed to reproduce it.  The multiplier file is the oracle's
generated safeprimes list (32769 lines).
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from tests import cases  # noqa: E402

SEEDS = (12345, 777)
FIXTURES = {
    "tiny": dict(photons=40000, per_voxel=33000),
    "mismatch": dict(photons=36000, per_voxel=33000),
    "glass": dict(photons=36000, per_voxel=33000),
    "mismatch_timed": dict(photons=36000, per_voxel=33000),
    "glass_timed_exit": dict(photons=36000, per_voxel=33000),
    "layered": dict(photons=36000, per_voxel=33000),
    "layered_timed_exit": dict(photons=36000, per_voxel=33000),
}


def main():
    pyoracle.build()
    ref = pyoracle.RefOracle()
    o = pyoracle.Oracle()
    with tempfile.TemporaryDirectory() as d:
        sp = os.path.join(d, "safeprimes_base32.txt")
        o.write_safeprimes(sp, 32769)
        for name, kw in FIXTURES.items():
            case = {**cases.ALL, **cases.LAYERED}[name](**kw)
            mci = case.write_mci(d)
            r = ref.run_mci(mci, sp, *SEEDS)
            out = os.path.join(HERE, f"ref_{name}.npz")
            extra = {} if r.time_xyt is None else {"time_xyt": r.time_xyt}
            np.savez_compressed(out, Rd=r.Rd, Tt=r.Tt, fhd=r.fhd, flR=r.flR, flT=r.flT, **extra,
                                photons_exc=r.photons_exc, photons_fl=r.photons_fl, fl_voxels=r.fl_voxels,
                                seeds=np.array(SEEDS, dtype=np.uint64),
                                mci=open(mci).read(),
                                bulk=open(mci.replace(".mci", ".bulk")).read() if hasattr(case, "labels") else "")
            print(out, r.photons_exc, r.photons_fl, r.fl_voxels)


if __name__ == "__main__":
    main()
