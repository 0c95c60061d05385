"""CPU statistical gate between the two RNG schemes of the oracle.

port(refstream, libm) is bit-identical to the reference (test_oracle_pinned);
port(photon, portable) is bit-identical to the CUDA exact-math kernel
(test_gpu_parity).  Here the two are compared as Monte Carlo estimators on
independent seeds: per-pixel R/T/photon-hitting-density and emission images
within 3 sigma of the batch-means standard error, and the integrated
reflectance, transmittance and absorbed fraction within 3 sigma.

The reference's first photon on each of its 32768 threads reuses its launch
random numbers for its first passes (CUDAMCFLtransport.cu:574-581); the
photon-indexed run reproduces that with launch_rng_reuse, so both sides carry
the same small correlation (in the emission phase 32768 of every voxel's
33000 photons are first photons).
"""
import os

import numpy as np
import pytest

from tests import cases, stats

B = 16


def _batches(fn):
    return [fn(b) for b in range(B)]


def test_photon_streams_agree_with_reference_streams(oracle, table32768, safeprimes_file):
    nthreads = os.cpu_count() or 1
    case = cases.tiny(photons=250_000, per_voxel=33000)
    sim = case.oracle_sim()
    ref = _batches(lambda b: oracle.run_refstream(sim, safeprimes_file, 1000 + b, 2000 + b, libm=True,
                                                  nthreads=nthreads))
    sim2 = case.oracle_sim()
    sim2.launch_rng_reuse = 1
    eng = _batches(lambda b: oracle.run_photon(sim2, table32768, 5000 + b, 6000 + b, libm=False))
    xy = case.det[2] * case.det[3]
    norm = lambda r: r.photons_exc  # noqa: E731
    for k in ("Rd", "Tt", "fhd"):
        a = np.stack([getattr(r, k)[:xy if k != "fhd" else None] / norm(r) for r in eng])
        b = np.stack([getattr(r, k)[:xy if k != "fhd" else None] / norm(r) for r in ref])
        stats.gate(a, b, frac_max=0.02, min_rel=1e-2, shape=None if k == "fhd" else (case.det[3], case.det[2]))
    for k in ("flR", "flT"):
        a = np.stack([getattr(r, k)[:xy] for r in eng])
        b = np.stack([getattr(r, k)[:xy] for r in ref])
        stats.gate(a, b, frac_max=0.02, min_rel=1e-2)
    w0 = case.start_weight()
    for i in (0, 1, 2):  # absorbed, left through z=0, left through z=esp
        stats.scalar_gate([r.balance[i] / (r.photons_exc * w0) for r in eng],
                          [r.balance[i] / (r.photons_exc * w0) for r in ref])
