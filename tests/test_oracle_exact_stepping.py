"""Voxel-boundary ("exact") stepping of the oracle against an independent
layered-slab Monte Carlo (tests/slab_mc.py).

A laterally wide voxel grid whose labels change only with depth is a layered
slab; the oracle's exact stepping (optical depth spent voxel by voxel,
Fresnel at every index step with the face's normal) must give the slab's
reflectance, transmittance and absorbed fraction within 3 sigma of the
independent implementation, with and without index steps.  The reference's
own stepping (the whole step with the start voxel's mu_t, z as the Fresnel
normal, and an interaction where a step clipped at a face ends, reflected
or not) is biased wherever indices differ; in a single-label slab without
an index step at its faces the two steppings agree.
"""
import numpy as np
import pytest

import cudamcfl_gb300 as mc
from tests import slab_mc, stats

B = 16
N = 20000


def _slab_sim(layers, n_out, photons, exact, lateral=(8, 0.1, 40.0)):
    """lateral: voxels across, voxels per cm and half extent of the grid."""
    from oracle import pyoracle
    nz = [int(round(l[0] * 100)) for l in layers]
    nl, gl, half = lateral
    lab = np.ones((sum(nz), nl, nl), np.uint8)
    z0 = 0
    for i, k in enumerate(nz):
        lab[z0:z0 + k] = i + 1
        z0 += k
    bulks = [mc.outer_bulk(n_out)] + [mc.bulk_from_mci_columns(l[4], l[1], l[2], g=l[3]) for l in layers] + \
        [mc.outer_bulk(n_out)]
    sim = pyoracle.sim_from_arrays(lab, bulks, half_x=half, half_y=half, thickness=sum(nz) / 100.0,
                                   vox_per_cm=[gl, gl, 100.0], photons=photons, per_voxel=0,
                                   det=(0.1, 0.1, 10, 10, 0.0, 0.0), do_fl=0)
    sim.exact_stepping = exact
    return sim


def _fractions(oracle, table, sim, seed):
    r = oracle.run_photon(sim, table, seed, seed + 1, libm=False)
    w0 = sim.start_weight * sim.number_of_photons
    return r.balance[1] / w0, r.balance[2] / w0, r.balance[0] / w0


CASES = {
    "matched": [(0.04, 1.0, 100.0, 0.9, 1.0), (0.06, 0.5, 80.0, 0.8, 1.0)],
    "two_layer_mismatch": [(0.04, 1.0, 100.0, 0.9, 1.37), (0.06, 0.5, 80.0, 0.8, 1.5)],
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_exact_stepping_matches_independent_slab_mc(name, oracle, table32768):
    layers = CASES[name]
    sim = _slab_sim(layers, 1.0, N, 1)
    port = np.array([_fractions(oracle, table32768, sim, 7000 + 13 * b) for b in range(B)])
    ref = np.array([slab_mc.run(layers, 1.0, 1.0, N, 9000 + b) for b in range(B)])
    for i in range(3):
        stats.scalar_gate(port[:, i], ref[:, i])


def test_reference_stepping_is_biased_on_index_steps_and_agrees_without_them(oracle, table32768):
    layers = CASES["two_layer_mismatch"]
    ex = np.array([_fractions(oracle, table32768, _slab_sim(layers, 1.0, N, 1), 300 + b) for b in range(B)])
    rc = np.array([_fractions(oracle, table32768, _slab_sim(layers, 1.0, N, 0), 300 + b) for b in range(B)])
    se = np.sqrt(ex.var(0, ddof=1) / B + rc.var(0, ddof=1) / B)
    assert abs(rc[:, 0].mean() - ex[:, 0].mean()) > 5 * se[0]  # reflectance differs well beyond the noise
    one = [(0.1, 1.0, 100.0, 0.9, 1.0)]
    ex1 = np.array([_fractions(oracle, table32768, _slab_sim(one, 1.0, N, 1), 500 + b) for b in range(B)])
    rc1 = np.array([_fractions(oracle, table32768, _slab_sim(one, 1.0, N, 0), 600 + b) for b in range(B)])
    for i in range(3):
        stats.scalar_gate(ex1[:, i], rc1[:, i])


def test_exact_stepping_beyond_a_narrow_grid_matches_independent_slab_mc(oracle, table32768):
    """A one-label slab whose voxel grid covers only 0.2 x 0.2 cm: photons
    spend most passes beyond the grid's lateral extent, where the medium of
    label 1 continues, so the slab is still homogeneous and infinite."""
    layers = [(0.1, 0.5, 20.0, 0.8, 1.4)]
    sim = lambda: _slab_sim(layers, 1.0, N, 1, lateral=(4, 20.0, 0.1))
    port = np.array([_fractions(oracle, table32768, sim(), 800 + 13 * b) for b in range(B)])
    ref = np.array([slab_mc.run(layers, 1.0, 1.0, N, 9500 + b) for b in range(B)])
    for i in range(3):
        stats.scalar_gate(port[:, i], ref[:, i])
