"""The 3-sigma gate itself, on synthetic batch tallies with known answers:
two samples of the same distribution pass; a small patch of biased pixels
(a localized error, e.g. a wrong voxel or detector index) fails the
clustering test; a scattered bias on a few per cent of the pixels fails the
count of pixels beyond 3 sigma."""
import numpy as np
import pytest

from tests import stats

NY, NX, B = 60, 80, 16


def _pair(seed, shift=None):
    rng = np.random.default_rng(seed)
    mean = 1000.0 + 200.0 * rng.random(NY * NX)
    a = rng.normal(mean, 40.0, size=(B, NY * NX))
    b = rng.normal(mean, 40.0, size=(B, NY * NX))
    if shift is not None:
        a = a + shift
    return a, b


@pytest.mark.parametrize("seed", range(5))
def test_same_distribution_passes(seed):
    a, b = _pair(seed)
    s = stats.gate(a, b, frac_max=0.02, shape=(NY, NX))
    assert s["pixels"] == NY * NX
    assert s["over_3sigma"] <= s["allowed_over"]


def test_allowed_count_follows_the_binomial_tail():
    a, b = _pair(11)
    s = stats.gate(a, b, frac_max=0.02, shape=(NY, NX))
    # 4800 pixels at 0.27 %: about 13 expected by chance, well below 2 %
    assert 13 <= s["allowed_over"] <= 30


def test_biased_patch_fails_the_clustering_test():
    shift = np.zeros(NY * NX)
    img = shift.reshape(NY, NX)
    img[20:23, 30:33] = 100.0  # 3x3 pixels moved by 7 standard errors
    a, b = _pair(3, shift)
    with pytest.raises(AssertionError) as e:
        stats.gate(a, b, frac_max=0.02, shape=(NY, NX))
    assert "neighbour_pairs_over" in str(e.value)
    # the same data without the clustering test passes the count (9 pixels)
    stats.gate(a, b, frac_max=0.02)


def test_scattered_bias_fails_the_count():
    rng = np.random.default_rng(5)
    shift = np.zeros(NY * NX)
    idx = rng.choice(NY * NX, size=NY * NX * 3 // 100, replace=False)
    shift[idx] = 100.0
    a, b = _pair(4, shift)
    with pytest.raises(AssertionError) as e:
        stats.gate(a, b, frac_max=0.02)
    assert "over_3sigma" in str(e.value)
