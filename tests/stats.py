"""Batch-means comparison of two Monte Carlo estimators (the 3-sigma gate).

Each engine runs B independent batches; per pixel the batch means give a
mean and a standard error, and z = (mean_a - mean_b) / sqrt(se_a^2 + se_b^2).
With standard errors estimated from B batches, z follows Student's t with
about 2B-2 degrees of freedom under the null hypothesis; the 3-sigma gate is
applied at the matching tail probability (0.27 %, two-sided), i.e. a pixel
fails when |z| exceeds the t quantile of that probability.

The gate then holds the number of failing pixels to what chance allows: at
most the count a binomial(n, 0.27 %) variable exceeds with probability 1e-4
(and at most frac_max of the pixels), with the mean of z^2 near its null
value.  For an image whose pixels are independent under the null hypothesis
(reflectance and transmittance: a photon leaves through one pixel at most),
the failing pixels must not cluster: the count of failing pixel pairs that
are neighbours along x or y is held to the Poisson(1e-4) bound for its
expectation under independence.
"""
import numpy as np
from scipy import stats as _st


P_TAIL = 0.0027   # two-sided tail probability of |z| > 3 for a normal z
P_CHANCE = 1e-4   # probability that a correct engine fails one gate by chance


def zscores(a: np.ndarray, b: np.ndarray, min_rel: float = 1e-3, full: bool = False):
    """a, b: (B, n) arrays of per-batch tallies.  Pixels whose mean is below
    min_rel of the maximum mean, or whose spread is zero, are skipped (NaN in
    the full-length array returned when full is set)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ma, mb = a.mean(0), b.mean(0)
    va, vb = a.var(0, ddof=1) / a.shape[0], b.var(0, ddof=1) / b.shape[0]
    peak = max(ma.max(), mb.max())
    keep = (va + vb > 0) & (np.maximum(ma, mb) >= min_rel * peak)
    z = (ma[keep] - mb[keep]) / np.sqrt(va[keep] + vb[keep])
    if full:
        zf = np.full(ma.shape, np.nan)
        zf[keep] = z
        return zf
    return z


def neighbour_pairs(over: np.ndarray, valid: np.ndarray):
    """Failing pixel pairs that are neighbours along x or y, and the number
    of neighbour pairs of compared pixels, on a (ny, nx) image."""
    hits = int(np.sum(over[:, 1:] & over[:, :-1]) + np.sum(over[1:, :] & over[:-1, :]))
    pairs = int(np.sum(valid[:, 1:] & valid[:, :-1]) + np.sum(valid[1:, :] & valid[:-1, :]))
    return hits, pairs


def gate(a, b, frac_max=0.01, min_pixels=10, min_rel=1e-3, shape=None):
    """Asserts the 3-sigma agreement; returns a summary dict.  shape: (ny, nx)
    of an image whose pixels are independent under the null hypothesis, for
    the clustering test."""
    zf = zscores(a, b, min_rel, full=True)
    valid = ~np.isnan(zf)
    z = zf[valid]
    assert z.size >= min_pixels, f"only {z.size} pixels to compare"
    df = max(2, np.asarray(a).shape[0] + np.asarray(b).shape[0] - 2)
    thr = float(_st.t.isf(P_TAIL / 2, df))  # the t counterpart of |z| > 3
    n_over = int(np.sum(np.abs(z) > thr))
    allowed = int(min(_st.binom.ppf(1 - P_CHANCE, z.size, P_TAIL), np.floor(frac_max * z.size)))
    m2 = float(np.mean(z * z))
    expect_m2 = df / (df - 2) if df > 2 else 3.0
    summary = {"pixels": int(z.size), "df": int(df), "threshold": thr, "over_3sigma": n_over,
               "allowed_over": allowed, "frac_over_3sigma": n_over / z.size, "mean_z2": m2,
               "expected_mean_z2": expect_m2, "max_abs_z": float(np.abs(z).max())}
    if shape is not None:
        over = np.zeros(zf.shape, dtype=bool)
        over[valid] = np.abs(zf[valid]) > thr
        hits, pairs = neighbour_pairs(over.reshape(shape), valid.reshape(shape))
        p = max(n_over / z.size, P_TAIL)
        summary.update(neighbour_pairs_over=hits,
                       neighbour_pairs_allowed=int(_st.poisson.ppf(1 - P_CHANCE, max(pairs * p * p, 1e-9))))
        assert hits <= summary["neighbour_pairs_allowed"], summary
    assert n_over <= allowed, summary
    assert m2 < 1.5 * expect_m2, summary
    return summary


def scalar_gate(a, b, rel_tol=None):
    """Integrated quantity: within 3 sigma, and within rel_tol relative when
    given.  a, b: per-batch values."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    se = np.sqrt(a.var(ddof=1) / a.size + b.var(ddof=1) / b.size)
    d = abs(a.mean() - b.mean())
    out = {"a": float(a.mean()), "b": float(b.mean()), "sigma": float(se), "rel_diff": float(d / abs(b.mean()))}
    assert d <= 3 * se + 1e-300, out
    if rel_tol is not None:
        assert d / abs(b.mean()) <= rel_tol, out
    return out
