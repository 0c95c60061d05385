"""Batch-means comparison of two Monte Carlo estimators (the 3-sigma gate).

Each engine runs B independent batches; per pixel the batch means give a
mean and a standard error, and z = (mean_a - mean_b) / sqrt(se_a^2 + se_b^2).
With standard errors estimated from B batches, z follows Student's t with
about 2B-2 degrees of freedom under the null hypothesis; the 3-sigma gate is
applied at the matching tail probability (0.27 %, two-sided), i.e. a pixel
fails when |z| exceeds the t quantile of that probability.
"""
import numpy as np
from scipy import stats as _st


def zscores(a: np.ndarray, b: np.ndarray, min_rel: float = 1e-3):
    """a, b: (B, n) arrays of per-batch tallies.  Pixels whose mean is below
    min_rel of the maximum mean, or whose spread is zero, are skipped."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ma, mb = a.mean(0), b.mean(0)
    va, vb = a.var(0, ddof=1) / a.shape[0], b.var(0, ddof=1) / b.shape[0]
    peak = max(ma.max(), mb.max())
    keep = (va + vb > 0) & (np.maximum(ma, mb) >= min_rel * peak)
    z = (ma[keep] - mb[keep]) / np.sqrt(va[keep] + vb[keep])
    return z


def gate(a, b, frac_max=0.01, min_pixels=10, min_rel=1e-3):
    """Asserts the 3-sigma agreement; returns a summary dict."""
    z = zscores(a, b, min_rel)
    assert z.size >= min_pixels, f"only {z.size} pixels to compare"
    df = max(2, np.asarray(a).shape[0] + np.asarray(b).shape[0] - 2)
    thr = float(_st.t.isf(0.0027 / 2, df))  # the t counterpart of |z| > 3
    over = float(np.mean(np.abs(z) > thr))
    m2 = float(np.mean(z * z))
    expect_m2 = df / (df - 2) if df > 2 else 3.0
    summary = {"pixels": int(z.size), "df": int(df), "threshold": thr, "frac_over_3sigma": over, "mean_z2": m2,
               "expected_mean_z2": expect_m2, "max_abs_z": float(np.abs(z).max())}
    assert over <= frac_max, summary
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
