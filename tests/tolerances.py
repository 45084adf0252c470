"""Parity rules shared by the GPU tests.

* coefficients within COEF_TOL (1e-5) absolute of the reference / oracle;
* lags identical except where the FP64 top-two peaks differ by less than
  GAP_TOL (1e-6) -- the two lags are then a tie at FP32 resolution;
* pairs whose FP64 coefficient is within COEF_TOL of +-threshold may flip
  between zero and non-zero;
* histogram counts may move between adjacent bins only for values within
  COEF_TOL of a bin edge.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O

COEF_TOL = 1e-5
GAP_TOL = 1e-6


def check_pairs(got, exp, fp64: "O.Fp64Result", threshold: float, tol: float = COEF_TOL,
                gap_tol: float = GAP_TOL, label: str = ""):
    """got/exp: (vals_pos, lags_pos, vals_neg, lags_neg) packed arrays."""
    gvp, glp, gvn, gln = (np.asarray(x) for x in got)
    evp, elp, evn, eln = (np.asarray(x) for x in exp)
    near_thr_p = np.abs(fp64.val_pos - threshold) < tol
    near_thr_n = np.abs(fp64.val_neg + threshold) < tol
    dp = np.abs(gvp.astype(np.float64) - evp)
    dn = np.abs(gvn.astype(np.float64) - evn)
    bad_p = (dp > tol) & ~near_thr_p
    bad_n = (dn > tol) & ~near_thr_n
    assert not bad_p.any(), f"{label} vals_pos off by {dp[bad_p].max():.3g} at {np.flatnonzero(bad_p)[:8]}"
    assert not bad_n.any(), f"{label} vals_neg off by {dn[bad_n].max():.3g} at {np.flatnonzero(bad_n)[:8]}"
    lag_bad_p = (glp != elp) & (fp64.gap_pos >= gap_tol) & ~near_thr_p
    lag_bad_n = (gln != eln) & (fp64.gap_neg >= gap_tol) & ~near_thr_n
    assert not lag_bad_p.any(), f"{label} lags_pos differ at {np.flatnonzero(lag_bad_p)[:8]}"
    assert not lag_bad_n.any(), f"{label} lags_neg differ at {np.flatnonzero(lag_bad_n)[:8]}"
    return dict(max_err=float(max(dp.max(initial=0), dn.max(initial=0))),
                lag_mismatch=int(((glp != elp) | (gln != eln)).sum()))


def check_hist(got_max, got_min, exp_max, exp_min, fp64: "O.Fp64Result", n_hist: int,
               tol: float = COEF_TOL):
    delta = 1.0 / n_hist
    for got, exp, vals in ((got_max, exp_max, fp64.val_pos), (got_min, exp_min, -fp64.val_neg)):
        got = np.asarray(got, np.int64)
        exp = np.asarray(exp, np.int64)
        assert got.sum() == exp.sum(), f"histogram totals differ: {got.sum()} vs {exp.sum()}"
        frac = vals / delta
        near_edge = np.abs(frac - np.round(frac)) * delta < tol
        allowed = int(near_edge.sum())
        assert np.abs(got - exp).sum() <= 2 * allowed, (
            f"histograms differ beyond edge cases: {got} vs {exp} (allowed moves {allowed})")
