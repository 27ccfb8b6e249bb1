"""Effective-sample-size estimators for the energy series (no counterpart in the reference,
which reports standard errors over walkers only, kernel.py:615-616).

series[t, w]: measurement t of walker w, t in run order.  The integrated autocorrelation
time uses Sokal's automatic window (the smallest M with M >= c * tau(M), c = 5) on the
autocorrelation averaged over walkers; batch means give an independent cross-check.
"""
from __future__ import annotations

import numpy as np


def autocorrelation(series, max_lag=None):
    x = np.asarray(series, dtype=np.float64)
    x = x - x.mean(axis=0, keepdims=True)
    T = x.shape[0]
    max_lag = T // 2 if max_lag is None else min(max_lag, T - 1)
    var = (x * x).mean()
    if var <= 0:
        return np.ones(1)
    return np.array([(x[:T - t] * x[t:]).mean() / var for t in range(max_lag + 1)])


def tau_int_sokal(series, c=5.0):
    rho = autocorrelation(series)
    tau = 0.5
    for M in range(1, len(rho)):
        tau += rho[M]
        if M >= c * tau:
            return max(tau, 0.5), M
    return max(tau, 0.5), len(rho) - 1


def tau_int_batch_means(series, n_batches=8):
    x = np.asarray(series, dtype=np.float64)
    T = (x.shape[0] // n_batches) * n_batches
    if T < n_batches * 2:
        return float("nan")
    x = x[:T]
    b = x.reshape(n_batches, T // n_batches, -1).mean(axis=1)
    var_b = b.var(axis=0, ddof=1).mean()
    var = x.var(axis=0, ddof=1).mean()
    return 0.5 * (T // n_batches) * var_b / var if var > 0 else float("nan")


def ess(series, c=5.0):
    """Effective samples in series[t, w] (all walkers)."""
    tau, _ = tau_int_sokal(series, c)
    return series.shape[0] * series.shape[1] / (2.0 * tau), tau
