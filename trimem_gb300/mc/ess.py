"""Effective sample size of a scalar Markov-chain trace.

Geyer's initial monotone sequence estimator (Geyer 1992, "Practical Markov
chain Monte Carlo", Statist. Sci. 7): with autocorrelations rho_k, the pair
sums Gamma_m = rho_{2m} + rho_{2m+1} are truncated at the first
non-positive one and made non-increasing; tau = -1 + 2 sum_m Gamma_m and
ESS = n / tau.
"""
import numpy as np


def autocorrelation(x):
    """Normalised autocorrelation of a 1-d trace (FFT, biased estimator)."""
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    if n < 2:
        return np.ones(1)
    y = x - x.mean()
    m = 1 << (2 * n - 1).bit_length()
    f = np.fft.rfft(y, m)
    ac = np.fft.irfft(f * np.conj(f), m)[:n]
    if ac[0] <= 0:
        return np.ones(n)
    return ac / ac[0]


def integrated_time(x):
    """Integrated autocorrelation time tau (>= 1/n)."""
    rho = autocorrelation(x)
    n = len(rho)
    gam = []
    for m in range(n // 2):
        g = rho[2 * m] + (rho[2 * m + 1] if 2 * m + 1 < n else 0.0)
        if g <= 0:
            break
        gam.append(g)
    if not gam:
        return 1.0
    gam = np.minimum.accumulate(np.asarray(gam))
    tau = -1.0 + 2.0 * gam.sum()
    return max(tau, 1.0 / n)


def ess(x):
    """Effective sample size of the trace x."""
    x = np.asarray(x, dtype=np.float64)
    if len(x) < 2 or np.all(x == x[0]):
        return float(len(x))
    return len(x) / integrated_time(x)
