"""ESS estimator against the closed form of an AR(1) process."""
import numpy as np

from trimem_gb300.mc.ess import ess, integrated_time


def ar1(n, phi, seed):
    rng = np.random.default_rng(seed)
    x = np.empty(n)
    x[0] = rng.normal() / np.sqrt(1 - phi**2)
    e = rng.normal(size=n)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + e[i]
    return x


def test_iid_trace_has_ess_near_n():
    x = np.random.default_rng(0).normal(size=20000)
    assert 0.85 < ess(x) / len(x) < 1.15


def test_ar1_integrated_time():
    for phi in (0.5, 0.9):
        taus = [integrated_time(ar1(40000, phi, s)) for s in range(4)]
        exact = (1 + phi) / (1 - phi)
        assert abs(np.mean(taus) - exact) / exact < 0.1


def test_constant_trace():
    assert ess(np.ones(10)) == 10


def _ar1(n, phi, seed):
    rng = np.random.default_rng(seed)
    x = np.empty(n)
    x[0] = rng.normal() / np.sqrt(1 - phi * phi)
    for i in range(1, n):
        x[i] = phi * x[i - 1] + rng.normal()
    return x


def test_drift_check_passes_stationary_and_flags_trending_traces():
    """bench.py's stationarity test of a chain trace (first against last
    quarter mean over their ESS-based standard errors): stationary AR(1)
    traces pass at the usual rate, a trend of a few standard deviations
    over the trace is flagged."""
    import bench

    passed = [bench.drift_check(_ar1(2000, 0.9, s))["stationary"] for s in range(40)]
    assert np.mean(passed) >= 0.85
    x = _ar1(2000, 0.9, 7) + np.linspace(0.0, 8.0, 2000)  # ~3.5 sd of the stationary trace
    d = bench.drift_check(x)
    assert not d["stationary"] and d["z"] > 3.0
