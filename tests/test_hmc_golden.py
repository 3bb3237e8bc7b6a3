"""Plain HMC against the reference's golden chain (tests/test_sampling.py of
the reference: seed 42, time_step 0.1, quadratic energy, 10 steps)."""
import json
import os

import numpy as np

from trimem_gb300.mc.hmc import HMC, _vv_integration

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hmc_icosahedron.json")


def test_hmc_matches_reference_chain():
    g = json.load(open(GOLD))
    np.random.seed(42)
    x0 = np.array(g["x0"])
    h = HMC(x0, lambda x: 0.5 * x.ravel().dot(x.ravel()), lambda x: x,
            options={"info_step": 10, "time_step": 1.0e-1})
    h.run(10)
    assert np.linalg.norm(h.x - np.array(g["ref_hmc"])) < 1.0e-14


def test_golden_start_is_unit_icosahedron():
    g = json.load(open(GOLD))
    x0 = np.array(g["x0"])
    assert x0.shape == (12, 3)
    assert np.abs(np.linalg.norm(x0, axis=1) - 1).max() < 1e-12
    d = np.linalg.norm(x0[:, None] - x0[None], axis=2)
    nn = np.sort(d, axis=1)[:, 1:6]
    assert np.ptp(nn) < 1e-12  # five equal nearest neighbours per vertex


def test_vv_integration_is_time_reversible():
    rng = np.random.default_rng(0)
    x0, p0 = rng.normal(size=(5, 3)), rng.normal(size=(5, 3))
    force = lambda x: -x**3
    x1, p1 = _vv_integration(x0, p0, force, 1.0, 0.01, 50)
    x2, p2 = _vv_integration(x1, -p1, force, 1.0, 0.01, 50)
    assert np.allclose(x2, x0, atol=1e-12) and np.allclose(-p2, p0, atol=1e-12)
