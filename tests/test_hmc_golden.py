"""The oracle's HMC restatement against the reference's golden chain
(tests/test_sampling.py of the reference: np.random.seed(42), time step 0.1,
100 velocity-Verlet steps, energy x.x/2, 10 moves from the vertices of an
icosahedron)."""
import json
import os

import numpy as np

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hmc_icosahedron.json")


def test_oracle_hmc_matches_reference_chain():
    g = json.load(open(GOLD))
    np.random.seed(42)
    x, acc = O.hmc_chain(np.array(g["x0"]), lambda x: 0.5 * x.ravel().dot(x.ravel()), lambda x: x,
                         n_steps=10, dt=0.1, n_leapfrog=100)
    assert np.linalg.norm(x - np.array(g["ref_hmc"])) < 1.0e-14
    assert acc == sum(g["accept_pattern"])


def test_golden_start_is_unit_icosahedron():
    g = json.load(open(GOLD))
    x0 = np.array(g["x0"])
    assert x0.shape == (12, 3)
    assert np.abs(np.linalg.norm(x0, axis=1) - 1).max() < 1e-12
    d = np.linalg.norm(x0[:, None] - x0[None], axis=2)
    nn = np.sort(d, axis=1)[:, 1:6]
    assert np.ptp(nn) < 1e-12  # five equal nearest neighbours per vertex


def test_leapfrog_is_time_reversible():
    rng = np.random.default_rng(0)
    x0, p0 = rng.normal(size=(5, 3)), rng.normal(size=(5, 3))
    force = lambda x: -x**3
    x1, p1 = O.leapfrog(x0, p0, force, 1.0, 0.01, 50)
    x2, p2 = O.leapfrog(x1, -p1, force, 1.0, 0.01, 50)
    assert np.allclose(x2, x0, atol=1e-12) and np.allclose(-p2, p0, atol=1e-12)
