"""Device L-BFGS against the reference's route (scipy L-BFGS-B over the
energy and gradient, neighbour list refreshed every evaluation): both reach
the same minimum energy from the same start."""
import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def test_device_lbfgs_reaches_the_scipy_minimum(built):
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.minim import minimize_device, minimize_scipy

    p, f = meshgen.jittered_icosphere(3, seed=8)
    prm = dict(workload_params(p, f, kappa_b=20.0), cont_lambda=0.0, kappa_a=1e3, kappa_v=1e3, kappa_t=10.0)
    m1 = capi.Mesh(p, f)
    e1 = capi.Energy(m1, capi.params(**prm))
    e0 = e1.energy(m1)
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    it_d, E_d = minimize_device(e1, m1, x, maxiter=3000)
    m2 = capi.Mesh(p, f)
    e2 = capi.Energy(m2, capi.params(**prm))
    it_s, E_s = minimize_scipy(e2, m2, maxiter=3000)
    assert E_d < 0.5 * e0 and E_s < 0.5 * e0
    assert abs(E_d - E_s) <= 1e-4 * abs(E_s), (E_d, E_s, it_d, it_s)
    # the returned energy is the manager's energy at the returned positions
    m1.points()[:] = x.cpu().numpy()
    e1.update_repulsion(m1)
    assert e1.energy(m1) == pytest.approx(E_d, rel=1e-12)
