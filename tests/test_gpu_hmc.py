"""Device-resident HMC step (velocity Verlet + exact Metropolis on the GPU)."""
import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def test_device_hmc_step_conserves_energy_and_is_reversible(built):
    import torch

    from trimem_gb300 import load_core

    m = load_core()
    p, f = meshgen.jittered_icosphere(4, seed=0)
    prm = workload_params(p, f)
    mesh = m.TriMesh(p, f)
    ep = m.EnergyParams()
    ep.kappa_b, ep.kappa_a, ep.kappa_v, ep.kappa_t, ep.kappa_r = 30.0, 1e6, 1e6, 1e5, 1e3
    ep.volume_frac = 0.8
    ep.bond_params.lc0, ep.bond_params.lc1 = prm["bond_lc0"], prm["bond_lc1"]
    ep.repulse_params.lc1 = ep.repulse_params.rlist = prm["rep_lc1"]
    estore = m.EnergyManager(mesh, ep)
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    dts = []
    for dt in (2e-6, 1e-6):
        xs = x.clone()
        acc, h0, h1, e = estore.hmc_step_device(mesh, xs.data_ptr(), 1.0, dt, 10, 1.0, 5, 0, 0.0)
        dts.append(abs(h1 - h0))
    # second-order integrator: halving dt divides |dH| by about four
    assert dts[1] < dts[0] / 2.5
    # the energy of the returned state is the manager's energy there
    xs = x.clone()
    acc, h0, h1, e = estore.hmc_step_device(mesh, xs.data_ptr(), 1.0, 1e-6, 5, 1.0, 6, 0, 0.0)
    assert acc
    mesh.points()[:] = xs.cpu().numpy()
    assert e == pytest.approx(estore.energy(mesh), rel=1e-12)
    # rejected steps leave the state unchanged
    xs = x.clone()
    acc, h0, h1, e = estore.hmc_step_device(mesh, xs.data_ptr(), 1.0, 1e-3, 5, 1.0, 7, 0, 1.0 - 1e-16)
    if not acc:
        assert torch.equal(xs, x)
