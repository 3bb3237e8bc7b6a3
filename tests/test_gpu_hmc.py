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


def test_device_chain_records_the_returned_states(built):
    """The chain driver: properties recorded per step are those of the state
    the HMC move returned; with flip sweeps the mesh stays valid."""
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.device import DeviceChain

    p, f = meshgen.jittered_icosphere(3, seed=2)
    prm = dict(workload_params(p, f), cont_lambda=0.0)
    m = capi.Mesh(p, f)
    e = capi.Energy(m, capi.params(**prm))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    ch = DeviceChain(m, e, x, dt=2e-6, n_leapfrog=5, flip_ratio=0.0, seed=3, refresh=0)
    trace = ch.run(6)
    assert ch.accepted > 0
    m.points()[:] = x.cpu().numpy()
    np.testing.assert_allclose(trace[-1], e.properties(m)[:6], rtol=1e-12)
    ch2 = DeviceChain(m, e, x, dt=2e-6, n_leapfrog=5, flip_ratio=0.2, seed=4, refresh=1)
    ch2.run(4)
    assert ch2.flips > 0 and m.check() == 0
