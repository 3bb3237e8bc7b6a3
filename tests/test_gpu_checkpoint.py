"""Checkpoints of device chains: a chain saved after some steps and loaded
into fresh handles continues bit for bit like the original (positions,
flipped topology with its edge numbering, reference properties, continuation
state, random generator); the topology setter rejects arrays that do not
describe a valid mesh before anything changes."""
import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def test_chain_checkpoint_resumes_bit_for_bit(built, tmp_path):
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.device import DeviceChain
    from trimem_gb300.mc.output import load_chain, save_chain

    p, f = meshgen.jittered_icosphere(3, seed=9)
    prm = dict(workload_params(p, f), cont_lambda=0.5, cont_delta=0.2)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    en.update_reference_properties()  # continuation state differs from the constructor's
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    ch = DeviceChain(mesh, en, x, dt=1e-6, n_leapfrog=5, flip_ratio=0.3, flip_batch=256, seed=21)
    ch.run(4)
    assert ch.flips > 0  # the topology (and edge numbering) has changed
    path = tmp_path / "chain.npz"
    save_chain(path, ch)
    trace_a = ch.run(4)
    xa, topo_a = ch.x.cpu().numpy(), mesh.topology()

    ch2, mesh2, en2 = load_chain(path)
    assert np.array_equal(en2.initial_props(), en.initial_props())
    assert en2.params().cont_lambda == en.params().cont_lambda
    trace_b = ch2.run(4)
    assert np.array_equal(trace_a, trace_b)
    assert np.array_equal(ch2.x.cpu().numpy(), xa)
    topo_b = mesh2.topology()
    for k in topo_a:
        assert np.array_equal(topo_a[k], topo_b[k]), k
    assert (ch2.accepted, ch2.flips, ch2.step_index) == (ch.accepted, ch.flips, ch.step_index)


def test_set_topology_validates(built):
    from trimem_gb300 import capi

    p, f = meshgen.icosphere(2)
    mesh = capi.Mesh(p, f)
    topo = mesh.topology()
    bad = {k: v.copy() for k, v in topo.items()}
    bad["next"][5] = len(bad["next"])  # out of range
    with pytest.raises(capi.TMError):
        mesh.set_topology(bad)
    bad = {k: v.copy() for k, v in topo.items()}
    bad["next"][0], bad["next"][1] = bad["next"][1], bad["next"][0]  # no longer triangles
    with pytest.raises(capi.TMError):
        mesh.set_topology(bad)
    assert mesh.check() == 0
    after = mesh.topology()
    for k in topo:  # rejected arrays left the mesh unchanged
        assert np.array_equal(after[k], topo[k]), k
    mesh.set_topology(topo)  # the mesh's own arrays are accepted
    assert mesh.check() == 0
