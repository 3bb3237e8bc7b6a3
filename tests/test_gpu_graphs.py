"""Evaluations replayed from captured CUDA graphs.

tm_energy_eval_device issues its launches as a captured graph (in each
stencil precision), re-captured whenever what the launches depend on
changes (buffers, parameters, the neighbour list).  tm_energy_eval_timed issues the same kernels one by one
(the repulsion pass in sequence instead of on the second stream).  Both must
give the same gradient bit for bit, across replays with new positions in
the same buffer, alternating output buffers, energy-only calls, neighbour
list rebuilds and a change of the reference properties.
"""
import ctypes

import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("stencil", [0, 1, 2])  # FP64, FP32, double-float
def test_graph_replays_match_direct_launches(built, stencil):
    import torch

    from trimem_gb300 import capi

    L = capi.lib()
    p, f = meshgen.jittered_icosphere(5, seed=3)  # 10,242 vertices
    prm = dict(workload_params(p, f), cont_lambda=0.5, cont_delta=0.1)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    capi.check(L.tm_energy_set_stencil_precision(en.h, stencil))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    gen = torch.Generator(device="cuda").manual_seed(1)
    bufs = [torch.empty_like(x), torch.empty_like(x)]
    g_direct = torch.empty_like(x)
    e_dev = torch.empty(1, dtype=torch.float64, device="cuda")
    ms5 = (ctypes.c_float * 5)()
    seen = []
    for it in range(8):
        x += 1e-4 * torch.randn(x.shape, device="cuda", dtype=torch.float64, generator=gen)
        if it in (3, 6):  # rebuilt neighbour list (new cells; near rows kept or rebuilt)
            capi.check(L.tm_energy_update_repulsion_device(en.h, mesh.h, _ptr(x), None))
        if it == 5:  # new reference properties: new penalty parameters in the launches
            capi.check(L.tm_energy_update_reference_properties(en.h))
        # an energy-only call between the gradient calls
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, _ptr(x), None, _ptr(e_dev), None))
        torch.cuda.synchronize()
        e_only = float(e_dev.item())
        g = bufs[it % 2]
        g.fill_(float("nan"))
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, _ptr(x), _ptr(g), _ptr(e_dev), None))
        torch.cuda.synchronize()
        e_graph = float(e_dev.item())
        capi.check(L.tm_energy_eval_timed(en.h, mesh.h, _ptr(x), _ptr(g_direct), ms5, None))
        torch.cuda.synchronize()
        assert torch.equal(g, g_direct), it
        assert e_only == e_graph, it
        seen.append(e_graph)
    assert np.all(np.isfinite(seen)) and len(set(seen)) == len(seen)


def test_graph_replays_on_other_streams(built):
    """A graph captured on one stream replays on another: alternating
    streams give the results of the direct launches."""
    import torch

    from trimem_gb300 import capi

    L = capi.lib()
    p, f = meshgen.jittered_icosphere(4, seed=5)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**workload_params(p, f)))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    g, g_direct = torch.empty_like(x), torch.empty_like(x)
    ms5 = (ctypes.c_float * 5)()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    for it in range(4):
        x += 1e-4 * (it + 1) * torch.ones_like(x)
        st = streams[it % 2]
        st.wait_stream(torch.cuda.current_stream())
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, _ptr(x), _ptr(g), None, ctypes.c_void_p(st.cuda_stream)))
        torch.cuda.synchronize()
        capi.check(L.tm_energy_eval_timed(en.h, mesh.h, _ptr(x), _ptr(g_direct), ms5, None))
        torch.cuda.synchronize()
        assert torch.equal(g, g_direct), it
