"""The allocation-free evaluation entry point.

tm_energy_eval_device_noalloc serves callers that must not allocate device
memory while they evaluate (a host running under someone else's memory
budget, or one that must stay out of the CUDA allocator while other streams
are busy): its scratch is a fixed device array compiled into the library.
It must give the same energy and gradient as tm_energy_eval_device, call
after call, and refuse meshes whose scratch would not fit.
"""
import ctypes

import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_matches_allocating_entry_point(built):
    import torch

    from trimem_gb300 import capi

    L = capi.lib()
    p, f = meshgen.jittered_icosphere(5, seed=11)  # 10,242 vertices
    prm = workload_params(p, f, excl=1, rep_scale=1.2)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    g_ref = torch.empty_like(x)
    e_ref = torch.empty(1, dtype=torch.float64, device="cuda")
    capi.check(L.tm_energy_eval_device(en.h, mesh.h, _ptr(x), _ptr(g_ref), _ptr(e_ref), None))
    torch.cuda.synchronize()
    # the oracle (the reference algorithm on the host) at the same state
    from oracle import oracle as O

    mo = O.Mesh(p, f)
    eo = O.Energy(mo, O.default_params(**prm))
    e_or, g_or = eo.energy(mo), eo.gradient(mo)
    outs = [(torch.full_like(x, float("nan")), torch.full((1,), float("nan"), dtype=torch.float64, device="cuda"))
            for _ in range(2)]
    # warm-up call: the first one on a device looks up the array's address
    capi.check(L.tm_energy_eval_device_noalloc(en.h, mesh.h, _ptr(x), _ptr(outs[0][0]), _ptr(outs[0][1]), None))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2):  # the shared scratch keeps the previous call's data
        g, e = outs[call]
        g.fill_(float("nan"))
        e.fill_(float("nan"))
        capi.check(L.tm_energy_eval_device_noalloc(en.h, mesh.h, _ptr(x), _ptr(g), _ptr(e), None))
        torch.cuda.synchronize()
    # the two calls allocated no device memory: the driver's free-memory count
    # is unchanged (no cudaMalloc, no allocating library routine; the checks
    # below, which do allocate, come after)
    assert torch.cuda.mem_get_info()[0] == free0
    for call, (g, e) in enumerate(outs):
        er, eg = float(e_ref.item()), float(e.item())
        assert abs(eg - er) <= 1e-10 * abs(er), (call, eg, er)
        rel = float(torch.linalg.norm(g - g_ref) / torch.linalg.norm(g_ref))
        assert rel < 1e-10, (call, rel)
        assert abs(eg - e_or) <= 1e-10 * abs(e_or), (call, eg, e_or)
        rel_or = np.linalg.norm(g.cpu().numpy() - g_or) / np.linalg.norm(g_or)
        assert rel_or < 1e-10, (call, rel_or)


def test_noalloc_rejects_meshes_above_its_scratch(built):
    import torch

    from trimem_gb300 import capi

    L = capi.lib()
    p, f = meshgen.icosphere(7)  # 163,842 vertices: needs about 62 MB of scratch
    prm = workload_params(p, f)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    g = torch.empty_like(x)
    rc = L.tm_energy_eval_device_noalloc(en.h, mesh.h, _ptr(x), _ptr(g), None, None)
    assert rc == capi.TM_ERR_ARG
    assert b"scratch" in L.tm_last_error()
