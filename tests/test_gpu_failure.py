"""Failure detection on the GPU without a fault: a bounded device wait that
runs out is reported to the host as TM_ERR_TIMEOUT, and the CUDA context
stays usable.

The tensor-core layer of the surrogate waits twice on mbarriers (its TMA
tile loads, then the tcgen05 MMA completion).  With a poll limit of zero the
first wait gives up at once; the kernel records the status, lets its own
copies land, frees its tensor memory and returns."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _layer(torch):
    gen = torch.Generator(device="cuda").manual_seed(3)
    h = torch.randn(300, 64, device="cuda", generator=gen).to(torch.bfloat16)
    m = torch.randn(300, 64, device="cuda", generator=gen).to(torch.bfloat16)
    w = (0.1 * torch.randn(64, 128, device="cuda", generator=gen)).to(torch.bfloat16)
    b = 0.1 * torch.randn(64, device="cuda", generator=gen)
    return h, m, w, b


def test_wait_that_runs_out_reports_timeout_and_the_context_survives(built):
    import torch

    from trimem_gb300 import capi

    L = capi.lib()
    h, m, w, b = _layer(torch)
    o = torch.zeros(300, 64, device="cuda", dtype=torch.bfloat16)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = L.tm_dense_silu_bf16_bounded(P(h), P(m), P(w), P(b), P(o), 300, 0, None)
    assert rc == capi.TM_ERR_TIMEOUT, rc
    assert b"timed out" in L.tm_last_error()
    # nothing was written for the rows whose wait gave up
    assert int(torch.count_nonzero(o)) == 0
    # a negative limit is an argument error
    assert L.tm_dense_silu_bf16_bounded(P(h), P(m), P(w), P(b), P(o), 300, -1, None) == capi.TM_ERR_ARG
    # the context is usable: the same layer with the default limit is right
    capi.check(L.tm_dense_silu_bf16(P(h), P(m), P(w), P(b), P(o), 300, None))
    torch.cuda.synchronize()
    ref = h.float() + torch.nn.functional.silu(torch.cat([h, m], 1).float() @ w.float().t() + b)
    err = float(((o.float() - ref).abs() / ref.abs().clamp(min=1.0)).max())
    assert err <= 2 * 2.0 ** -8, err
