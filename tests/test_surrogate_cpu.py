"""Host side of the learned surrogate (no GPU): the weight blob that
tm_surrogate_create parses round-trips, and the torch reference network's
bf16 emulation stays close to its FP32 form."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from trimem_gb300 import surrogate as S  # noqa: E402


def _net(seed):
    torch.manual_seed(seed)
    net = S.make_net()
    with torch.no_grad():
        net.wo.normal_(0, 0.3)
        net.wn.normal_(0, 0.3)
        net.scales.copy_(torch.tensor([0.01, 1e-4, 50.0]))
    return net


def test_blob_round_trip():
    net = _net(0)
    b = S.to_blob(net)
    assert b.dtype == np.float32 and b.size == S.BLOB_SIZE == 26442
    assert list(b[:5]) == [1.0, S.FV, S.FE, S.H, S.NR]
    b2 = S.to_blob(S.from_blob(b))
    assert np.array_equal(b, b2)


class _Inputs:
    pass


def _random_inputs(nv=300, d=6, seed=1):
    g = torch.Generator().manual_seed(seed)
    inp = _Inputs()
    inp.u = torch.randn(nv, S.FV, generator=g)
    inp.nrm = torch.randn(nv, 4, generator=g)
    nbr = torch.stack([torch.randperm(nv, generator=g) for _ in range(d)])
    nbr[d - 1, ::3] = -1  # ragged rings
    inp.nbr = nbr
    valid = (nbr >= 0)[..., None]
    inp.ef = torch.randn(d, nv, S.FE, generator=g) * valid
    inp.dirs = torch.randn(d, nv, 3, generator=g) * valid
    return inp


def test_bf16_emulation_stays_close():
    net = _net(3)
    inp = _random_inputs(seed=4)
    with torch.no_grad():
        f32 = net(inp.u, inp.nrm, inp.nbr, inp.ef, inp.dirs)
        f16 = net(inp.u, inp.nrm, inp.nbr, inp.ef, inp.dirs, bf16=True)
    assert float((f32 - f16).norm() / f32.norm()) < 5e-2
