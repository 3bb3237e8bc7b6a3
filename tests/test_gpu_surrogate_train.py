"""Training kernels of the learned surrogate (tm_surrogate_train_*) against a
CPU reference: the same network in torch, float64 on the host, with the
CUDA forward's bf16 roundings of activations and dense weights emulated and
differentiated straight through, its gradients by autograd.

Tolerances: loss within 1e-3 relative, forces and every parameter group's
gradient within 2e-2 relative (norm-wise): bf16 activations through three
rounds, where an FP32 pre-activation can round to the neighbouring bf16
value of the float64 one.  Adam's update is checked to float rounding, and
a few steps on chain states must lower the loss."""
import ctypes

import numpy as np
import pytest

from helpers import workload_params
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _state(seed=3, level=3):
    import torch

    from trimem_gb300 import capi
    from trimem_gb300 import surrogate as S

    p, f = meshgen.jittered_icosphere(level, seed=seed)
    prm = dict(workload_params(p, f, kappa_b=20.0), cont_lambda=0.0)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    torch.manual_seed(seed)
    net = S.make_net()
    lbar, abar = S.mesh_scales(p, f)
    with torch.no_grad():
        net.scales.copy_(torch.tensor([lbar, abar, 30.0]))
        net.wo.normal_(0, 0.3)
        net.wn.normal_(0, 0.3)
    blob = S.to_blob(net)
    sg = capi.Surrogate(mesh, blob)
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    inp = S.Inputs(sg, en, mesh, x, 16)
    g = torch.empty_like(x)
    capi.check(capi.lib().tm_energy_eval_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()),
                                                ctypes.c_void_p(g.data_ptr()), None, None))
    torch.cuda.synchronize()
    inp.target = (inp.gloc - g).float().contiguous()
    return mesh, en, x, sg, inp, blob


def cpu_reference(blob, inp, rms):
    """(loss, force, gradient in blob order without the header) of the
    network on the host in float64, bf16 roundings emulated."""
    import torch

    from trimem_gb300 import surrogate as S

    b = torch.tensor(np.asarray(blob[S.BLOB_HEADER:], np.float64), requires_grad=True)
    q = [0]

    def take(*shape):
        n = int(np.prod(shape))
        t = b[q[0]:q[0] + n].reshape(shape)
        q[0] += n
        return t

    win, bin_ = take(S.H, S.FV), take(S.H)
    rounds = [(take(S.H, S.FE), take(S.H), take(S.H, 2 * S.H), take(S.H)) for _ in range(S.NR)]
    wo, bo, wn, bn = take(S.H), take(1)[0], take(S.H), take(1)[0]
    fs = float(blob[7])
    cpu = lambda t: t.detach().cpu().double()
    u, nrm, ef, dirs, T = cpu(inp.u), cpu(inp.nrm), cpu(inp.ef), cpu(inp.dirs), cpu(inp.target)
    nbr = inp.nbr.cpu().long()
    rnd = lambda t: t.to(torch.bfloat16).to(torch.float64)
    silu = torch.nn.functional.silu
    mask = (nbr >= 0).double()
    idx = nbr.clamp(min=0)
    h = rnd(silu(u @ win.t() + bin_))
    for we, be, W, bd in rounds:
        gate = ef @ we.t() + be
        m = rnd((mask[..., None] * gate * h[idx]).sum(0))
        h = rnd(h + silu(torch.cat([h, m], 1) @ rnd(W).t() + bd))
    c = ((h[None] * h[idx]) * wo).sum(-1) + bo
    c = c * mask
    cn = h @ wn + bn
    F = fs * ((c[..., None] * dirs).sum(0) + cn[:, None] * nrm[:, :3])
    loss = ((F - T) ** 2).sum() / (3 * F.shape[0] * rms * rms)
    loss.backward()
    return float(loss), F.detach().numpy(), b.grad.numpy()


def groups():
    from trimem_gb300 import surrogate as S

    H, FV, FE = S.H, S.FV, S.FE
    out, o = [("W_in", H * FV), ("b_in", H)], []
    for r in range(S.NR):
        out += [(f"W_e{r}", H * FE), (f"b_e{r}", H), (f"W{r}", 2 * H * H), (f"b{r}", H)]
    out += [("w_o", H), ("b_o", 1), ("w_n", H), ("b_n", 1)]
    k = 0
    for name, n in out:
        o.append((name, k, k + n))
        k += n
    return o


def test_training_gradient_matches_the_cpu_reference(built):
    from trimem_gb300 import surrogate as S

    _, _, _, _, inp, blob = _state()
    rms = float((inp.target ** 2).mean().sqrt())
    tr = S.DeviceTrainer(inp.u.shape[0], inp.D, blob)
    loss, F, g = tr.grad(inp, rms)
    loss2, _, g2 = tr.grad(inp, rms)
    assert loss2 == loss and bool((g2 == g).all())  # fixed-order reductions: bit-reproducible
    l_ref, F_ref, g_ref = cpu_reference(blob, inp, rms)
    assert abs(loss - l_ref) <= 1e-3 * abs(l_ref), (loss, l_ref)
    F = F.cpu().numpy()
    assert np.linalg.norm(F - F_ref) <= 2e-2 * np.linalg.norm(F_ref)
    g = g.cpu().numpy()
    for name, a, b in groups():
        err = np.linalg.norm(g[a:b] - g_ref[a:b]) / max(np.linalg.norm(g_ref[a:b]), 1e-30)
        assert err < 2e-2, (name, err)


def test_adam_step_applies_the_update_rule(built):
    from trimem_gb300 import surrogate as S

    _, _, _, _, inp, blob = _state(seed=5)
    rms = float((inp.target ** 2).mean().sqrt())
    tr = S.DeviceTrainer(inp.u.shape[0], inp.D, blob)
    _, _, g = tr.grad(inp, rms)
    g = g.cpu().numpy().astype(np.float64)
    lr, b1, b2, eps = 1e-3, 0.9, 0.999, 1e-8
    tr.step(inp, rms, lr=lr, beta1=b1, beta2=b2, eps=eps)
    w = tr.weights()
    m = (1 - b1) * g / (1 - b1)
    v = (1 - b2) * g * g / (1 - b2)
    want = blob[S.BLOB_HEADER:].astype(np.float64) - lr * m / (np.sqrt(v) + eps)
    assert np.allclose(w[S.BLOB_HEADER:], want, rtol=1e-5, atol=1e-7)
    assert np.array_equal(w[:S.BLOB_HEADER], blob[:S.BLOB_HEADER])


def test_training_steps_lower_the_loss(built):
    import torch

    from trimem_gb300 import surrogate as S
    from trimem_gb300.mc.device import DeviceChain

    mesh, en, x, sg, inp, blob = _state(seed=7)
    states = [inp]
    ch = DeviceChain(mesh, en, x, dt=1e-6, n_leapfrog=5, flip_ratio=0.0, seed=1, refresh=0)
    g = torch.empty_like(x)
    from trimem_gb300 import capi

    for _ in range(3):
        ch.run(2)
        d = S.Inputs(sg, en, mesh, x, 16)
        capi.check(capi.lib().tm_energy_eval_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()),
                                                    ctypes.c_void_p(g.data_ptr()), None, None))
        torch.cuda.synchronize()
        d.target = (d.gloc - g).float().contiguous()
        states.append(d)
    rms = float(torch.sqrt(torch.stack([(d.target ** 2).mean() for d in states]).mean()))
    D = max(d.D for d in states)
    tr = S.DeviceTrainer(inp.u.shape[0], D, blob)
    before = np.mean([tr.grad(d, rms, want_grad=False)[0] for d in states])
    for it in range(60):
        tr.step(states[it % len(states)], rms, lr=3e-3)
    after = np.mean([tr.grad(d, rms, want_grad=False)[0] for d in states])
    assert after < 0.7 * before, (before, after)
