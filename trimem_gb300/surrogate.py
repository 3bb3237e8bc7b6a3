"""Learned surrogate force: the network in torch (training, and the FP32
reference of the CUDA forward), the weight blob of tm_surrogate_create, and
the training driver.

The CUDA side (csrc/surrogate.cu) evaluates, per vertex i with ring j,

    h   = SiLU(W_in u + b_in)
    m   = sum_j (W_e^r e_ij + b_e^r) * h_j                 r = 0, 1, 2
    h   = h + SiLU(W^r [h ; m] + b^r)
    F_i = s (sum_j c_ij d_ij + c_i N_i),  c_ij = <w_o, h_i * h_j> + b_o,
                                          c_i  = <w_n, h_i> + b_n

with d_ij the unit edge direction and N_i the vertex normal; the leapfrog
gradient is g_local - F, g_local the exact gradient of the local penalty
terms.  The network is trained on F_target = g_local - g_exact from states
of a device chain (MSE on forces, Adam).

Run ``python -m trimem_gb300.surrogate --out weights.npy`` on a GPU to train
the weights for the 163,842-vertex benchmark membrane.
"""
import argparse
import ctypes
import os
import time

import numpy as np

H, FV, FE, NR = 64, 8, 4, 3
BLOB_HEADER = 8
BLOB_SIZE = BLOB_HEADER + H * FV + H + NR * (H * FE + H + H * 2 * H + H) + H + 1 + H + 1
WEIGHTS_L7 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "surrogate_L7.npy")


def _torch():
    import torch
    return torch


def make_net():
    torch = _torch()
    nn = torch.nn

    class SurrogateNet(nn.Module):
        def __init__(self):
            super().__init__()
            self.win = nn.Linear(FV, H)
            self.we = nn.ModuleList([nn.Linear(FE, H) for _ in range(NR)])
            self.dense = nn.ModuleList([nn.Linear(2 * H, H) for _ in range(NR)])
            self.wo = nn.Parameter(torch.zeros(H))
            self.bo = nn.Parameter(torch.zeros(()))
            self.wn = nn.Parameter(torch.zeros(H))
            self.bn = nn.Parameter(torch.zeros(()))
            with torch.no_grad():
                for d in self.dense:
                    d.weight.mul_(0.5)
                self.wo.normal_(0, 0.05)
                self.wn.normal_(0, 0.05)
            self.register_buffer("scales", torch.tensor([1.0, 1.0, 1.0]))  # lbar, abar, fscale

        def forward(self, u, nrm, nbr, ef, dirs, bf16=False):
            """u (nv, 8), nrm (nv, 4), nbr (D, nv) int64 with -1 padding,
            ef (D, nv, 4), dirs (D, nv, 3) -> F (nv, 3).  bf16=True rounds
            activations and dense weights like the CUDA forward."""
            F_ = torch.nn.functional
            rnd = (lambda t: t.to(torch.bfloat16).float()) if bf16 else (lambda t: t)
            mask = (nbr >= 0).to(u.dtype)
            idx = nbr.clamp(min=0)
            h = rnd(F_.silu(self.win(u)))
            for r in range(NR):
                g = self.we[r](ef)
                m = rnd((mask[..., None] * g * h[idx]).sum(0))
                W = rnd(self.dense[r].weight)
                h = rnd(h + F_.silu(torch.cat([h, m], 1) @ W.t() + self.dense[r].bias))
            c = ((h[None] * h[idx]) * self.wo).sum(-1) + self.bo
            c = c * mask
            cn = h @ self.wn + self.bn
            F = (c[..., None] * dirs).sum(0) + cn[:, None] * nrm[:, :3]
            return self.scales[2] * F

        def forward_sparse(self, sp):
            """The same function with the ring sums as sparse products
            (training): m = sum_k W_e[:, k] * (E_k h) + b_e * (A h), with
            E_k / A the adjacency weighted by edge feature k / by one, and
            sum_j c_ij d_ij = ((w_o * h) . (D h)) + b_o D 1 per component."""
            F_ = torch.nn.functional
            h = F_.silu(self.win(sp.u))
            for r in range(NR):
                Y = [torch.sparse.mm(a, h) for a in sp.E]
                m = sum(self.we[r].weight[:, k] * Y[k] for k in range(FE)) + self.we[r].bias * Y[FE]
                h = h + F_.silu(torch.cat([h, m], 1) @ self.dense[r].weight.t() + self.dense[r].bias)
            hw = h * self.wo
            F = torch.stack([(hw * torch.sparse.mm(d, h)).sum(1) for d in sp.D], 1) + self.bo * sp.dsum
            F = F + (h @ self.wn + self.bn)[:, None] * sp.nrm[:, :3]
            return self.scales[2] * F

    return SurrogateNet()


class SparseInputs:
    """Inputs as sparse adjacency matrices (COO, shared pattern): E_0..E_3
    weighted by the edge features, E_4 by one, D_x, D_y, D_z by the unit
    edge directions."""

    def __init__(self, inp):
        torch = _torch()
        D, nv = inp.nbr.shape
        sel = inp.nbr >= 0
        rows = torch.arange(nv, device=inp.nbr.device).expand(D, nv)[sel]
        cols = inp.nbr[sel]
        ind = torch.stack([rows, cols])

        def mat(v):
            return torch.sparse_coo_tensor(ind, v, (nv, nv), check_invariants=False).coalesce()

        self.E = [mat(inp.ef[..., k][sel]) for k in range(FE)] + [mat(torch.ones_like(inp.ef[..., 0][sel]))]
        self.D = [mat(inp.dirs[..., k][sel]) for k in range(3)]
        self.dsum = (inp.dirs * sel[..., None]).sum(0)
        self.u = inp.u
        self.nrm = inp.nrm
        self.target = getattr(inp, "target", None)


def to_blob(net):
    """float32 blob in the layout tm_surrogate_create parses."""
    lbar, abar, fscale = [float(x) for x in net.scales]
    parts = [np.array([1.0, FV, FE, H, NR, lbar, abar, fscale], np.float32)]

    def add(t):
        parts.append(t.detach().float().cpu().numpy().reshape(-1).astype(np.float32))

    add(net.win.weight)
    add(net.win.bias)
    for r in range(NR):
        add(net.we[r].weight)
        add(net.we[r].bias)
        add(net.dense[r].weight)
        add(net.dense[r].bias)
    add(net.wo)
    add(net.bo.reshape(1))
    add(net.wn)
    add(net.bn.reshape(1))
    b = np.concatenate(parts)
    assert b.size == BLOB_SIZE
    return b


def from_blob(b):
    torch = _torch()
    b = np.asarray(b, np.float32)
    assert b.size == BLOB_SIZE and b[0] == 1.0
    net = make_net()
    q = BLOB_HEADER

    def take(shape):
        nonlocal q
        n = int(np.prod(shape))
        t = torch.tensor(b[q:q + n].reshape(shape))
        q += n
        return t

    with torch.no_grad():
        net.scales.copy_(torch.tensor(b[5:8]))
        net.win.weight.copy_(take((H, FV)))
        net.win.bias.copy_(take((H,)))
        for r in range(NR):
            net.we[r].weight.copy_(take((H, FE)))
            net.we[r].bias.copy_(take((H,)))
            net.dense[r].weight.copy_(take((H, 2 * H)))
            net.dense[r].bias.copy_(take((H,)))
        net.wo.copy_(take((H,)))
        net.bo.copy_(take((1,))[0])
        net.wn.copy_(take((H,)))
        net.bn.copy_(take((1,))[0])
    return net


def mesh_scales(p, f):
    """mean edge length and mean vertex area (a third of the face areas)"""
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    lbar = float(np.linalg.norm(p[e[:, 0]] - p[e[:, 1]], axis=1).mean())
    a = 0.5 * np.linalg.norm(np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]]), axis=1)
    return lbar, float(a.sum() / len(p))


class Inputs:
    """Device tensors of one state: network inputs and the exact gradients."""

    def __init__(self, sg, energy, mesh, x, max_valence, stream=0):
        torch = _torch()
        from . import capi

        nv = x.shape[0]
        dev = x.device
        self.u = torch.empty(nv, FV, device=dev)
        self.nrm = torch.empty(nv, 4, device=dev)
        nbr = torch.empty(max_valence, nv, dtype=torch.int32, device=dev)
        self.ef = torch.empty(max_valence, nv, FE, device=dev)
        self.dirs = torch.empty(max_valence, nv, 3, device=dev)
        self.gloc = torch.empty(nv, 3, dtype=torch.float64, device=dev)
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        capi.check(capi.lib().tm_surrogate_inputs_device(sg.h, energy.h, mesh.h, P(x), max_valence, P(self.u),
                                                         P(self.nrm), P(nbr), P(self.ef), P(self.dirs), P(self.gloc),
                                                         ctypes.c_void_p(stream)))
        d = int((nbr >= 0).any(dim=1).sum())  # rows past the largest valence hold no neighbour
        self.nbr = nbr[:d].long()
        self.ef = self.ef[:d].contiguous()
        self.dirs = self.dirs[:d].contiguous()


def generate(n_snap, every=2, burn=10, level=7, seed=5, max_valence=16, log=print):
    """States of the benchmark chain (the 163,842-vertex membrane relaxed by
    L-BFGS, initial area / volume targets; HMC with 20 velocity-Verlet steps
    at the tuned time step + a flip sweep of ratio 0.2 per step) with the
    network inputs and the training target g_local - g_exact."""
    torch = _torch()
    from . import capi, meshgen
    from .mc.device import DeviceChain, relaxed_state, tune_dt
    from .workloads import workload_params

    p, f = meshgen.jittered_icosphere(level, seed=0)
    prm = dict(workload_params(p, f, kappa_b=20.0, vfrac=0.65), cont_lambda=0.0)
    x0, info = relaxed_state(p, f, prm)
    log(f"relaxed start: {info}")
    mesh = capi.Mesh(x0, f)
    en = capi.Energy(mesh, capi.params(**prm))
    lbar, abar = mesh_scales(x0, f)
    net = make_net()
    with torch.no_grad():
        net.scales.copy_(torch.tensor([lbar, abar, 1.0]))
    sg = capi.Surrogate(mesh, to_blob(net))
    x = torch.tensor(x0, dtype=torch.float64, device="cuda").contiguous()
    dt, pilot = tune_dt(mesh, en, x)
    log(f"time step {dt} (pilot acceptance {pilot})")
    ch = DeviceChain(mesh, en, x, dt=dt, n_leapfrog=20, flip_ratio=0.2, seed=seed)
    ch.run(burn)
    L = capi.lib()
    data = []
    g = torch.empty_like(x)
    for k in range(n_snap):
        ch.run(every)
        inp = Inputs(sg, en, mesh, x, max_valence)
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(g.data_ptr()),
                                           None, None))
        torch.cuda.synchronize()
        inp.target = (inp.gloc - g).float()
        del inp.gloc
        data.append(inp)
        if log and (k + 1) % 10 == 0:
            log(f"snapshot {k + 1}/{n_snap}, acceptance so far {ch.accepted / ch.step_index:.2f}")
    return data, (lbar, abar), dict(prm, dt=dt)


def train(data, scales, iters=1500, lr=2e-3, seed=0, log=print, budget_s=420.0):
    torch = _torch()
    torch.manual_seed(seed)
    lbar, abar = scales
    tgt_rms = float(torch.sqrt(torch.stack([(d.target ** 2).mean() for d in data]).mean()))
    net = make_net().cuda()
    with torch.no_grad():
        net.scales.copy_(torch.tensor([lbar, abar, tgt_rms]))
    opt = torch.optim.Adam(net.parameters(), lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, iters)
    n_val = max(1, len(data) // 8)
    train_set, val_set = data[:-n_val], data[-n_val:]
    sparse = [SparseInputs(d) for d in train_set]
    t0 = time.time()
    for it in range(iters):
        if time.time() - t0 > budget_s:
            log(f"time budget reached after {it} iterations")
            break
        d = sparse[it % len(sparse)]
        F = net.forward_sparse(d)
        loss = ((F - d.target) ** 2).mean() / tgt_rms ** 2
        opt.zero_grad()
        loss.backward()
        opt.step()
        sched.step()
        if log and (it % 250 == 0 or it == iters - 1):
            log(f"iter {it} loss {loss.item():.4f} ({time.time() - t0:.0f} s)")
    with torch.no_grad():
        errs = []
        for d in val_set:
            F = net(d.u, d.nrm, d.nbr, d.ef, d.dirs, bf16=True)
            errs.append(float(((F - d.target) ** 2).mean() / (d.target ** 2).mean()))
    return net, float(np.mean(errs)), tgt_rms


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--snapshots", type=int, default=48)
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--out", default=WEIGHTS_L7)
    ap.add_argument("--budget", type=float, default=420.0, help="training time limit in seconds")
    args = ap.parse_args()
    log = lambda *a: print(*a, flush=True)
    data, scales, _ = generate(args.snapshots, log=log)
    net, val, rms = train(data, scales, iters=args.iters, log=log, budget_s=args.budget)
    b = to_blob(net.cpu())
    np.save(args.out, b)
    print(f"validation relative MSE (bf16 forward) {val:.4f}, target rms {rms:.4g}, weights -> {args.out}")


if __name__ == "__main__":
    main()
