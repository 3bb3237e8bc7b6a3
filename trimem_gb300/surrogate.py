"""Learned surrogate force: the weight blob of tm_surrogate_create, the
training data (states of plain device HMC chains) and the training driver
over the library's own training kernels (tm_surrogate_train_*).

The CUDA side (csrc/surrogate.cu) evaluates, per vertex i with ring j,

    h   = SiLU(W_in u + b_in)
    m   = sum_j (W_e^r e_ij + b_e^r) * h_j                 r = 0, 1, 2
    h   = h + SiLU(W^r [h ; m] + b^r)
    F_i = s (sum_j c_ij d_ij + c_i N_i),  c_ij = <w_o, h_i * h_j> + b_o,
                                          c_i  = <w_n, h_i> + b_n

with d_ij the unit edge direction and N_i the vertex normal; the leapfrog
gradient is g_local - F, g_local the exact gradient of the local penalty
terms.  The network is trained on F_target = g_local - g_exact from states
of device chains at the reduced volumes of the learned-surrogate
configuration (MSE on forces, Adam), by hand-written forward and backward
kernels on the GPU; the training set stays resident in device memory.
``make_net`` is the same network in torch, the floating-point reference the
tests check those kernels against.

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
            idx = nbr.clamp(min=0).long()
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

    return SurrogateNet()


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
    """Device tensors of one state: network inputs, and the exact local and
    total gradients' difference as the target (float32)."""

    def __init__(self, sg, energy, mesh, x, max_valence, stream=0):
        torch = _torch()
        from . import capi

        nv = x.shape[0]
        dev = x.device
        self.u = torch.empty(nv, FV, device=dev)
        self.nrm = torch.empty(nv, 4, device=dev)
        nbr = torch.empty(max_valence, nv, dtype=torch.int32, device=dev)
        ef = torch.empty(max_valence, nv, FE, device=dev)
        dirs = torch.empty(max_valence, nv, 3, device=dev)
        self.gloc = torch.empty(nv, 3, dtype=torch.float64, device=dev)
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        capi.check(capi.lib().tm_surrogate_inputs_device(sg.h, energy.h, mesh.h, P(x), max_valence, P(self.u),
                                                         P(self.nrm), P(nbr), P(ef), P(dirs), P(self.gloc),
                                                         ctypes.c_void_p(stream)))
        d = int((nbr >= 0).any(dim=1).sum())  # rows past the largest valence hold no neighbour
        self.nbr = nbr[:d].contiguous()
        self.ef = ef[:d].contiguous()
        self.dirs = dirs[:d].contiguous()

    @property
    def D(self):
        return self.nbr.shape[0]


class DeviceTrainer:
    """The training kernels (tm_surrogate_train_*) for meshes of nv
    vertices and up to max_valence ring slots, started from a weight blob."""

    def __init__(self, nv, max_valence, blob):
        from . import capi

        self.capi = capi
        self.L = capi.lib()
        self.nv = int(nv)
        self.blob = np.ascontiguousarray(blob, dtype=np.float32)
        h = ctypes.c_void_p()
        capi.check(self.L.tm_surrogate_train_create(self.nv, int(max_valence), self.blob.ctypes.data_as(ctypes.c_void_p),
                                                    self.blob.size, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.L.tm_surrogate_train_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _args(self, d):
        P = lambda t: ctypes.c_void_p(t.data_ptr())
        return [P(d.u), P(d.nrm), P(d.nbr), P(d.ef), P(d.dirs), P(d.target), self.nv, d.D]

    def grad(self, d, target_rms, want_grad=True, stream=0):
        """(loss, force, gradient) of one state; gradient in blob order
        without the header (None unless want_grad)."""
        torch = _torch()
        dev = d.u.device
        F = torch.empty(self.nv, 3, device=dev)
        loss = torch.empty(1, device=dev)
        g = torch.empty(BLOB_SIZE - BLOB_HEADER, device=dev) if want_grad else None
        P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
        self.capi.check(self.L.tm_surrogate_train_grad(self.h, *self._args(d), float(target_rms), P(F), P(loss), P(g),
                                                       ctypes.c_void_p(stream)))
        return float(loss.item()), F, g

    def step(self, d, target_rms, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, loss_out=None, stream=0):
        """One Adam step on state d (asynchronous); the loss before the step
        goes to loss_out (a one-element device tensor) when given."""
        P = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
        self.capi.check(self.L.tm_surrogate_train_step(self.h, *self._args(d), float(target_rms), float(lr),
                                                       float(beta1), float(beta2), float(eps), P(loss_out),
                                                       ctypes.c_void_p(stream)))

    def weights(self):
        b = np.empty(BLOB_SIZE, np.float32)
        self.capi.check(self.L.tm_surrogate_train_get_weights(self.h, b.ctypes.data_as(ctypes.c_void_p), b.size))
        return b


VOLUMES = (0.65, 0.75, 0.85)


def generate(n_per_volume, volumes=VOLUMES, every=2, burn=10, level=7, seed=5, max_valence=16, log=print):
    """Training states: for each reduced volume, the 163,842-vertex membrane
    (level-7 icosphere, kb 20, the other parameters of the benchmark) at
    that volume target: the committed equilibrated chain state where one
    exists for it (the benchmark chains' start), else brought to the target
    and heated by equilibrated_state; then a plain device HMC chain (20
    velocity-Verlet steps at the warm-up's time step + a flip sweep of ratio
    0.2 per step) whose every `every`-th state gives one snapshot: the
    network inputs and the target g_local - g_exact.  Everything stays in
    device memory.  Returns (snapshots, (lbar, abar), per-volume info)."""
    torch = _torch()
    from . import capi, meshgen
    from .mc.device import DeviceChain, equilibrated_state
    from .mc.equilibrate import load_state
    from .workloads import workload_params

    p, f = meshgen.jittered_icosphere(level, seed=0)
    data, info = [], []
    scales = None
    g = None
    L = capi.lib()
    for vi, v in enumerate(volumes):
        prm = workload_params(p, f, kappa_b=20.0, vfrac=v)
        t0 = time.perf_counter()
        st = load_state(prm, len(p))  # the committed equilibrated state (0.65 target)
        if st is None:
            st = equilibrated_state(p, f, prm, seed=1000 + 100 * vi)
        mesh = capi.Mesh(st["x"], st["faces"])
        if st["topo"] is not None:
            mesh.set_topology(st["topo"])
        en = capi.Energy(mesh, capi.params(**prm))
        en.set_initial_props(st["initial"])
        if scales is None:
            scales = mesh_scales(st["x"], st["faces"])
            net = make_net()
            with torch.no_grad():
                net.scales.copy_(torch.tensor([scales[0], scales[1], 1.0]))
        sg = capi.Surrogate(mesh, to_blob(net))
        x = torch.tensor(st["x"], dtype=torch.float64, device="cuda").contiguous()
        dt = st["info"]["warm_dt"]
        ch = DeviceChain(mesh, en, x, dt=dt, n_leapfrog=20, flip_ratio=0.2, seed=seed + vi)
        ch.run(burn)
        if g is None:
            g = torch.empty_like(x)
        for k in range(n_per_volume):
            ch.run(every)
            inp = Inputs(sg, en, mesh, x, max_valence)
            capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()),
                                               ctypes.c_void_p(g.data_ptr()), None, None))
            torch.cuda.synchronize()
            inp.target = (inp.gloc - g).float().contiguous()
            del inp.gloc
            data.append(inp)
        info.append({"volume_frac": v, "start": st["info"], "dt": dt, "steps": ch.step_index,
                     "acceptance": round(ch.accepted / max(ch.step_index, 1), 3),
                     "seconds": round(time.perf_counter() - t0, 2)})
        if log:
            log(f"volume {v}: {n_per_volume} snapshots, dt {dt}, acceptance {info[-1]['acceptance']}, "
                f"{info[-1]['seconds']} s")
    return data, scales, info


def train(data, scales, epochs=20, lr=1e-3, seed=0, log=print, n_val=None):
    """Adam at a constant learning rate over the snapshots (shuffled per
    epoch), on the GPU with the library's training kernels.  Returns
    (weights blob, validation relative MSE with the bf16 forward, target
    rms, seconds, steps)."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    lbar, abar = scales
    tgt_rms = float(torch.sqrt(torch.stack([(d.target ** 2).mean() for d in data]).mean()))
    torch.manual_seed(seed)
    net = make_net()
    with torch.no_grad():
        net.scales.copy_(torch.tensor([lbar, abar, tgt_rms]))
    n_val = n_val if n_val is not None else max(1, len(data) // 10)
    val_idx = set(range(len(data))[::max(1, len(data) // n_val)][:n_val])
    train_set = [d for k, d in enumerate(data) if k not in val_idx]
    val_set = [d for k, d in enumerate(data) if k in val_idx]
    D = max(d.D for d in data)
    tr = DeviceTrainer(data[0].u.shape[0], D, to_blob(net))
    loss = torch.zeros(1, device=data[0].u.device)
    t0 = time.perf_counter()
    steps = 0
    for ep in range(epochs):
        for k in rng.permutation(len(train_set)):
            tr.step(train_set[k], tgt_rms, lr=lr, loss_out=loss)
            steps += 1
        if log:
            torch.cuda.synchronize()
            log(f"epoch {ep + 1}/{epochs}: last loss {float(loss.item()):.4f} ({time.perf_counter() - t0:.1f} s)")
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    val = [tr.grad(d, tgt_rms, want_grad=False)[0] for d in val_set]
    return tr.weights(), float(np.mean(val)), tgt_rms, secs, steps


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--per-volume", type=int, default=200, help="snapshots per reduced volume")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default=WEIGHTS_L7)
    args = ap.parse_args()
    log = lambda *a: print(*a, flush=True)
    data, scales, info = generate(args.per_volume, log=log)
    blob, val, rms, secs, steps = train(data, scales, epochs=args.epochs, lr=args.lr, log=log)
    np.save(args.out, blob)
    print(f"{steps} Adam steps in {secs:.1f} s ({1e3 * secs / max(steps, 1):.2f} ms each); validation relative MSE "
          f"{val:.4f}, target rms {rms:.4g}, weights -> {args.out}")


if __name__ == "__main__":
    main()
