"""Equilibrated start state of the learned-surrogate and ESS chains on the
163,842-vertex benchmark membrane (level-7 icosphere, jitter seed 0, kb 20,
reduced-volume target 0.65, the other parameters of the benchmark).

``equilibrated_state`` brings the sphere to the volume target (L-BFGS and
flip rounds) and heats it (long-trajectory HMC); this script then runs the
sampling chains' own moves (20 velocity-Verlet steps + one flip sweep of
ratio 0.2 per step) for --steps steps, printing the bending energy's block
means, and saves the final state: positions (float32), faces, the energy's
reference properties and the block means.  bench.py starts its chains from
this file when it is present and matches the workload; otherwise it runs
``equilibrated_state`` itself (shorter, and its chains then show the
remaining drift).

    python -m trimem_gb300.mc.equilibrate --steps 30000 --out trimem_gb300/data/chain_state_L7.npz
    python -m trimem_gb300.mc.equilibrate --steps 40000 --resume trimem_gb300/data/chain_state_L7.npz
"""
import argparse
import os
import time

import numpy as np

STATE_L7 = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data", "chain_state_L7.npz")


def workload_key(prm, nv):
    """Identifies the energy a saved state belongs to."""
    keys = sorted(k for k, v in prm.items() if isinstance(v, (int, float)))
    return np.array([nv] + [float(prm[k]) for k in keys], dtype=np.float64)


def load_state(prm, nv, path=STATE_L7):
    """The saved state as a chain-state dict (x, faces, topo None, initial,
    prm, info), or None when the file is absent or belongs to another
    workload."""
    if not os.path.exists(path):
        return None
    z = np.load(path)
    if z["key"].shape != workload_key(prm, nv).shape or not np.array_equal(z["key"], workload_key(prm, nv)):
        return None
    return {"x": z["x"].astype(np.float64), "faces": z["faces"].astype(np.int32), "topo": None,
            "initial": z["initial"], "prm": prm,
            "info": {"source": os.path.basename(path), "steps": int(z["steps"]), "warm_dt": float(z["dt"]),
                     "bending_block_means": [round(float(b), 1) for b in z["block_means"]],
                     "block_steps": int(z["block_steps"])}}


def main():
    import torch

    from .. import workloads
    from .device import DeviceChain, equilibrated_state

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--steps", type=int, default=30000)
    ap.add_argument("--block", type=int, default=2000)
    ap.add_argument("--out", default=STATE_L7)
    ap.add_argument("--resume", default=None, help="continue from a state saved by this script")
    args = ap.parse_args()
    p, f, prm = workloads.very_large_mesh()
    t0 = time.perf_counter()
    done, means = 0, []
    if args.resume:
        st = load_state(prm, len(p), args.resume)
        if st is None:
            raise SystemExit(f"{args.resume}: no state of this workload")
        done, means = st["info"]["steps"], list(st["info"]["bending_block_means"])
    else:
        st = equilibrated_state(p, f, prm)
    print("start:", st["info"], flush=True)
    from .. import capi

    mesh = capi.Mesh(st["x"], st["faces"])
    if st["topo"] is not None:
        mesh.set_topology(st["topo"])
    en = capi.Energy(mesh, capi.params(**prm))
    en.set_initial_props(st["initial"])
    x = torch.tensor(st["x"], dtype=torch.float64, device="cuda").contiguous()
    dt = st["info"]["warm_dt"]
    ch = DeviceChain(mesh, en, x, dt=dt, n_leapfrog=20, flip_ratio=0.2, seed=2024 + done)
    for b in range(0, args.steps, args.block):
        tr = ch.run(min(args.block, args.steps - b))
        bend = prm["kappa_b"] * tr[:, 3]
        rv = 6.0 * np.sqrt(np.pi) * tr[:, 1] / tr[:, 0] ** 1.5
        means.append(float(bend.mean()))
        print(f"steps {done + b + len(tr)}: bending mean {bend.mean():.1f} sd {bend.std():.1f}, reduced volume "
              f"{rv.mean():.5f}, acceptance {ch.accepted / ch.step_index:.3f} ({time.perf_counter() - t0:.0f} s)",
              flush=True)
    torch.cuda.synchronize()
    np.savez_compressed(args.out, x=x.cpu().numpy().astype(np.float32), faces=mesh.fv_indices().astype(np.int32),
                        initial=np.asarray(st["initial"], np.float64), key=workload_key(prm, len(p)),
                        steps=done + args.steps, dt=dt, block_means=np.array(means), block_steps=args.block)
    print("saved", args.out, os.path.getsize(args.out), "bytes")


if __name__ == "__main__":
    main()
