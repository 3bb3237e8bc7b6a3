"""Sampled observables: the device chain (tm_hmc_step_device + the windowed
device flip sweep) against a host chain of the same moves built from the
oracle (the reference's energy and gradient, its velocity-Verlet HMC move
src/trimem/mc/hmc.py:14-26 restated, and its serial flip sweep from
src/flips.cpp:22-165: uniform proposals with replacement, each tried on the
current state, the distribution the device's windows reproduce; the
reference's try-lock parallel sweep instead skips proposals whose patch is
busy) on the 642-vertex membrane.  The two chains use different random
streams and proposal orders, so only their distributions can agree: the
means of the bending energy, the reduced volume and the area, the HMC
acceptance and the accepted flips per sweep are compared with batch-means
standard errors (z <= 4.5)."""
import os

import numpy as np
import pytest

from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu

N_BURN, N_REC, N_BATCH = 300, 2000, 20


def batch_se(x, nb=N_BATCH):
    """Standard error of the mean of a correlated series by batch means."""
    b = np.array([c.mean() for c in np.array_split(np.asarray(x, dtype=np.float64), nb)])
    return b.std(ddof=1) / np.sqrt(nb)


def host_chain(x0, f, prm, dt, n_leapfrog, ratio, n_steps, seed):
    """(props after each HMC move, accepted moves, accepted flips per sweep)."""
    from oracle import oracle as O

    O.set_threads(min(8, os.cpu_count() or 1))
    mo = O.Mesh(x0, f)
    eo = O.Energy(mo, O.default_params(**prm))
    x = mo.points()
    rng = np.random.default_rng(seed)
    trace = np.empty((n_steps, 6))
    acc = np.zeros(n_steps)
    flips = np.zeros(n_steps)
    for i in range(n_steps):
        eo.update_repulsion(mo)
        xs = x.copy()
        pm = rng.standard_normal(x.shape)
        h0 = eo.energy(mo) + 0.5 * float((pm * pm).sum())
        a = -eo.gradient(mo)
        for _ in range(n_leapfrog):
            x += pm * dt + (0.5 * dt * dt) * a
            a1 = -eo.gradient(mo)
            pm += (0.5 * dt) * (a + a1)
            a = a1
        h1 = eo.energy(mo) + 0.5 * float((pm * pm).sum())
        if rng.random() <= np.exp(min(0.0, h0 - h1)):
            acc[i] = 1
        else:
            x[:] = xs
        trace[i] = eo.properties(mo)
        flips[i] = O.flip_serial(mo, eo, ratio, int(rng.integers(1 << 31)))
    return trace, acc, flips


def test_device_chain_samples_the_host_chains_distribution(built):
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.device import DeviceChain, relaxed_state, tune_dt
    from trimem_gb300.workloads import workload_params

    p, f = meshgen.jittered_icosphere(3, seed=1)
    prm = dict(workload_params(p, f, kappa_b=20.0, vfrac=0.65), cont_lambda=0.0)
    x0, _ = relaxed_state(p, f, prm)
    L, ratio = 10, 0.2
    mesh = capi.Mesh(x0, f)
    en = capi.Energy(mesh, capi.params(**prm))
    x = torch.tensor(x0, dtype=torch.float64, device="cuda").contiguous()
    dt, _ = tune_dt(mesh, en, x, candidates=(1e-3, 5e-4, 2e-4, 1e-4, 5e-5, 2e-5), n_leapfrog=L, target=0.6)
    # the host chain's targets: the same initial properties (relaxed state)
    ch = DeviceChain(mesh, en, x, dt=dt, n_leapfrog=L, flip_ratio=ratio, seed=17)
    ch.run(N_BURN)
    dev = np.empty((N_REC, 6))
    dacc = np.zeros(N_REC)
    dfl = np.zeros(N_REC)
    for i in range(N_REC):
        before = ch.flips
        ok, dev[i], _ = ch.step()
        dacc[i] = float(ok)
        dfl[i] = ch.flips - before
    host, hacc, hfl = host_chain(x0, f, prm, dt, L, ratio, N_BURN + N_REC, seed=23)
    host, hacc, hfl = host[N_BURN:], hacc[N_BURN:], hfl[N_BURN:]

    kb = prm["kappa_b"]
    obs = {
        "bending": (kb * dev[:, 3], kb * host[:, 3]),
        "reduced volume": (6.0 * np.sqrt(np.pi) * dev[:, 1] / dev[:, 0] ** 1.5,
                           6.0 * np.sqrt(np.pi) * host[:, 1] / host[:, 0] ** 1.5),
        "area": (dev[:, 0], host[:, 0]),
        "HMC acceptance": (dacc, hacc),
        "accepted flips per sweep": (dfl, hfl),
    }
    report, zs = [], []
    for name, (a, b) in obs.items():
        se = np.hypot(batch_se(a), batch_se(b))
        z = abs(a.mean() - b.mean()) / se if se > 0 else 0.0
        zs.append(z)
        report.append(f"{name}: device {a.mean():.6g} host {b.mean():.6g} z {z:.2f}")
    print("\n".join(report))
    assert max(zs) <= 4.5, report
    assert 0.2 < dacc.mean() < 1.0 and dfl.mean() > 0.0  # both moves mix
