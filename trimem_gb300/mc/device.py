"""Device-resident Markov chains over the C ABI.

Each step is one HMC move (velocity Verlet on the GPU, exact Metropolis on
the FP64 Hamiltonian, src/trimem/mc/hmc.py:14-26,129-158) followed by one
edge-flip sweep (src/flips.cpp:22-165); the neighbour list is rebuilt every
``refresh`` steps like the reference's evaluator callback
(src/trimem/mc/evaluators.py).  The reference mixes the two moves by a coin
flip per step (src/trimem/mc/hmc.py:325-372); running both every step keeps
the schedule of the large-mesh runs (L velocity-Verlet steps + one sweep).
Positions never leave the device; the six global properties of every
returned state are recorded so that observables such as the bending energy
can be traced without a host copy of the mesh.
"""
import ctypes
import time

import numpy as np


class DeviceChain:
    """Chain on the device positions ``x`` (a contiguous CUDA float64 tensor
    of shape (n_vertices, 3)) of ``mesh``/``energy`` (capi handles)."""

    def __init__(self, mesh, energy, x, mass=1.0, dt=5e-5, n_leapfrog=20, temperature=1.0, flip_ratio=0.2,
                 flip_mode=1, flip_batch=4096, refresh=1, seed=0, stream=None, force=None):
        from .. import capi

        self.capi = capi
        self.lib = capi.lib()
        self.mesh, self.energy, self.x = mesh, energy, x
        self.mass, self.dt, self.L, self.T = float(mass), float(dt), int(n_leapfrog), float(temperature)
        self.flip_ratio, self.flip_mode, self.flip_batch = float(flip_ratio), int(flip_mode), int(flip_batch)
        self.refresh = int(refresh)
        self.seed = int(seed)
        self.stream = ctypes.c_void_p(stream or 0)
        self.force = force  # None: exact gradient; else a surrogate handle
        self.rng = np.random.default_rng(seed)
        self.step_index = 0
        self.accepted = 0
        self.flips = 0
        self.seconds = {"hmc": 0.0, "flip": 0.0, "refresh": 0.0}  # wall time per move (each call synchronises)

    def _ptr(self):
        return ctypes.c_void_p(self.x.data_ptr())

    def step(self):
        """One HMC move and one flip sweep; returns (accepted, props6, energy)."""
        out4 = (ctypes.c_double * 4)()
        props = (ctypes.c_double * 6)()
        u = float(self.rng.uniform())
        t0 = time.perf_counter()
        if self.force is None:
            self.capi.check(self.lib.tm_hmc_step_device(
                self.energy.h, self.mesh.h, self._ptr(), self.mass, self.dt, self.L, self.T, self.seed,
                self.step_index, u, out4, props, self.stream))
        else:
            self.capi.check(self.lib.tm_surrogate_hmc_step_device(
                self.force.h, self.energy.h, self.mesh.h, self._ptr(), self.mass, self.dt, self.L, self.T,
                self.seed, self.step_index, u, out4, props, self.stream))
        acc = out4[0] != 0.0
        self.accepted += int(acc)
        t1 = time.perf_counter()
        self.seconds["hmc"] += t1 - t0
        if self.flip_ratio > 0.0:
            nacc = ctypes.c_int32()
            self.capi.check(self.lib.tm_flip_device(
                self.mesh.h, self.energy.h, self._ptr(), self.flip_ratio,
                (self.seed * 1000003 + self.step_index) & 0xFFFFFFFFFFFFFFFF, self.flip_mode, self.flip_batch,
                ctypes.byref(nacc), self.stream))
            self.flips += nacc.value
        t2 = time.perf_counter()
        self.seconds["flip"] += t2 - t1
        self.step_index += 1
        if self.refresh and self.step_index % self.refresh == 0:
            self.capi.check(self.lib.tm_energy_update_repulsion_device(self.energy.h, self.mesh.h, self._ptr(),
                                                                       self.stream))
        self.seconds["refresh"] += time.perf_counter() - t2
        return acc, np.array(props[:]), out4[3]

    def run(self, n):
        """n steps; returns an (n, 6) array of the global properties after
        each HMC move (before that step's sweep)."""
        trace = np.empty((n, 6))
        for i in range(n):
            _, trace[i], _ = self.step()
        return trace


def relaxed_state(p, f, prm, maxiter=3000, stream=None):
    """Positions of a local energy minimum reached from (p, f) by the device
    L-BFGS (neighbour list refreshed every evaluation): a start for chains
    that would otherwise begin far from equilibrium.  Returns (x, info)."""
    import time

    import torch

    from .. import capi
    from .minim import minimize_device

    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    e0 = en.energy(mesh)
    t0 = time.perf_counter()
    it, e1 = minimize_device(en, mesh, x, maxiter=maxiter, stream=stream)
    torch.cuda.synchronize()
    return x.cpu().numpy(), {"iterations": it, "energy_start": e0, "energy_min": e1,
                             "seconds": round(time.perf_counter() - t0, 3)}


def tune_dt(mesh, energy, x, candidates=(5e-5, 2e-5, 1e-5, 5e-6, 2e-6, 1e-6), n_leapfrog=20, target=0.5,
            pilot=6, seed=99, stream=None, force=None):
    """Largest time step whose pilot acceptance (pilot HMC steps without
    flips, from a copy of x) reaches target; the smallest candidate if none
    does.  Returns (dt, pilot acceptances)."""
    seen = {}
    for dt in candidates:
        xc = x.clone()
        ch = DeviceChain(mesh, energy, xc, dt=dt, n_leapfrog=n_leapfrog, flip_ratio=0.0, refresh=0, seed=seed,
                         stream=stream, force=force)
        ch.run(pilot)
        seen[dt] = ch.accepted / pilot
        if seen[dt] >= target:
            return dt, seen
    return candidates[-1], seen


def equilibrated_state(p, f, prm, rounds=12, maxiter=4000, sweeps=3, warm_steps=100, heat_steps=300,
                       heat_leapfrog=200, dt_candidates=(5e-6, 2e-6, 1e-6, 5e-7, 2e-7), seed=1000, stream=None):
    """A start for chains that sample at equilibrium, from the input mesh
    (p, f) whose energy targets (area, volume: fractions of the input's) may
    lie far from its shape, such as a sphere with a reduced-volume target of
    0.65:

    1. `rounds` rounds of the device L-BFGS (maxiter iterations each, the
       neighbour list refreshed at every evaluation), each followed by
       `sweeps` flip sweeps of ratio 0.2 at T 1, which let the triangulation
       follow the large shape change (a sphere shrinking towards the volume
       target at constant area buckles into a budded or stomatocyte-like
       shape; without flips L-BFGS stalls in the symmetric shrunken sphere);
    2. `warm_steps` HMC moves of 20 velocity-Verlet steps, each with one flip
       sweep, which bring the fast modes to temperature 1 (long
       trajectories from the energy minimum are mostly rejected);
    3. `heat_steps` HMC moves of `heat_leapfrog` velocity-Verlet steps, each
       with one flip sweep: trajectories ten times longer than the sampling
       chains' 20 steps carry the slow long-wavelength bending modes to
       their thermal amplitudes in a few hundred moves instead of the
       hundreds of thousands that short trajectories need (their motion is
       diffusive below the trajectory's frequency).

    Each phase runs at the largest of dt_candidates whose pilot acceptance
    (at that phase's trajectory length) reaches 0.5.

    The energy's reference properties stay those of the input mesh.  Returns
    a dict: x (positions), faces and topo (the flipped triangulation with
    its edge numbering), initial (reference properties), prm, info."""
    import torch

    from .. import capi
    from .minim import minimize_device

    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    initial = en.initial_props()
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    lib = capi.lib()
    sp = ctypes.c_void_p(stream or 0)
    e0 = en.energy(mesh)
    t0 = time.perf_counter()
    relax = []
    for r in range(rounds):
        it, e = minimize_device(en, mesh, x, maxiter=maxiter, stream=stream)
        nacc = 0
        for k in range(sweeps):
            n = ctypes.c_int32()
            capi.check(lib.tm_flip_device(mesh.h, en.h, ctypes.c_void_p(x.data_ptr()), 0.2,
                                          seed + sweeps * r + k, 1, 4096, ctypes.byref(n), sp))
            nacc += n.value
        capi.check(lib.tm_energy_update_repulsion_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()), sp))
        relax.append({"iterations": it, "energy": e, "flips": nacc})
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    dtw, _ = tune_dt(mesh, en, x, candidates=dt_candidates, stream=stream)
    cw = DeviceChain(mesh, en, x, dt=dtw, n_leapfrog=20, flip_ratio=0.2, seed=seed + 5, stream=stream)
    cw.run(warm_steps)
    dt, pilot = tune_dt(mesh, en, x, candidates=dt_candidates, n_leapfrog=heat_leapfrog, stream=stream)
    ch = DeviceChain(mesh, en, x, dt=dt, n_leapfrog=heat_leapfrog, flip_ratio=0.2, seed=seed + 7, stream=stream)
    trace = ch.run(heat_steps)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    rv = 6.0 * np.sqrt(np.pi) * trace[:, 1] / trace[:, 0] ** 1.5
    bend = prm["kappa_b"] * trace[:, 3]
    info = {"energy_start": e0, "relax_rounds": rounds, "relax_iterations": maxiter, "relax_sweeps": sweeps,
            "relax_energy": [round(r_["energy"], 1) for r_ in relax], "relax_seconds": round(t1 - t0, 2),
            "warm_steps": warm_steps, "warm_dt": dtw,
            "warm_acceptance": round(cw.accepted / max(warm_steps, 1), 3),
            "heat_steps": heat_steps, "heat_leapfrog": heat_leapfrog, "heat_dt": dt, "heat_pilot": pilot,
            "heat_acceptance": round(ch.accepted / max(heat_steps, 1), 3), "heat_seconds": round(t2 - t1, 2),
            "heat_bending_quarter_means": [round(float(b.mean()), 1) for b in np.array_split(bend, 4)],
            "heat_reduced_volume_quarter_means": [round(float(b.mean()), 4) for b in np.array_split(rv, 4)]}
    return {"x": x.cpu().numpy(), "faces": mesh.fv_indices(), "topo": mesh.topology(), "initial": initial,
            "prm": prm, "info": info}
