"""Hamiltonian Monte Carlo with optional cooling, edge-flip sweeps as Monte
Carlo moves and their mixture (src/trimem/mc/hmc.py in the reference).

The random-number calls follow the reference's order (``np.random.normal``
for the momenta, then one ``np.random.uniform`` per step; ``np.random.choice``
in the mixture), so seeded runs reproduce the reference's chains.
"""
from collections import Counter

import numpy as np


def _core():
    from .. import load_core
    return load_core()


def _vv_integration(x0, p0, force, m, dt, N):
    """Velocity Verlet with momenta (src/trimem/mc/hmc.py:14-26)."""
    x, p = x0, p0
    a = force(x)
    for _ in range(N):
        x = x + (p * dt + 0.5 * a * dt**2) / m
        an = force(x)
        p = p + 0.5 * (a + an) * dt
        a = an
    return x, p


def get_step_counters():
    """Counter with keys 'move' and 'flip'."""
    return Counter(move=0, flip=0)


_hmc_default_options = {
    "mass": 1.0,
    "time_step": 1.0e-4,
    "num_integration_steps": 100,
    "initial_temperature": 1.0,
    "minimal_temperature": 1.0e-6,
    "cooling_factor": 0.0,
    "cooling_start_step": 0,
    "info_step": 100,
}


def _print_options(title, options):
    print("\n" + "-" * (len(title) + 4))
    print(title)
    width = max(len(str(k)) for k in options)
    for k, v in options.items():
        print(f"  {k: <{width}}: {v}")


class HMC:
    """Plain HMC on a state array with exponential cooling
    T = clamp(exp(-f (i - c)) T0, Tmin, T0) (src/trimem/mc/hmc.py:48-190).

    As in the reference, ``run`` keeps its own callback slot but does not call
    it; :class:`MeshMonteCarlo` invokes its callback every step.
    """

    def __init__(self, x, nlog_prob, grad_nlog_prob, callback=None, counter=None, options=None):
        self.nlog_prob = nlog_prob
        self.grad_nlog_prob = grad_nlog_prob
        self.cb = lambda x, s: None if callback is None else callback
        options = {**_hmc_default_options, **(options or {})}
        self.m = options["mass"]
        self.dt = options["time_step"]
        self.L = options["num_integration_steps"]
        self.Tinit = options["initial_temperature"]
        self.Tmin = options["minimal_temperature"]
        self.fT = options["cooling_factor"]
        self.cN = options["cooling_start_step"]
        self.istep = options["info_step"]
        _print_options("Hamiltonian Monte Carlo Initialization:", options)
        self.counter = counter if counter is not None else get_step_counters()
        self.i = 0
        self.acc = 0
        self.T = self.Tinit
        self.x = x

    def _hamiltonian(self, x, p):
        return self.nlog_prob(x) + 0.5 * p.ravel().dot(p.ravel()) / self.m

    def _step(self):
        p = np.random.normal(size=self.x.shape) * np.sqrt(self.m * self.T)
        force = lambda x: -self.grad_nlog_prob(x)
        xn, pn = _vv_integration(self.x, p, force, self.m, self.dt, self.L)
        dh = (self._hamiltonian(xn, pn) - self._hamiltonian(self.x, p)) / self.T
        a = 1.0 if dh <= 0 else np.exp(-dh)
        u = np.random.uniform()
        if u <= a:
            self.x = xn
            self.acc += 1
        self.i += 1

    def info(self):
        i_total = sum(self.counter.values())
        if self.istep and i_total % self.istep == 0:
            ar = self.acc / self.i if self.i != 0 else 0.0
            print("\n-- HMC-Step ", self.counter["move"])
            print("----- acc-rate:   ", ar)
            print("----- temperature:", self.T)
            self.acc = 0
            self.i = 0

    def _update_temperature(self):
        i = sum(self.counter.values())
        Tn = np.exp(-self.fT * (i - self.cN)) * self.Tinit
        self.T = max(min(Tn, self.Tinit), self.Tmin)

    def step(self):
        self._update_temperature()
        self._step()
        self.counter["move"] += 1

    def run(self, N):
        for _ in range(N):
            self.step()
            self.info()
            self.cb(self.x, self.counter)


class MeshHMC(HMC):
    """HMC whose state is a :class:`~trimem_gb300.mc.mesh.Mesh`; the mesh
    vertices follow the chain after every step."""

    def __init__(self, mesh, nlog_prob, grad_nlog_prob, callback=None, counter=None, options=None):
        super().__init__(mesh.x, nlog_prob, grad_nlog_prob, callback, counter, options)
        self.mesh = mesh

    def step(self):
        super().step()
        self.mesh.x = self.x


_mc_flip_default_options = {
    "flip_type": "parallel",
    "flip_ratio": 0.1,
    "info_step": 100,
}


class MeshFlips:
    """Edge-flip sweeps as a Monte Carlo move (src/trimem/mc/hmc.py:242-322).

    ``seed`` (optional) makes the sweeps reproducible: sweep k uses seed
    ``seed + k``; without it every sweep is seeded from the clock like the
    reference."""

    def __init__(self, mesh, estore, counter=None, options=None, seed=None):
        m = _core()
        self.mesh = mesh
        self.estore = estore
        options = {**_mc_flip_default_options, **(options or {})}
        self.istep = options["info_step"]
        self.fr = options["flip_ratio"]
        self.ft = options["flip_type"]
        _print_options("Flips Monte Carlo Initialization:", options)
        self._seed = seed
        self._nsweep = 0

        def seed_k():
            if self._seed is None:
                return None
            self._nsweep += 1
            return self._seed + self._nsweep - 1

        if self.ft == "none" or self.fr == 0.0:
            self._flips = lambda: 0
        elif self.ft == "serial":
            self._flips = lambda: m.flip(self.mesh.trimesh, self.estore, self.fr, seed=seed_k())
        elif self.ft == "parallel":
            self._flips = lambda: m.pflip(self.mesh.trimesh, self.estore, self.fr, seed=seed_k())
        else:
            raise ValueError("Wrong flip-type: {}".format(self.ft))
        self.i = 0
        self.acc = 0
        self.counter = counter if counter is not None else get_step_counters()

    def info(self):
        i_total = sum(self.counter.values())
        if self.istep and i_total % self.istep == 0:
            n_edges = self.mesh.trimesh.n_edges()
            ar = self.acc / (self.i * n_edges) if self.i != 0 else 0.0
            print("\n-- MCFlips-Step ", self.counter["flip"])
            print("----- flip-accept: ", ar)
            print("----- flip-rate:   ", self.fr)
            self.acc = 0
            self.i = 0

    def step(self):
        self.acc += self._flips()
        self.i += 1
        self.counter["flip"] += 1

    def run(self, N):
        for _ in range(N):
            self.step()
            self.info()


class MeshMonteCarlo:
    """Each step is an HMC step or a flip sweep with equal probability
    (src/trimem/mc/hmc.py:325-372)."""

    def __init__(self, hmc, flips, counter=None, callback=None):
        self.hmc = hmc
        self.flips = flips
        self.cb = (lambda x, s: None) if callback is None else callback
        self.counter = counter if counter is not None else get_step_counters()
        self.hmc.counter = self.counter
        self.flips.counter = self.counter

    def step(self):
        if np.random.choice(2) == 0:
            self.hmc.step()
        else:
            self.flips.step()

    def run(self, N):
        for _ in range(N):
            self.step()
            self.hmc.info()
            self.flips.info()
            self.cb(self.flips.mesh.x, self.counter)
