"""Energy, gradient and step callback as functions of the vertex positions
(src/trimem/mc/evaluators.py in the reference)."""
import time
from datetime import datetime, timedelta

import numpy as np

_eval_default_options = {
    "info_step": 100,
    "output_step": 1000,
    "cpt_step": 0,
    "refresh_step": 10,
    "flatten": False,
    "num_steps": None,
    "write_cpt": lambda m, e, s: None,
}


class EnergyEvaluators:
    """``fun``/``grad`` write x into the mesh and evaluate the energy manager;
    ``callback`` prints, writes output and checkpoints, refreshes the
    neighbour list every ``refresh_step`` steps and advances the parameter
    continuation."""

    def __init__(self, mesh, estore, output, options):
        self.mesh = mesh
        self.estore = estore
        self.output = output
        options = {**_eval_default_options, **options}
        print("\n------------------------")
        print("Energy Evaluators Setup:")
        width = max(len(str(k)) for k in options)
        for k, v in options.items():
            print(f"  {k: <{width}}: {v}")
        self.info_step = max(options["info_step"], 0)
        self.out_step = max(options["output_step"], 0)
        self.cpt_step = max(options["cpt_step"], 0)
        self.refresh_step = max(options["refresh_step"], 0)
        self.write_cpt = options["write_cpt"]
        self._ravel = (lambda x: np.ravel(x)) if options["flatten"] else (lambda x: x)

    def _update_mesh(func):
        def wrap(self, x, *args, **kwargs):
            self.mesh.x = x.reshape(self.mesh.x.shape)
            return func(self, x, *args, **kwargs)

        wrap.__doc__ = func.__doc__
        wrap.__name__ = func.__name__
        return wrap

    @_update_mesh
    def fun(self, x):
        """Energy at positions x."""
        return self.estore.energy(self.mesh.trimesh)

    @_update_mesh
    def grad(self, x):
        """Gradient of the energy at positions x."""
        return self._ravel(self.estore.gradient(self.mesh.trimesh))

    @_update_mesh
    def callback(self, x, steps):
        i = sum(steps.values())
        if self.info_step and (i % self.info_step == 0):
            print("\n-- Energy-Evaluation-Step ", i)
            self.estore.print_info(self.mesh.trimesh)
        if self.out_step and (i % self.out_step == 0):
            self.output.write_points_cells(self.mesh.x, self.mesh.f)
        if self.cpt_step and (i % self.cpt_step == 0):
            self.write_cpt(self.mesh, self.estore, steps)
        if self.refresh_step and (i % self.refresh_step == 0):
            self.estore.update_repulsion(self.mesh.trimesh)
        self.estore.update_reference_properties()


class TimingEnergyEvaluators(EnergyEvaluators):
    """Adds a wall-clock speed estimate every ``info_step`` steps."""

    def __init__(self, mesh, estore, output, options):
        super().__init__(mesh, estore, output, options)
        self.timestamps = []
        self.n = options["num_steps"] // self.info_step
        self.start = datetime.now()

    def callback(self, x, steps):
        super().callback(x, steps)
        i = sum(steps.values())
        if self.info_step and (i % self.info_step == 0):
            self.timestamps.append(time.time())
            if len(self.timestamps) == 2:
                tspan = self.timestamps[1] - self.timestamps[0]
                speed = tspan / self.info_step
                finish = self.start + timedelta(seconds=tspan) * self.n
                print("\n-- Performance measurements")
                print(f"----- estimated speed: {speed:.3e} s/step")
                print(f"----- estimated end:   {finish}")
                self.timestamps.pop(0)
