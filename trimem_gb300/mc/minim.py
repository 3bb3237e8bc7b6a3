"""Energy minimisation (src/trimem/mc/util.py:240-306).

``minimize_device`` runs L-BFGS on device-resident positions
(tm_minimize_device: the iterate, gradient and correction pairs stay in
device memory, the cell list is rebuilt at every evaluation).
``minimize_scipy`` is the reference's own route: scipy's L-BFGS-B over the
energy and gradient of the mesh, neighbour list refreshed every evaluation.
"""
import ctypes

import numpy as np


def minimize_device(energy, mesh, x, maxiter=1000, history=10, gtol=1e-5, ftol=2.220446049250313e-09, stream=None):
    """Minimise in place; x is a contiguous CUDA float64 tensor (nv, 3).
    Returns (iterations, energy)."""
    from .. import capi

    it = ctypes.c_int32()
    en = ctypes.c_double()
    capi.check(capi.lib().tm_minimize_device(energy.h, mesh.h, ctypes.c_void_p(x.data_ptr()), int(maxiter),
                                             int(history), float(gtol), float(ftol), ctypes.byref(it),
                                             ctypes.byref(en), ctypes.c_void_p(stream or 0)))
    return it.value, en.value


def minimize_scipy(energy, mesh, maxiter=1000):
    """scipy L-BFGS-B over the host API (capi Mesh/Energy), like the
    reference's run_minim; the mesh points are left at the minimiser.
    Returns (iterations, energy)."""
    from scipy.optimize import minimize

    pts = mesh.points()
    shape = pts.shape

    def fun(x):
        pts[:] = x.reshape(shape)
        energy.update_repulsion(mesh)
        return energy.energy(mesh)

    def grad(x):
        pts[:] = x.reshape(shape)
        energy.update_repulsion(mesh)
        return energy.gradient(mesh).ravel()

    res = minimize(fun, pts.ravel().copy(), jac=grad, method="L-BFGS-B", options={"maxiter": maxiter})
    pts[:] = res.x.reshape(shape)
    return res.nit, float(res.fun)
