"""ctypes front-end of the oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (oracle.cpp) is a CPU restatement of the reference's
energy/gradient/neighbour-list/flip path.  This module exposes it to the
tests, to smoke() as the checker, and to bench.py's CPU-baseline leg.  The
product package never imports it.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# TRIMEM_ORACLE_BUILD selects the build this process loads: "parity" (the
# default; no FMA contraction, what the tests check against) or "timing"
# (-O3 -fopenmp with the compiler's default contraction, the timed CPU
# baseline).  Read once, at the first use.
BUILD = os.environ.get("TRIMEM_ORACLE_BUILD", "parity")
if BUILD not in ("parity", "timing"):
    raise ValueError(f"TRIMEM_ORACLE_BUILD must be 'parity' or 'timing', not {BUILD!r}")
_LIB_PATH = os.path.join(_HERE, "_build", platform.machine(),
                         "liboracle.so" if BUILD == "parity" else "liboracle_timing.so")
_lib = None

_d = ctypes.c_double
_i = ctypes.c_int
_p = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Params(ctypes.Structure):
    _fields_ = [
        ("kappa_b", _d), ("kappa_a", _d), ("kappa_v", _d), ("kappa_c", _d), ("kappa_t", _d), ("kappa_r", _d),
        ("area_frac", _d), ("volume_frac", _d), ("curvature_frac", _d),
        ("bond_lc0", _d), ("bond_lc1", _d), ("bond_a0", _d),
        ("bond_r", ctypes.c_int32), ("bond_type", ctypes.c_int32),
        ("rep_lc1", _d), ("rep_r", ctypes.c_int32), ("n_search", ctypes.c_int32),
        ("rlist", _d), ("exclusion_level", ctypes.c_int32), ("pad0", ctypes.c_int32),
        ("cont_delta", _d), ("cont_lambda", _d),
    ]


def default_params(**kw):
    """Defaults of the reference's EnergyParams (src/params.h:19-71)."""
    p = Params(kappa_b=0, kappa_a=0, kappa_v=0, kappa_c=0, kappa_t=0, kappa_r=0,
               area_frac=1, volume_frac=1, curvature_frac=1,
               bond_lc0=1, bond_lc1=0, bond_a0=1, bond_r=2, bond_type=0,
               rep_lc1=0, rep_r=2, n_search=0, rlist=0.1, exclusion_level=2,
               cont_delta=0, cont_lambda=1)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        sig = {
            "om_last_error": (ctypes.c_char_p, []),
            "om_set_threads": (None, [_i]),
            "om_get_threads": (_i, []),
            "om_mesh_create": (_p, [_dp, _i, _ip, _i]),
            "om_mesh_clone": (_p, [_p]),
            "om_mesh_destroy": (None, [_p]),
            "om_mesh_nv": (_i, [_p]), "om_mesh_ne": (_i, [_p]), "om_mesh_nf": (_i, [_p]),
            "om_mesh_points": (_dp, [_p]),
            "om_mesh_fv": (None, [_p, _ip]),
            "om_mesh_topology": (None, [_p, _ip, _ip, _ip, _ip, _ip]),
            "om_mesh_next": (_i, [_p, _i]), "om_mesh_to": (_i, [_p, _i]),
            "om_mesh_check": (_i, [_p]),
            "om_edge_length": (_d, [_p, _i]), "om_edge_length_grad": (None, [_p, _i, _dp]),
            "om_face_area": (_d, [_p, _i]), "om_face_area_grad": (None, [_p, _i, _dp]),
            "om_face_volume": (_d, [_p, _i]), "om_face_volume_grad": (None, [_p, _i, _dp]),
            "om_dihedral_angle": (_d, [_p, _i]), "om_dihedral_angle_grad": (None, [_p, _i, _dp]),
            "om_energy_create": (_p, [_p, ctypes.POINTER(Params)]),
            "om_energy_destroy": (None, [_p]),
            "om_energy_properties": (None, [_p, _p, _dp]),
            "om_energy_vertex_properties": (None, [_p, _p, _dp]),
            "om_energy_energy": (_d, [_p, _p]),
            "om_energy_energy_props": (_d, [_p, _dp]),
            "om_energy_components": (None, [_p, _p, _dp]),
            "om_energy_gradient": (None, [_p, _p, _dp]),
            "om_energy_update_reference": (None, [_p]),
            "om_energy_update_repulsion": (None, [_p, _p]),
            "om_energy_initial_props": (None, [_p, _dp]),
            "om_energy_set_initial_props": (None, [_p, _dp]),
            "om_energy_ref_props": (None, [_p, _dp]),
            "om_energy_lambda": (_d, [_p]),
            "om_nlist_create": (_p, [_p, _i, _i, _d]),
            "om_nlist_destroy": (None, [_p]),
            "om_nlist_distance_matrix": (ctypes.c_int64, [_p, _p, _d]),
            "om_nlist_point_distances": (ctypes.c_int64, [_p, _p, _i, _d]),
            "om_nlist_fetch": (None, [_p, _dp, _ip, _ip]),
            "om_nlist_fetch_points": (None, [_p, _dp, _ip]),
            "om_nlist_cell_info": (None, [_p, _dp, _dp, _ip]),
            "om_flip_serial": (_i, [_p, _p, _d, ctypes.c_uint64]),
            "om_flip_parallel": (_i, [_p, _p, _d, ctypes.c_uint64]),
            "om_flip_windowed": (_i, [_p, _p, _d, ctypes.c_uint64, _i, _i]),
            "om_area": (_d, [_p]), "om_edges_length": (_d, [_p]),
            "om_fd_gradient": (None, [_p, _p, _d, _dp]),
            "om_time_energy_gradient": (_d, [_p, _p, _i]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


def set_threads(n):
    lib().om_set_threads(int(n))


def get_threads():
    return lib().om_get_threads()


class Mesh:
    def __init__(self, points, faces, _handle=None):
        L = lib()
        if _handle is not None:
            self.h = _handle
        else:
            p = np.ascontiguousarray(points, dtype=np.float64)
            f = np.ascontiguousarray(faces, dtype=np.int32)
            self.h = L.om_mesh_create(_ptr(p), len(p), _ptr(f, _ip), len(f))
            if not self.h:
                raise RuntimeError(L.om_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.om_mesh_destroy(self.h)
            self.h = None

    def clone(self):
        return Mesh(None, None, _handle=lib().om_mesh_clone(self.h))

    def n_vertices(self):
        return lib().om_mesh_nv(self.h)

    def n_edges(self):
        return lib().om_mesh_ne(self.h)

    def n_faces(self):
        return lib().om_mesh_nf(self.h)

    def points(self):
        n = self.n_vertices()
        ptr = lib().om_mesh_points(self.h)
        return np.ctypeslib.as_array(ptr, shape=(n, 3))

    def fv_indices(self):
        out = np.empty((self.n_faces(), 3), dtype=np.int32)
        lib().om_mesh_fv(self.h, _ptr(out, _ip))
        return out

    def topology(self):
        nh = 2 * self.n_edges()
        to = np.empty(nh, np.int32)
        nx = np.empty(nh, np.int32)
        fc = np.empty(nh, np.int32)
        vo = np.empty(self.n_vertices(), np.int32)
        fh = np.empty(self.n_faces(), np.int32)
        lib().om_mesh_topology(self.h, *[_ptr(a, _ip) for a in (to, nx, fc, vo, fh)])
        return {"to": to, "next": nx, "face": fc, "vout": vo, "fhe": fh}

    def check(self):
        return lib().om_mesh_check(self.h)


def prim(mesh, name, he):
    """Geometry primitive ``name`` on halfedge ``he``: (value, gradient)."""
    L = lib()
    rows = {"edge_length": 2, "face_area": 3, "face_volume": 3, "dihedral_angle": 4}[name]
    val = getattr(L, "om_" + name)(mesh.h, int(he))
    g = np.empty((rows, 3))
    getattr(L, "om_" + name + "_grad")(mesh.h, int(he), _ptr(g))
    return val, g


class Energy:
    def __init__(self, mesh, params):
        self.params = params
        self.h = lib().om_energy_create(mesh.h, ctypes.byref(params))
        if not self.h:
            raise RuntimeError(lib().om_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.om_energy_destroy(self.h)
            self.h = None

    def properties(self, mesh):
        out = np.empty(6)
        lib().om_energy_properties(self.h, mesh.h, _ptr(out))
        return out

    def vertex_properties(self, mesh):
        out = np.empty((mesh.n_vertices(), 6))
        lib().om_energy_vertex_properties(self.h, mesh.h, _ptr(out))
        return out

    def energy(self, mesh):
        return lib().om_energy_energy(self.h, mesh.h)

    def energy_props(self, props):
        p = np.ascontiguousarray(props, dtype=np.float64)
        return lib().om_energy_energy_props(self.h, _ptr(p))

    def components(self, mesh):
        out = np.empty(7)
        lib().om_energy_components(self.h, mesh.h, _ptr(out))
        return out

    def gradient(self, mesh):
        out = np.empty((mesh.n_vertices(), 3))
        lib().om_energy_gradient(self.h, mesh.h, _ptr(out))
        return out

    def update_reference_properties(self):
        lib().om_energy_update_reference(self.h)

    def update_repulsion(self, mesh):
        lib().om_energy_update_repulsion(self.h, mesh.h)

    def initial_props(self):
        out = np.empty(6)
        lib().om_energy_initial_props(self.h, _ptr(out))
        return out

    def set_initial_props(self, props6):
        p = np.ascontiguousarray(props6, dtype=np.float64)
        lib().om_energy_set_initial_props(self.h, _ptr(p))

    def ref_props(self):
        out = np.empty(6)
        lib().om_energy_ref_props(self.h, _ptr(out))
        return out

    def fd_gradient(self, mesh, eps):
        out = np.empty((mesh.n_vertices(), 3))
        lib().om_fd_gradient(mesh.h, self.h, float(eps), _ptr(out))
        return out

    def time_energy_gradient(self, mesh, n):
        return lib().om_time_energy_gradient(self.h, mesh.h, int(n))


class NList:
    def __init__(self, mesh, n_search, exclusion, rlist):
        self.h = lib().om_nlist_create(mesh.h, int(n_search), int(exclusion), float(rlist))
        if not self.h:
            raise RuntimeError(lib().om_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.om_nlist_destroy(self.h)
            self.h = None

    def distance_matrix(self, mesh, dmax):
        n = lib().om_nlist_distance_matrix(self.h, mesh.h, float(dmax))
        d = np.empty(n)
        i = np.empty(n, np.int32)
        j = np.empty(n, np.int32)
        lib().om_nlist_fetch(self.h, _ptr(d), _ptr(i, _ip), _ptr(j, _ip))
        return d, i, j

    def point_distances(self, mesh, pid, dmax):
        n = lib().om_nlist_point_distances(self.h, mesh.h, int(pid), float(dmax))
        d = np.empty((n, 3))
        j = np.empty(n, np.int32)
        lib().om_nlist_fetch_points(self.h, _ptr(d), _ptr(j, _ip))
        return d, j

    def cell_info(self):
        box = np.empty(6)
        rl = np.empty(3)
        sh = np.empty(3, np.int32)
        lib().om_nlist_cell_info(self.h, _ptr(box), _ptr(rl), _ptr(sh, _ip))
        return box, rl, sh


def flip_serial(mesh, energy, ratio, seed):
    r = lib().om_flip_serial(mesh.h, energy.h, float(ratio), int(seed))
    if r < 0:
        raise RuntimeError(lib().om_last_error().decode())
    return r


def flip_parallel(mesh, energy, ratio, seed):
    r = lib().om_flip_parallel(mesh.h, energy.h, float(ratio), int(seed))
    if r < 0:
        raise ValueError(lib().om_last_error().decode())
    return r


def flip_windowed(mesh, energy, ratio, seed, mode, batch):
    r = lib().om_flip_windowed(mesh.h, energy.h, float(ratio), int(seed), int(mode), int(batch))
    if r < 0:
        raise ValueError(lib().om_last_error().decode())
    return r


def area(mesh):
    return lib().om_area(mesh.h)


def edges_length(mesh):
    return lib().om_edges_length(mesh.h)


# ---------------------------------------------------------------------------
# HMC chain (src/trimem/mc/hmc.py:14-26 velocity Verlet, :138-165 Metropolis
# step), restated for the checks: numpy's global generator is drawn in the
# reference's order -- one normal array for the momenta, then one uniform for
# the acceptance -- so a chain started from np.random.seed(s) reproduces the
# reference's chain step for step.
# ---------------------------------------------------------------------------
def leapfrog(x, p, force, mass, dt, n):
    """n velocity-Verlet steps in position/momentum form (hmc.py:14-26)."""
    a = force(x)
    for _ in range(n):
        x = x + (p * dt + 0.5 * dt * dt * a) / mass
        a_new = force(x)
        p = p + 0.5 * dt * (a + a_new)
        a = a_new
    return x, p


def hmc_chain(x, energy, gradient, n_steps, dt, n_leapfrog, mass=1.0, temperature=1.0):
    """n_steps Metropolis-corrected HMC moves at a fixed temperature
    (hmc.py:138-165).  Returns (final state, number of accepted moves)."""
    accepted = 0
    for _ in range(n_steps):
        p = np.random.normal(size=x.shape) * np.sqrt(mass * temperature)
        xn, pn = leapfrog(x, p, lambda y: -gradient(y), mass, dt, n_leapfrog)
        h_new = energy(xn) + 0.5 * float(pn.ravel() @ pn.ravel()) / mass
        h_old = energy(x) + 0.5 * float(p.ravel() @ p.ravel()) / mass
        dh = (h_new - h_old) / temperature
        if np.random.uniform() <= (1.0 if dh <= 0 else np.exp(-dh)):
            x = xn
            accepted += 1
    return x, accepted
