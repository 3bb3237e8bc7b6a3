"""ctypes binding of the C ABI (``include/trimem_gpu.h``).

This is the boundary a non-Python host binds; the tests use it to drive the
library exactly the way such a host would.
"""
import ctypes
import os
import re

import numpy as np

from . import LIB_PATH, PKG_DIR

HEADER = os.path.join(os.path.dirname(PKG_DIR), "include", "trimem_gpu.h")

TM_OK = 0
TM_ERR_ARG = -1
TM_ERR_CUDA = -2
TM_ERR_TOPOLOGY = -3
TM_ERR_RANGE = -4
TM_ERR_TIMEOUT = -5
TM_ERR_NOMEM = -6
TM_MAXVAL = 32

_d = ctypes.c_double
_p = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f32 = ctypes.c_float
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_pp = ctypes.POINTER(ctypes.c_void_p)


class Params(ctypes.Structure):
    """``tm_params``: EnergyParams flattened (src/params.h:11-71)."""
    _fields_ = [
        ("kappa_b", _d), ("kappa_a", _d), ("kappa_v", _d), ("kappa_c", _d), ("kappa_t", _d), ("kappa_r", _d),
        ("area_frac", _d), ("volume_frac", _d), ("curvature_frac", _d),
        ("bond_lc0", _d), ("bond_lc1", _d), ("bond_a0", _d),
        ("bond_r", _i32), ("bond_type", _i32),
        ("rep_lc1", _d), ("rep_r", _i32), ("n_search", _i32),
        ("rlist", _d), ("exclusion_level", _i32), ("pad0", _i32),
        ("cont_delta", _d), ("cont_lambda", _d),
    ]


def params(**kw):
    """tm_params with the reference's defaults, overridden by ``kw``."""
    p = Params(kappa_b=0, kappa_a=0, kappa_v=0, kappa_c=0, kappa_t=0, kappa_r=0,
               area_frac=1, volume_frac=1, curvature_frac=1,
               bond_lc0=1, bond_lc1=0, bond_a0=1, bond_r=2, bond_type=0,
               rep_lc1=0, rep_r=2, n_search=0, rlist=0.1, exclusion_level=2,
               cont_delta=0, cont_lambda=1)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


_SIGS = {
    "tm_last_error": (ctypes.c_char_p, []),
    "tm_device_name": (_i32, [ctypes.c_char_p, _i32]),
    "tm_host_alloc": (_i32, [_i64, _pp]),
    "tm_host_free": (_i32, [_p]),
    "tm_mesh_create": (_i32, [_dp, _i64, _ip, _i64, _pp]),
    "tm_mesh_destroy": (_i32, [_p]),
    "tm_mesh_counts": (_i32, [_p, _i64p, _i64p, _i64p]),
    "tm_mesh_points": (_dp, [_p]),
    "tm_mesh_fv_indices": (_i32, [_p, _ip]),
    "tm_mesh_halfedge": (_i32, [_p, _i32, _i64, _i64p]),
    "tm_mesh_topology": (_i32, [_p, _ip, _ip, _ip, _ip, _ip]),
    "tm_mesh_check": (_i32, [_p, _ip]),
    "tm_edge_length": (_i32, [_p, _i64, _dp, _dp]),
    "tm_face_area": (_i32, [_p, _i64, _dp, _dp]),
    "tm_face_volume": (_i32, [_p, _i64, _dp, _dp]),
    "tm_dihedral_angle": (_i32, [_p, _i64, _dp, _dp]),
    "tm_energy_create": (_i32, [_p, ctypes.POINTER(Params), _pp]),
    "tm_energy_destroy": (_i32, [_p]),
    "tm_energy_get_params": (_i32, [_p, ctypes.POINTER(Params)]),
    "tm_energy_initial_props": (_i32, [_p, _dp]),
    "tm_energy_properties": (_i32, [_p, _p, _dp]),
    "tm_energy_vertex_properties": (_i32, [_p, _p, _dp]),
    "tm_energy_energy": (_i32, [_p, _p, _dp]),
    "tm_energy_energy_props": (_i32, [_p, _dp, _dp]),
    "tm_energy_components": (_i32, [_p, _p, _dp]),
    "tm_energy_gradient": (_i32, [_p, _p, _dp, _dp]),
    "tm_energy_update_reference_properties": (_i32, [_p]),
    "tm_energy_update_repulsion": (_i32, [_p, _p]),
    "tm_energy_set_stencil_precision": (_i32, [_p, _i32]),
    "tm_energy_eval_device": (_i32, [_p, _p, _p, _p, _p, _p]),
    "tm_energy_update_repulsion_device": (_i32, [_p, _p, _p, _p]),
    "tm_energy_eval_timed": (_i32, [_p, _p, _p, _p, ctypes.POINTER(ctypes.c_float), _p]),
    "tm_energy_eval_device_noalloc": (_i32, [_p, _p, _p, _p, _p, _p]),
    "tm_nlist_create": (_i32, [_p, ctypes.POINTER(Params), _pp]),
    "tm_nlist_destroy": (_i32, [_p]),
    "tm_nlist_distance_matrix": (_i32, [_p, _p, _d, _i64p]),
    "tm_nlist_point_distances": (_i32, [_p, _p, _i64, _d, _i64p]),
    "tm_nlist_fetch": (_i32, [_p, _dp, _ip, _ip]),
    "tm_flip": (_i32, [_p, _p, _d, ctypes.c_uint64, _i32, _i32, _ip]),
    "tm_flip_device": (_i32, [_p, _p, _p, _d, ctypes.c_uint64, _i32, _i32, _ip, _p]),
    "tm_area": (_i32, [_p, _dp]),
    "tm_edges_length": (_i32, [_p, _dp]),
    "tm_avg_tri_props": (_i32, [_p, _dp, _dp]),
    "tm_fd_gradient": (_i32, [_p, _p, _d, _dp]),
    "tm_hmc_step_device": (_i32, [_p, _p, _p, _d, _d, _i32, _d, ctypes.c_uint64, ctypes.c_uint64, _d, _dp, _dp, _p]),
    "tm_batch_create": (_i32, [_i32, ctypes.POINTER(_dp), _i64p, ctypes.POINTER(_ip), _i64p, ctypes.POINTER(Params), _pp]),
    "tm_batch_destroy": (_i32, [_p]),
    "tm_batch_layout": (_i32, [_p, _i64p, _i64p]),
    "tm_batch_positions": (_i32, [_p, _dp, _i32]),
    "tm_batch_energy": (_i32, [_p, _dp, _dp]),
    "tm_batch_update_repulsion": (_i32, [_p]),
    "tm_batch_hmc": (_i32, [_p, _i32, _i32, _d, _d, _d, ctypes.c_uint64, _i32, _ip]),
    "tm_batch_set_refresh": (_i32, [_p, _i32]),
    "tm_energy_set_initial_props": (_i32, [_p, _dp]),
    "tm_mesh_set_topology": (_i32, [_p, _ip, _ip, _ip, _ip, _ip]),
    "tm_minimize_device": (_i32, [_p, _p, _p, _i32, _i32, _d, _d, _ip, _dp, _p]),
    "tm_surrogate_create": (_i32, [_p, ctypes.POINTER(ctypes.c_float), _i64, _pp]),
    "tm_surrogate_destroy": (_i32, [_p]),
    "tm_surrogate_gradient_device": (_i32, [_p, _p, _p, _p, _p, _p]),
    "tm_surrogate_inputs_device": (_i32, [_p, _p, _p, _p, _i32, _p, _p, _p, _p, _p, _p, _p]),
    "tm_surrogate_hmc_step_device": (_i32, [_p, _p, _p, _p, _d, _d, _i32, _d, ctypes.c_uint64, ctypes.c_uint64, _d,
                                            _dp, _dp, _p]),
    "tm_dense_silu_bf16": (_i32, [_p, _p, _p, _p, _p, _i64, _p]),
    "tm_dense_silu_bf16_bounded": (_i32, [_p, _p, _p, _p, _p, _i64, _i32, _p]),
    "tm_surrogate_train_create": (_i32, [_i64, _i32, _p, _i64, _p]),
    "tm_surrogate_train_destroy": (_i32, [_p]),
    "tm_surrogate_train_get_weights": (_i32, [_p, _p, _i64]),
    "tm_surrogate_train_grad": (_i32, [_p, _p, _p, _p, _p, _p, _p, _i64, _i32, _f32, _p, _p, _p, _p]),
    "tm_surrogate_train_step": (_i32, [_p, _p, _p, _p, _p, _p, _p, _i64, _i32, _f32, _f32, _f32, _f32, _f32, _p,
                                       _p]),
    "tm_surrogate_train_status": (_i32, [_p]),
    "tm_batch_tuning": (_i32, [_p, _p, _p]),
}

_lib = None


def header_functions():
    """Names of the functions declared in include/trimem_gpu.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(tm_\w+)\(", txt, flags=re.M)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is not built")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class TMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(rc):
    if rc != TM_OK:
        raise TMError(rc, lib().tm_last_error().decode())


def _dptr(a):
    return a.ctypes.data_as(_dp)


def _iptr(a):
    return a.ctypes.data_as(_ip)


class Mesh:
    """tm_mesh handle."""

    def __init__(self, points, faces):
        p = np.ascontiguousarray(points, dtype=np.float64)
        f = np.ascontiguousarray(faces, dtype=np.int32)
        h = ctypes.c_void_p()
        check(lib().tm_mesh_create(_dptr(p), len(p), _iptr(f), len(f), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().tm_mesh_destroy(self.h)
            self.h = None

    __del__ = close

    def counts(self):
        a, b, c = _i64(), _i64(), _i64()
        check(lib().tm_mesh_counts(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def points(self):
        nv = self.counts()[0]
        return np.ctypeslib.as_array(lib().tm_mesh_points(self.h), shape=(nv, 3))

    def fv_indices(self):
        out = np.empty((self.counts()[2], 3), np.int32)
        check(lib().tm_mesh_fv_indices(self.h, _iptr(out)))
        return out

    def topology(self):
        nv, ne, nf = self.counts()
        arrs = [np.empty(2 * ne, np.int32) for _ in range(3)] + [np.empty(nv, np.int32), np.empty(nf, np.int32)]
        check(lib().tm_mesh_topology(self.h, *[_iptr(a) for a in arrs]))
        return dict(zip(["to", "next", "face", "vout", "fhe"], arrs))

    def set_topology(self, topo):
        """Connectivity from half-edge arrays (the dict ``topology`` returns)."""
        arrs = [np.ascontiguousarray(topo[k], dtype=np.int32) for k in ["to", "next", "face", "vout", "fhe"]]
        nv, ne, nf = self.counts()
        if [len(a) for a in arrs] != [2 * ne] * 3 + [nv, nf]:
            raise ValueError("topology arrays do not match the mesh sizes")
        check(lib().tm_mesh_set_topology(self.h, *[_iptr(a) for a in arrs]))

    def check(self):
        s = ctypes.c_int32()
        check(lib().tm_mesh_check(self.h, ctypes.byref(s)))
        return s.value

    def prim(self, name, he):
        rows = {"edge_length": 2, "face_area": 3, "face_volume": 3, "dihedral_angle": 4}[name]
        v = _d()
        g = np.empty((rows, 3))
        check(getattr(lib(), "tm_" + name)(self.h, int(he), ctypes.byref(v), _dptr(g)))
        return v.value, g

    def area(self):
        v = _d()
        check(lib().tm_area(self.h, ctypes.byref(v)))
        return v.value

    def edges_length(self):
        v = _d()
        check(lib().tm_edges_length(self.h, ctypes.byref(v)))
        return v.value

    def avg_tri_props(self):
        a, l = _d(), _d()
        check(lib().tm_avg_tri_props(self.h, ctypes.byref(a), ctypes.byref(l)))
        return a.value, l.value


class Energy:
    """tm_energy handle (EnergyManager)."""

    def __init__(self, mesh, prm):
        h = ctypes.c_void_p()
        check(lib().tm_energy_create(mesh.h, ctypes.byref(prm), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().tm_energy_destroy(self.h)
            self.h = None

    __del__ = close

    def properties(self, mesh):
        out = np.empty(6)
        check(lib().tm_energy_properties(self.h, mesh.h, _dptr(out)))
        return out

    def vertex_properties(self, mesh):
        out = np.empty((mesh.counts()[0], 6))
        check(lib().tm_energy_vertex_properties(self.h, mesh.h, _dptr(out)))
        return out

    def energy(self, mesh):
        v = _d()
        check(lib().tm_energy_energy(self.h, mesh.h, ctypes.byref(v)))
        return v.value

    def energy_props(self, props):
        p = np.ascontiguousarray(props, dtype=np.float64)
        v = _d()
        check(lib().tm_energy_energy_props(self.h, _dptr(p), ctypes.byref(v)))
        return v.value

    def components(self, mesh):
        out = np.empty(7)
        check(lib().tm_energy_components(self.h, mesh.h, _dptr(out)))
        return out

    def gradient(self, mesh, with_energy=False):
        out = np.empty((mesh.counts()[0], 3))
        e = _d()
        check(lib().tm_energy_gradient(self.h, mesh.h, _dptr(out), ctypes.byref(e)))
        return (e.value, out) if with_energy else out

    def initial_props(self):
        out = np.empty(6)
        check(lib().tm_energy_initial_props(self.h, _dptr(out)))
        return out

    def set_initial_props(self, props6):
        v = np.ascontiguousarray(props6, dtype=np.float64)
        if v.shape != (6,):
            raise ValueError("six initial properties expected")
        check(lib().tm_energy_set_initial_props(self.h, _dptr(v)))

    def params(self):
        out = Params()
        check(lib().tm_energy_get_params(self.h, ctypes.byref(out)))
        return out

    def update_reference_properties(self):
        check(lib().tm_energy_update_reference_properties(self.h))

    def update_repulsion(self, mesh):
        check(lib().tm_energy_update_repulsion(self.h, mesh.h))

    def set_stencil_precision(self, mode):
        check(lib().tm_energy_set_stencil_precision(self.h, int(mode)))
        self.stencil = int(mode)

    def fd_gradient(self, mesh, eps):
        out = np.empty((mesh.counts()[0], 3))
        check(lib().tm_fd_gradient(mesh.h, self.h, float(eps), _dptr(out)))
        return out


class NList:
    def __init__(self, mesh, prm):
        h = ctypes.c_void_p()
        check(lib().tm_nlist_create(mesh.h, ctypes.byref(prm), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().tm_nlist_destroy(self.h)
            self.h = None

    __del__ = close

    def distance_matrix(self, mesh, rdist):
        n = _i64()
        check(lib().tm_nlist_distance_matrix(self.h, mesh.h, float(rdist), ctypes.byref(n)))
        d = np.empty(n.value)
        i = np.empty(n.value, np.int32)
        j = np.empty(n.value, np.int32)
        check(lib().tm_nlist_fetch(self.h, _dptr(d), _iptr(i), _iptr(j)))
        return d, i, j

    def point_distances(self, mesh, pid, rdist):
        n = _i64()
        check(lib().tm_nlist_point_distances(self.h, mesh.h, int(pid), float(rdist), ctypes.byref(n)))
        d = np.empty((n.value, 3))
        j = np.empty(n.value, np.int32)
        check(lib().tm_nlist_fetch(self.h, _dptr(d), None, _iptr(j)))
        return d, j


class Batch:
    """tm_batch handle: replicas evaluated and sampled together."""

    def __init__(self, meshes, params_list):
        R = len(meshes)
        self._pts = [np.ascontiguousarray(p, dtype=np.float64) for p, _ in meshes]
        self._fcs = [np.ascontiguousarray(f, dtype=np.int32) for _, f in meshes]
        pp = (_dp * R)(*[_dptr(a) for a in self._pts])
        fp = (_ip * R)(*[_iptr(a) for a in self._fcs])
        npts = (_i64 * R)(*[len(a) for a in self._pts])
        nfcs = (_i64 * R)(*[len(a) for a in self._fcs])
        prm = (Params * R)(*params_list)
        h = ctypes.c_void_p()
        check(lib().tm_batch_create(R, pp, npts, fp, nfcs, prm, ctypes.byref(h)))
        self.h = h
        self.R = R
        n = _i64()
        off = (_i64 * (R + 1))()
        check(lib().tm_batch_layout(self.h, ctypes.byref(n), off))
        self.n_total = n.value
        self.offsets = np.array(off[:], dtype=np.int64)
        self.sizes = [len(a) for a in self._pts]

    def close(self):
        if getattr(self, "h", None):
            lib().tm_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def positions(self):
        x = np.empty((self.n_total, 3))
        check(lib().tm_batch_positions(self.h, _dptr(x), 0))
        return [x[o:o + n] for o, n in zip(self.offsets[:-1], self.sizes)]

    def set_positions(self, xs):
        x = np.zeros((self.n_total, 3))
        for o, n, xi in zip(self.offsets[:-1], self.sizes, xs):
            x[o:o + n] = xi
        check(lib().tm_batch_positions(self.h, _dptr(x), 1))

    def energy(self, with_grad=False):
        e = np.empty(self.R)
        g = np.empty((self.n_total, 3)) if with_grad else None
        check(lib().tm_batch_energy(self.h, _dptr(e), _dptr(g) if with_grad else None))
        if with_grad:
            return e, [g[o:o + n] for o, n in zip(self.offsets[:-1], self.sizes)]
        return e

    def update_repulsion(self):
        check(lib().tm_batch_update_repulsion(self.h))

    def tuning(self):
        """Size classes: (first vertex, end vertex, block sizes of the split,
        face, edge and gradient kernels) per class."""
        n = ctypes.c_int32()
        info = (ctypes.c_int32 * (6 * 8))()
        check(lib().tm_batch_tuning(self.h, ctypes.byref(n), info))
        return [tuple(int(v) for v in info[6 * c:6 * c + 6]) for c in range(n.value)]

    def hmc(self, n_steps, n_leapfrog, dt, mass=1.0, temperature=1.0, seed=0, use_graph=True, refresh=None):
        """n_steps HMC steps of every replica; accepted steps per replica.
        refresh: rebuild the neighbour list after every refresh-th step
        (0: never; None keeps the current setting, initially 1)."""
        if refresh is not None:
            check(lib().tm_batch_set_refresh(self.h, int(refresh)))
        acc = np.zeros(self.R, np.int32)
        check(lib().tm_batch_hmc(self.h, int(n_steps), int(n_leapfrog), float(dt), float(mass),
                                 float(temperature), int(seed), int(bool(use_graph)), _iptr(acc)))
        return acc


class Surrogate:
    """tm_surrogate handle: the learned force model of a mesh (weights: the
    float32 blob of trimem_gb300.surrogate)."""

    def __init__(self, mesh, weights):
        w = np.ascontiguousarray(weights, dtype=np.float32)
        h = ctypes.c_void_p()
        check(lib().tm_surrogate_create(mesh.h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(w),
                                        ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().tm_surrogate_destroy(self.h)
            self.h = None

    __del__ = close


def flip(mesh, energy, ratio, seed, mode, batch=256):
    acc = ctypes.c_int32()
    check(lib().tm_flip(mesh.h, energy.h, float(ratio), int(seed), int(mode), int(batch), ctypes.byref(acc)))
    return acc.value
