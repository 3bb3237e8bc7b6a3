"""Shared inputs of the parity tests: meshes and energy parameters of the
workloads, for the oracle (oracle.Params) and the product (capi.Params)."""
import numpy as np

from trimem_gb300 import meshgen
from trimem_gb300.workloads import mesh_stats, workload_params  # noqa: F401  (shared with bench.py)


def unit_params(p, f, bond_type=0, frac=0.8):
    """All kappa 1, fractions 0.8 (the reference's gradient test)."""
    a, l = mesh_stats(p, f)
    return dict(kappa_b=1.0, kappa_a=1.0, kappa_v=1.0, kappa_c=1.0, kappa_t=1.0, kappa_r=0.0,
                area_frac=frac, volume_frac=frac, curvature_frac=frac,
                bond_lc0=1.15 * l, bond_lc1=0.85 * l, bond_a0=a, bond_r=2, bond_type=bond_type,
                rep_lc1=0.0, rep_r=2, n_search=0, rlist=0.1, exclusion_level=2, cont_delta=0.0, cont_lambda=1.0)


def facet_pair(alpha):
    """Two triangles sharing edge (0,1) at dihedral +-pi/4 (the reference's
    primitive test geometry)."""
    x = np.cos(alpha) * 0.5
    z = np.sin(alpha) * 0.5
    pts = np.array([[0.0, -0.5, 0.0], [0.0, 0.5, 0.0], [-x, 0.0, z], [x, 0.0, z]])
    cells = np.array([[0, 1, 2], [1, 0, 3]], dtype=np.int32)
    return pts, cells


def autograd_primitives(pts):
    """Values and gradients of edge length, face area, face volume and
    dihedral angle of halfedge 0 (0 -> 1) by torch autograd in float64."""
    import torch

    def fnu(p):
        return torch.linalg.cross(p[0] - p[1], p[2] - p[1])

    def dih(p):
        n0 = fnu(p[[0, 1, 2]])
        n1 = fnu(p[[1, 0, 3]])
        n0 = n0 / n0.norm()
        n1 = n1 / n1.norm()
        sgn = torch.dot(torch.linalg.cross(n0, n1), p[1] - p[0])
        a = torch.arccos(torch.dot(n0, n1))
        return a if sgn > 0 else -a

    funcs = {
        "edge_length": (lambda p: (p[1] - p[0]).norm(), [0, 1]),
        "face_area": (lambda p: fnu(p).norm() / 2, [0, 1, 2]),
        "face_volume": (lambda p: torch.dot(p[0], torch.linalg.cross(p[1], p[2])) / 6, [0, 1, 2]),
        "dihedral_angle": (dih, [0, 1, 2, 3]),
    }
    out = {}
    for name, (f, idx) in funcs.items():
        q = torch.tensor(pts[idx], dtype=torch.float64, requires_grad=True)
        v = f(q)
        (g,) = torch.autograd.grad(v, q)
        out[name] = (v.item(), g.numpy())
    return out


def canonical_faces(fv):
    """Face set independent of face order and vertex rotation."""
    f = np.sort(np.asarray(fv), axis=1)
    return f[np.lexsort(f.T[::-1])]
