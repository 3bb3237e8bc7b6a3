"""Energy parameters of the benchmark membranes (the large-mesh runs of the
reference: smooth tether, flat-bottom repulsion via the cell list)."""
import numpy as np

from . import meshgen


def mesh_stats(p, f):
    """(mean face area, mean edge length), as avg_tri_props."""
    a = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    area = 0.5 * np.linalg.norm(a, axis=1).mean()
    return area, meshgen.mean_edge_length(p, f)


def workload_params(p, f, kappa_b=30.0, vfrac=0.8, bond_type=0, n_search=0, excl=2, rep_scale=0.8):
    """Parameters of the benchmark workloads (kb 30, ka 1e6, kv 1e6, kc 0,
    kt 1e5, kr 1e3, smooth tether lc0 1.15 l / lc1 0.85 l, repulsion cut-off
    rep_scale * l via the neighbour list, exclusion 2, target volume vfrac)."""
    a, l = mesh_stats(p, f)
    return dict(kappa_b=kappa_b, kappa_a=1e6, kappa_v=1e6, kappa_c=0.0, kappa_t=1e5, kappa_r=1e3,
                area_frac=1.0, volume_frac=vfrac, curvature_frac=1.0,
                bond_lc0=1.15 * l, bond_lc1=0.85 * l, bond_a0=a, bond_r=2, bond_type=bond_type,
                rep_lc1=rep_scale * l, rep_r=2, n_search=n_search, rlist=rep_scale * l, exclusion_level=excl,
                cont_delta=0.0, cont_lambda=1.0)


def very_large_mesh():
    """The 163,842-vertex membrane (level-7 icosphere, jitter seed 0) with the
    very-large-mesh energy: kb 20, reduced-volume target 0.65, the other
    parameters as workload_params.  Returns (points, faces, params)."""
    p, f = meshgen.jittered_icosphere(7, seed=0)
    return p, f, workload_params(p, f, kappa_b=20.0, vfrac=0.65)


def small_mesh():
    """The CPU-sized membrane: level-4 icosphere (2,562 vertices), vertices
    jittered by N(0, 0.01) (seed 0), workload_params (kb 30, volume target
    0.8).  Returns (points, faces, params)."""
    p, f = meshgen.jittered_icosphere(4, seed=0)
    return p, f, workload_params(p, f)
