"""The reference's own test-suite (tests/*.py of bio-phys/trimem) restated on
the drop-in module ``trimem_gb300.core``, plus its error behaviour."""
import json
import os

import numpy as np
import pytest

from helpers import autograd_primitives, facet_pair
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def m(built):
    from trimem_gb300 import load_core
    return load_core()


@pytest.mark.parametrize("alpha", [np.pi / 4, -np.pi / 4])
def test_properties_module(m, alpha):
    pts, cells = facet_pair(alpha)
    mesh = m.TriMesh(pts, cells)
    e = mesh.halfedge_handle(0)
    ref = autograd_primitives(pts)
    for name in ["edge_length", "face_area", "face_volume", "dihedral_angle"]:
        v = getattr(m, name)(mesh, e)
        g = getattr(m, name + "_grad")(mesh, e)
        rv, rg = ref[name]
        assert abs(v - rv) < 1e-10 * max(1, abs(rv))
        assert np.linalg.norm(g - rg) / np.linalg.norm(rg) < 1e-10


@pytest.mark.parametrize("name,r", [("sphere", 1.0), ("sphere", 0.5), ("tube", 1.0), ("tube", 0.5)])
def test_energy_module(m, name, r):
    if name == "sphere":
        p, f = meshgen.icosphere(5)
        mesh = m.TriMesh(p * r, f)
        ref = (4 * np.pi * r**2, 4 / 3 * np.pi * r**3, 4 * np.pi * r, 8 * np.pi)
    else:
        p, f = meshgen.tube(length=1, radius=r, segments=32)
        mesh = m.TriMesh(p, f)
        ref = (2 * np.pi * r, 2 / 3 * np.pi * r**2, np.pi, np.pi / r)
    estore = m.EnergyManager(mesh, m.EnergyParams())
    pr = estore.properties(mesh)
    for v, rv in zip((pr.area, pr.volume, pr.curvature, pr.bending), ref):
        assert abs(v - rv) / rv < 1e-2


def _estore(m, mesh, bond_type, frac=0.8):
    a, l = m.avg_tri_props(mesh)
    bp = m.BondParams()
    bp.type = bond_type
    bp.lc0 = 1.15 * l
    bp.lc1 = 0.85 * l
    bp.a0 = a
    ep = m.EnergyParams()
    ep.kappa_b = ep.kappa_a = ep.kappa_v = ep.kappa_c = ep.kappa_t = 1.0
    ep.area_frac = ep.volume_frac = ep.curvature_frac = frac
    ep.bond_params = bp
    return m.EnergyManager(mesh, ep)


@pytest.mark.parametrize("bt", ["Edge", "Area"])
def test_gradient_module(m, bt):
    p, f = meshgen.icosphere(3)
    mesh = m.TriMesh(p, f)
    estore = _estore(m, mesh, getattr(m.BondType, bt))
    ref = np.empty((mesh.n_vertices(), 3))
    m.gradient(mesh, estore, ref, 1.0e-8)
    g = estore.gradient(mesh)
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 1.0e-4


@pytest.mark.parametrize("ltype", ["cell-list", "verlet-list"])
def test_neighbours_module(m, ltype):
    from scipy.sparse import coo_matrix
    from scipy.spatial import KDTree

    p, f = meshgen.rect(20, 20)
    mesh = m.TriMesh(p, f)
    x = mesh.points()
    for rlist in (0.2, 0.5, 1.2):
        params = m.EnergyParams()
        params.repulse_params.n_search = ltype
        params.repulse_params.rlist = rlist
        params.repulse_params.exclusion_level = 0
        nl = m.make_nlist(mesh, params)
        d, i, j = nl.distance_matrix(mesh, 0.123)
        M = coo_matrix((d, (i, j)), shape=(len(x), len(x)))
        if ltype == "cell-list":
            M = M + M.T
        T = KDTree(x)
        assert np.allclose(T.sparse_distance_matrix(T, 0.123).todense(), M.todense())
    for excl, nn in ((0, 44), (1, 38), (2, 26)):
        params = m.EnergyParams()
        params.repulse_params.n_search = ltype
        params.repulse_params.rlist = 0.2
        params.repulse_params.exclusion_level = excl
        _, jdx = m.make_nlist(mesh, params).point_distances(mesh, 151, 0.2)
        assert len(jdx) == nn


@pytest.mark.parametrize("fn", ["flip", "pflip"])
def test_flips_module(m, fn):
    p, f = meshgen.icosphere(3)
    mesh = m.TriMesh(p, f)
    estore = _estore(m, mesh, m.BondType.Edge, frac=1.0)
    acc = getattr(m, fn)(mesh, estore, 0.5)
    assert acc > 100
    assert mesh.check() == 0
    assert len(np.unique(np.sort(mesh.fv_indices(), axis=1), axis=0)) == mesh.fv_indices().shape[0]


def test_points_view_is_zero_copy(m):
    p, f = meshgen.icosphere(2)
    mesh = m.TriMesh(p, f)
    x = mesh.points()
    assert x.base is not None
    x[0, 0] += 0.25
    assert mesh.points()[0, 0] == x[0, 0]
    assert np.array_equal(mesh.fv_indices(), f)


def test_errors_match_reference(m):
    with pytest.raises(RuntimeError):
        m.TriMesh(np.zeros((4, 2)), np.zeros((1, 3), np.int32))
    with pytest.raises(RuntimeError):
        m.TriMesh(np.zeros((4, 3)), np.zeros((1, 4), np.int32))
    p, f = meshgen.icosphere(2)
    mesh = m.TriMesh(p, f)
    ep = m.EnergyParams()
    ep.repulse_params.n_search = "kd-tree"
    with pytest.raises(RuntimeError):
        m.make_nlist(mesh, ep)
    ep = m.EnergyParams()
    ep.repulse_params.exclusion_level = 3
    with pytest.raises(RuntimeError):
        m.EnergyManager(mesh, ep)
    ep = m.EnergyParams()
    ep.bond_params.type = getattr(m.BondType, "None")
    with pytest.raises(RuntimeError):
        m.EnergyManager(mesh, ep)
    estore = m.EnergyManager(mesh, m.EnergyParams())
    with pytest.raises(ValueError):
        m.pflip(mesh, estore, 1.5)
    # out-of-range face entries are dropped, like the reference
    mesh2 = m.TriMesh(p, np.vstack([f, [[0, 1, 10**6]]]).astype(np.int32))
    assert mesh2.fv_indices().shape == f.shape


def test_energy_manager_state(m):
    p, f = meshgen.icosphere(3)
    mesh = m.TriMesh(p, f)
    ep = m.EnergyParams()
    ep.kappa_b = 1.0
    ep.continuation_params.delta = 0.5
    ep.continuation_params.lam = 0.0
    estore = m.EnergyManager(mesh, ep)
    ip = estore.initial_props
    assert ip.area == pytest.approx(4 * np.pi, rel=1e-2)
    assert estore.eparams.continuation_params.lam == 0.0
    estore.update_reference_properties()
    assert estore.eparams.continuation_params.lam == 0.5
    vp = estore.properties(mesh)
    assert estore.energy(vp) == pytest.approx(estore.energy(mesh), rel=1e-14)
    estore.update_repulsion(mesh)
    estore.print_info(mesh)
