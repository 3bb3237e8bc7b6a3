"""Parity of the CUDA path (called through the C ABI) with the oracle.

Tolerances: FP64 properties, energies and gradients within 1e-10 relative
(norm-wise for the gradient); neighbour pair sets, pair distances and flipped
topologies bit-exact."""
import numpy as np
import pytest

from helpers import autograd_primitives, facet_pair, unit_params, workload_params
from oracle import oracle as O
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu

RTOL = 1e-10


@pytest.fixture(scope="module")
def C(built):
    from trimem_gb300 import capi
    return capi


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("alpha", [np.pi / 4, -np.pi / 4])
def test_primitives_vs_autograd(C, alpha):
    pts, cells = facet_pair(alpha)
    m = C.Mesh(pts, cells)
    for name, (rv, rg) in autograd_primitives(pts).items():
        v, g = m.prim(name, 0)
        assert abs(v - rv) <= RTOL * max(1.0, abs(rv)), name
        assert rel(g, rg) < RTOL, name


def _pair(C, p, f, prm):
    mo = O.Mesh(p, f)
    eo = O.Energy(mo, O.default_params(**prm))
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    return mo, eo, mg, eg


CASES = [
    ("L3 cell excl2 edge", 3, dict()),
    ("L4 cell excl2 edge", 4, dict()),
    ("L3 area bonds", 3, dict(bond_type=1)),
    ("L3 verlet excl2", 3, dict(n_search=1)),
    ("L3 repulsive excl1", 3, dict(excl=1, rep_scale=1.3)),
    ("L3 repulsive excl0 verlet", 3, dict(excl=0, rep_scale=0.9, n_search=1)),
]


@pytest.mark.parametrize("stencil", [0, 2], ids=["fp64", "df64"])
@pytest.mark.parametrize("name,level,kw", CASES, ids=[c[0] for c in CASES])
def test_energy_and_gradient_parity(C, name, level, kw, stencil):
    """FP64 and double-float stencils against the oracle, 1e-10 relative."""
    p, f = meshgen.jittered_icosphere(level, seed=level)
    prm = workload_params(p, f, **kw)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    eg.set_stencil_precision(stencil)
    np.testing.assert_allclose(eg.initial_props(), eo.initial_props(), rtol=RTOL, atol=0)
    # move the vertices after construction: the cell list keeps its bins
    rng = np.random.default_rng(7)
    d = rng.normal(0, 1e-3 * meshgen.mean_edge_length(p, f), size=p.shape)
    mo.points()[:] += d
    mg.points()[:] += d
    po, pg = eo.properties(mo), eg.properties(mg)
    for k in range(6):
        assert abs(pg[k] - po[k]) <= RTOL * max(abs(po[k]), 1e-300), (k, pg[k], po[k])
    assert abs(eg.energy(mg) - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
    # the area, volume and curvature components are kappa (P/R - 1)^2: an
    # error eps in the property P moves them by about 2 kappa |P/R - 1| eps,
    # which for P close to its reference (here |P/R - 1| ~ 1e-5) exceeds
    # RTOL |component| even at eps ~ 1e-15; those three are held to the
    # error their property's stencil precision implies (1e-15 relative
    # FP64, 1e-13 double-float), the others to RTOL
    cg, co = eg.components(mg), eo.components(mo)
    eps = 1e-15 if stencil == 0 else 1e-13
    for k, kappa in enumerate([prm["kappa_a"], prm["kappa_v"], prm["kappa_c"]] + [0.0] * 4):
        x = np.sqrt(co[k] / kappa) if kappa > 0 else 0.0
        tol = RTOL * abs(co[k]) + 2.0 * kappa * x * (1.0 + x) * eps + 1e-300
        assert abs(cg[k] - co[k]) <= tol, (k, cg[k], co[k], tol)
    vo, vg = eo.vertex_properties(mo), eg.vertex_properties(mg)
    scale = np.abs(vo).max(axis=0) + 1e-300
    assert (np.abs(vg - vo) / scale).max() < RTOL
    go = eo.gradient(mo)
    eng, gg = eg.gradient(mg, with_energy=True)
    assert rel(gg, go) < RTOL
    assert abs(eng - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
    if kw.get("rep_scale", 0.8) > 1.0:
        assert po[5] > 0  # the repulsion is exercised


def test_gradient_is_deterministic(C):
    p, f = meshgen.jittered_icosphere(4, seed=1)
    prm = workload_params(p, f)
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    g1 = eg.gradient(mg)
    g2 = eg.gradient(mg)
    assert np.array_equal(g1, g2)


@pytest.mark.parametrize("bond_type", [0, 1])
def test_gradient_vs_finite_differences(C, bond_type):
    p, f = meshgen.icosphere(3)
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**unit_params(p, f, bond_type)))
    fd = eg.fd_gradient(mg, 1e-8)
    assert rel(eg.gradient(mg), fd) < 1e-4


def test_reference_state_and_continuation(C):
    p, f = meshgen.jittered_icosphere(3, seed=2)
    prm = workload_params(p, f, vfrac=0.7)
    prm.update(cont_delta=0.25, cont_lambda=0.0, area_frac=0.9, curvature_frac=0.8, kappa_c=10.0)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    for _ in range(6):
        assert abs(eg.energy(mg) - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
        assert rel(eg.gradient(mg), eo.gradient(mo)) < RTOL
        eg.update_reference_properties()
        eo.update_reference_properties()


def test_energy_of_given_properties(C):
    p, f = meshgen.jittered_icosphere(3, seed=4)
    prm = workload_params(p, f)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    props = eo.properties(mo) * 1.01
    assert abs(eg.energy_props(props) - eo.energy_props(props)) <= RTOL * abs(eo.energy_props(props))


@pytest.mark.parametrize("n_search", [0, 1])
@pytest.mark.parametrize("excl,nn", [(0, 44), (1, 38), (2, 26)])
def test_neighbour_exclusion_counts(C, n_search, excl, nn):
    p, f = meshgen.rect(20, 20)
    m = C.Mesh(p, f)
    nl = C.NList(m, C.params(n_search=n_search, exclusion_level=excl, rlist=0.2))
    _, j = nl.point_distances(m, 151, 0.2)
    assert len(j) == nn


def _pairs(d, i, j):
    o = np.lexsort((j, i))
    return np.stack([i[o], j[o]], 1), d[o]


@pytest.mark.parametrize("n_search", [0, 1])
@pytest.mark.parametrize("excl", [0, 1, 2])
@pytest.mark.parametrize("mesh", ["rect", "sphere"])
def test_pair_sets_bit_exact(C, n_search, excl, mesh):
    if mesh == "rect":
        p, f = meshgen.rect(20, 20)
        rl, rq = 0.2, 0.123
    else:
        p, f = meshgen.jittered_icosphere(4, sigma_rel=0.2, seed=5)
        l = meshgen.mean_edge_length(p, f)
        rl, rq = 2.4 * l, 2.1 * l  # beyond the 2-ring, so every exclusion level keeps pairs
    mo = O.Mesh(p, f)
    mg = C.Mesh(p, f)
    no = O.NList(mo, n_search, excl, rl)
    ng = C.NList(mg, C.params(n_search=n_search, exclusion_level=excl, rlist=rl))
    # stale bins: query with moved positions
    rng = np.random.default_rng(1)
    d = rng.normal(0, 0.2 * rl, size=p.shape)
    mo.points()[:] += d
    mg.points()[:] += d
    (po, do), (pg, dg) = _pairs(*no.distance_matrix(mo, rq)), _pairs(*ng.distance_matrix(mg, rq))
    assert len(po) > 0
    assert np.array_equal(po, pg)
    assert np.array_equal(do, dg)  # bit-identical distances
    for pid in range(0, len(p), max(1, len(p) // 37)):
        d3o, jo = no.point_distances(mo, pid, rq)
        d3g, jg = ng.point_distances(mg, pid, rq)
        assert np.array_equal(jo, jg)
        assert np.array_equal(d3o, d3g)


def _flip_case(C, level=3, kb=1.0):
    p, f = meshgen.icosphere(level)
    prm = unit_params(p, f, 0, frac=1.0)
    prm["kappa_b"] = kb
    return p, f, prm


@pytest.mark.parametrize("mode,batch", [(0, 256), (1, 64), (1, 1024)])
def test_flip_sweeps_match_cpu_port(C, mode, batch):
    p, f, prm = _flip_case(C)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    for seed in (3, 4):
        ao = O.flip_windowed(mo, eo, 0.5, seed, mode, batch)
        ag = C.flip(mg, eg, 0.5, seed, mode, batch)
        assert ag == ao
        assert mg.check() == 0 and mo.check() == 0
        tg, to = mg.topology(), mo.topology()
        for k in to:
            assert np.array_equal(tg[k], to[k]), k
        assert np.array_equal(mg.fv_indices(), mo.fv_indices())
    assert ag > 100


def test_flip_on_jittered_mesh_with_repulsion(C):
    p, f = meshgen.jittered_icosphere(4, seed=9)
    prm = workload_params(p, f, excl=1, rep_scale=1.2)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    ao = O.flip_windowed(mo, eo, 0.2, 21, 1, 512)
    ag = C.flip(mg, eg, 0.2, 21, 1, 512)
    assert ag == ao
    assert np.array_equal(mg.fv_indices(), mo.fv_indices())
    # energies on the flipped meshes agree as well (the repulsion re-tests
    # exclusions on the new topology), also after a small displacement
    assert abs(eg.energy(mg) - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
    d = np.random.default_rng(2).normal(0, 1e-3 * meshgen.mean_edge_length(p, f), size=p.shape)
    mo.points()[:] += d
    mg.points()[:] += d
    for stencil in (0, 2):
        eg.set_stencil_precision(stencil)
        eng, gg = eg.gradient(mg, with_energy=True)
        assert abs(eng - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
        assert rel(gg, eo.gradient(mo)) < RTOL


@pytest.mark.parametrize("stencil", [0, 2], ids=["fp64", "df64"])
def test_repulsion_with_cell_changes_inside_the_skin(C, stencil):
    """Every vertex moved by up to 0.45 lc1 since the cell-list build (inside
    the near rows' skin of lc1/2): many vertices are in another cell than at
    the build and are still answered from the near rows, in the reference's
    order; everything matches the oracle on the same cells."""
    p, f = meshgen.jittered_icosphere(3, seed=6)
    prm = workload_params(p, f, excl=1, rep_scale=1.3)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    eg.set_stencil_precision(stencil)
    rng = np.random.default_rng(4)
    d = rng.uniform(-1.0, 1.0, size=p.shape) * (0.45 / np.sqrt(3.0)) * prm["rep_lc1"]
    mo.points()[:] += d
    mg.points()[:] += d
    po = eo.properties(mo)
    assert po[5] > 0
    assert abs(eg.properties(mg)[5] - po[5]) <= RTOL * po[5]
    eng, gg = eg.gradient(mg, with_energy=True)
    assert abs(eng - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
    assert rel(gg, eo.gradient(mo)) < RTOL


def test_near_rows_across_cell_list_rebuilds(C):
    """The near rows outlive cell-list rebuilds while no vertex has moved
    lc1/2 from where they were built, and are rebuilt on the device when one
    has; every evaluation matches the oracle with the same cell lists."""
    p, f = meshgen.jittered_icosphere(3, seed=7)
    prm = workload_params(p, f, excl=1, rep_scale=1.3)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    rng = np.random.default_rng(9)
    lc1 = prm["rep_lc1"]
    for step, scale in enumerate([0.2, 0.2, 0.3, 0.05]):
        d = rng.uniform(-1.0, 1.0, size=p.shape) * (scale / np.sqrt(3.0)) * lc1
        mo.points()[:] += d
        mg.points()[:] += d
        if step:
            eo.update_repulsion(mo)
            eg.update_repulsion(mg)
        po = eo.properties(mo)
        assert abs(eg.properties(mg)[5] - po[5]) <= RTOL * max(po[5], 1e-300), step
        eng, gg = eg.gradient(mg, with_energy=True)
        assert abs(eng - eo.energy(mo)) <= RTOL * abs(eo.energy(mo)), step
        assert rel(gg, eo.gradient(mo)) < RTOL, step


def test_repulsion_after_a_large_move(C):
    """One vertex moved by more than half the repulsion cut-off since the
    cell-list build: the evaluation leaves the near rows for the full
    candidate rows and still matches the oracle on the same cells."""
    p, f = meshgen.jittered_icosphere(3, seed=5)
    prm = workload_params(p, f, excl=1, rep_scale=1.3)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    rng = np.random.default_rng(3)
    d = rng.normal(0, 1e-3 * meshgen.mean_edge_length(p, f), size=p.shape)
    d[17, 0] += 0.7 * prm["rep_lc1"]
    mo.points()[:] += d
    mg.points()[:] += d
    assert eo.properties(mo)[5] > 0  # pairs inside the cut-off exist
    for stencil in (0, 1, 2):
        eg.set_stencil_precision(stencil)
        tol = 1e-5 if stencil == 1 else RTOL
        eng, gg = eg.gradient(mg, with_energy=True)
        assert abs(eng - eo.energy(mo)) <= tol * abs(eo.energy(mo)), stencil
        assert rel(gg, eo.gradient(mo)) < tol * 10, stencil
        assert abs(eg.properties(mg)[5] - eo.properties(mo)[5]) <= RTOL * eo.properties(mo)[5], stencil


def test_flip_ratio_errors(C):
    p, f, prm = _flip_case(C)
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    with pytest.raises(C.TMError) as ei:
        C.flip(mg, eg, 1.5, 1, 1)
    assert ei.value.code == C.TM_ERR_RANGE


def test_utilities(C):
    p, f = meshgen.jittered_icosphere(4, seed=3)
    mo, mg = O.Mesh(p, f), C.Mesh(p, f)
    assert abs(mg.area() - O.area(mo)) <= RTOL * O.area(mo)
    assert abs(mg.edges_length() - O.edges_length(mo)) <= RTOL * O.edges_length(mo)
    a, l = mg.avg_tri_props()
    assert abs(a - O.area(mo) / mo.n_faces()) <= RTOL * a


@pytest.mark.parametrize("stencil", [0, 2], ids=["fp64", "df64"])
def test_large_mesh_properties(C, stencil):
    """Level-6 icosphere (40,962 vertices): parity with the oracle and the
    size-independent invariances (closed surface: translation leaves the
    energy unchanged, so the gradient sums to zero)."""
    p, f = meshgen.jittered_icosphere(6, seed=0)
    prm = workload_params(p, f)
    mo, eo, mg, eg = _pair(C, p, f, prm)
    eg.set_stencil_precision(stencil)
    e, g = eg.gradient(mg, with_energy=True)
    assert abs(e - eo.energy(mo)) <= RTOL * abs(e)
    assert rel(g, eo.gradient(mo)) < RTOL
    assert np.linalg.norm(g.sum(0)) < 1e-8 * np.linalg.norm(g)


def test_fp32_stencil_error_bounds(C):
    """FP32-stencil variant: local geometry in FP32, global sums FP64.  Its
    error against the FP64 result is bounded per quantity (energy and global
    properties 1e-5 relative, gradient 1e-4 relative norm-wise)."""
    p, f = meshgen.jittered_icosphere(5, seed=2)
    prm = workload_params(p, f, excl=1, rep_scale=1.2)
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    eg.set_stencil_precision(0)
    e64, g64 = eg.gradient(mg, with_energy=True)
    p64 = eg.properties(mg)
    eg.set_stencil_precision(1)
    e32, g32 = eg.gradient(mg, with_energy=True)
    p32 = eg.properties(mg)
    eg.set_stencil_precision(0)
    assert np.array_equal(eg.gradient(mg), g64)  # switching back restores FP64
    assert abs(e32 - e64) <= 1e-5 * abs(e64)
    for k in range(6):
        assert abs(p32[k] - p64[k]) <= 1e-5 * max(abs(p64[k]), 1e-12), k
    assert rel(g32, g64) < 1e-4


def test_annealing_run_with_continuation(C):
    """A continuation (annealing) run on the device, as the reference's
    HMC callback drives it (src/trimem/mc/hmc.py:174-177, src/energy.cpp:30-55):
    a device chain with flips, the reference properties advanced every five
    steps until lambda reaches 1, area difference on (kc 10).  At the end the
    device energy and gradient of the final (moved and flipped) membrane
    match the oracle's, whose reference properties come from the same
    initial state and the same number of continuation updates."""
    import torch

    from trimem_gb300.mc.device import DeviceChain

    p, f = meshgen.jittered_icosphere(3, seed=6)
    prm = workload_params(p, f, vfrac=0.8)
    prm.update(cont_delta=0.1, cont_lambda=0.0, area_frac=0.95, curvature_frac=0.9, kappa_c=10.0)
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    mo0 = O.Mesh(p, f)
    eo = O.Energy(mo0, O.default_params(**prm))
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    ch = DeviceChain(mg, eg, x, dt=1e-6, n_leapfrog=10, flip_ratio=0.2, seed=8)
    for _ in range(12):
        ch.run(5)
        eg.update_reference_properties()
        eo.update_reference_properties()
    assert eg.params().cont_lambda >= 1.0 and ch.flips > 0
    xf = ch.x.cpu().numpy()
    mg.points()[:] = xf
    mo = O.Mesh(xf, mg.fv_indices())
    eo.update_repulsion(mo)
    eg.update_repulsion(mg)
    assert abs(eg.energy(mg) - eo.energy(mo)) <= RTOL * abs(eo.energy(mo))
    assert rel(eg.gradient(mg), eo.gradient(mo)) < RTOL
