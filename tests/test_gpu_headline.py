"""Parity at the benchmarked configurations, through the C ABI.

* The 163,842-vertex membrane of the throughput benchmark (level-7
  icosphere, jitter seed 0, kb 20, reduced-volume target 0.65, cell list,
  exclusion 2): energy, global and per-vertex properties and gradient
  against the oracle within 1e-10 relative, with the FP64 and the
  double-float stencils, at the constructed state and after moving vertices
  and rebuilding the neighbour list (src/energy.cpp:79-124).
* One parallel flip sweep (ratio 0.2) of that membrane: the accept count and
  the flipped topology equal the oracle's port of the windowed sweep with the
  same seed, and the mesh stays a valid closed manifold (src/flips.cpp:82-165).
* The CPU-sized run: 2,562-vertex membrane (level 4, N(0, 0.01) jitter),
  1,000 hybrid steps of 20 velocity-Verlet steps at dt 1e-4 plus a parallel
  flip sweep of ratio 0.1, energy and gradient against the oracle at step 0
  and every 100 steps.
"""
import numpy as np
import pytest

from oracle import oracle as O
from trimem_gb300 import workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def L7(built):
    from trimem_gb300 import capi

    p, f, prm = workloads.very_large_mesh()
    return capi, p, f, prm


def _compare_state(eg, mg, eo, mo, what):
    e, g = eg.gradient(mg, with_energy=True)
    e_or, g_or = eo.energy(mo), eo.gradient(mo)
    assert abs(e - e_or) <= RTOL * abs(e_or), (what, e, e_or)
    r = rel(g, g_or)
    assert r < RTOL, (what, r)
    pg, po = eg.properties(mg), eo.properties(mo)
    for k in range(6):
        assert abs(pg[k] - po[k]) <= RTOL * max(abs(po[k]), 1e-300), (what, k, pg[k], po[k])
    return r


@pytest.mark.parametrize("stencil", [0, 2], ids=["fp64", "df64"])
def test_l7_benchmark_membrane_matches_the_oracle(L7, stencil):
    C, p, f, prm = L7
    mo = O.Mesh(p, f)
    eo = O.Energy(mo, O.default_params(**prm))
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    eg.set_stencil_precision(stencil)
    np.testing.assert_allclose(eg.initial_props(), eo.initial_props(), rtol=RTOL, atol=0)
    _compare_state(eg, mg, eo, mo, "constructed")
    vg, vo = eg.vertex_properties(mg), eo.vertex_properties(mo)
    for k in range(6):
        assert rel(vg[:, k], vo[:, k]) < RTOL, k
    # move every vertex a little and 2,000 of them by up to 0.6 of the
    # repulsion cut-off (cell changes, new pairs), then rebuild the lists
    rng = np.random.default_rng(17)
    lc1 = prm["rep_lc1"]
    d = rng.normal(0, 1e-3 * lc1, size=p.shape)
    pick = rng.choice(len(p), 2000, replace=False)
    d[pick] += rng.uniform(-0.6, 0.6, size=(2000, 3)) * lc1 / np.sqrt(3)
    x = p + d
    mo.points()[:] = x
    mg.points()[:] = x
    # stale bins first (the lists still hold the constructed state)
    _compare_state(eg, mg, eo, mo, "moved, stale lists")
    eo.update_repulsion(mo)
    eg.update_repulsion(mg)
    _compare_state(eg, mg, eo, mo, "moved, rebuilt lists")


def test_l7_flip_sweep_matches_the_oracle(L7):
    C, p, f, prm = L7
    mg = C.Mesh(p, f)
    eg = C.Energy(mg, C.params(**prm))
    mo = O.Mesh(p, f)
    eo = O.Energy(mo, O.default_params(**prm))
    for seed in (1, 2):
        ag = C.flip(mg, eg, 0.2, seed, 1, 4096)
        ao = O.flip_windowed(mo, eo, 0.2, seed, 1, 4096)
        assert ag == ao, (seed, ag, ao)
        assert ag > 0
        assert mg.check() == 0 and mo.check() == 0
        assert np.array_equal(mg.fv_indices(), mo.fv_indices()), seed
        fv = mg.fv_indices()
        assert len(np.unique(np.sort(fv, axis=1), axis=0)) == len(fv)  # no duplicate faces
        e = np.sort(np.concatenate([fv[:, [0, 1]], fv[:, [1, 2]], fv[:, [2, 0]]]), axis=1)
        ue, cnt = np.unique(e, axis=0, return_counts=True)
        assert (cnt == 2).all()  # every edge in exactly two faces: no double edges, closed
        assert np.bincount(ue.ravel(), minlength=len(p)).min() >= 3  # valence >= 3
        assert len(p) - len(ue) + len(fv) == 2  # Euler characteristic of a sphere
    # the energy after the sweeps is the oracle's on the same topology
    _compare_state(eg, mg, eo, mo, "after two sweeps")


def test_small_membrane_hybrid_run_matches_the_oracle(built):
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.device import DeviceChain

    p, f, prm = workloads.small_mesh()
    mg = capi.Mesh(p, f)
    eg = capi.Energy(mg, capi.params(**prm))
    initial = eg.initial_props()
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    ch = DeviceChain(mg, eg, x, dt=1e-4, n_leapfrog=20, flip_ratio=0.1, flip_mode=1, refresh=1, seed=2024)
    checks = []
    for step in range(0, 1001):
        if step % 100 == 0:
            xs = x.cpu().numpy()
            mg.points()[:] = xs
            mo = O.Mesh(xs, mg.fv_indices())
            eo = O.Energy(mo, O.default_params(**prm))
            eo.set_initial_props(initial)
            eg.update_repulsion(mg)
            checks.append(_compare_state(eg, mg, eo, mo, f"step {step}"))
            assert mg.check() == 0
        if step < 1000:
            ch.step()
    assert len(checks) == 11
    assert ch.flips > 0
    # at dt 1e-4 the jittered membrane's forces reject every HMC move (the
    # reference's integrator behaves the same); the run continues with the
    # largest time step that accepts, checked the same way
    from trimem_gb300.mc.device import tune_dt

    dt, _ = tune_dt(mg, eg, x, candidates=(1e-5, 5e-6, 2e-6, 1e-6, 5e-7, 2e-7))
    ch2 = DeviceChain(mg, eg, x, dt=dt, n_leapfrog=20, flip_ratio=0.1, flip_mode=1, refresh=1, seed=7)
    for step in range(1, 301):
        ch2.step()
        if step % 100 == 0:
            xs = x.cpu().numpy()
            mg.points()[:] = xs
            mo = O.Mesh(xs, mg.fv_indices())
            eo = O.Energy(mo, O.default_params(**prm))
            eo.set_initial_props(initial)
            eg.update_repulsion(mg)
            checks.append(_compare_state(eg, mg, eo, mo, f"dt {dt:g} step {step}"))
            assert mg.check() == 0
    assert ch2.accepted > 0
    print(f"small membrane run: {ch.accepted} of 1000 HMC moves accepted at dt 1e-4, {ch.flips} flips; "
          f"{ch2.accepted} of 300 at dt {dt:g}, {ch2.flips} flips; largest gradient deviation {max(checks):.1e}")
