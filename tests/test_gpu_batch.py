"""Batches of replicas: the size-class launches must give each replica the
result of its own single-mesh evaluation (FP32 stencils, FP64 sums, the
replica's own exclusion level), and the batched HMC must be deterministic
with and without graphs."""
import numpy as np
import pytest

from helpers import workload_params
from oracle import oracle as O
from trimem_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _replicas():
    """Four replicas of three sizes (three size classes), each with its own
    bending rigidity, volume target and exclusion level."""
    out = []
    for level, seed, kb, vf, excl in [(2, 1, 10.0, 0.9, 1), (3, 2, 30.0, 0.7, 2), (3, 3, 50.0, 0.95, 0),
                                      (4, 4, 20.0, 0.6, 1)]:
        p, f = meshgen.jittered_icosphere(level, seed=seed)
        prm = workload_params(p, f, kappa_b=kb, vfrac=vf, excl=excl, rep_scale=1.2)
        out.append((p, f, prm))
    return out


@pytest.fixture(scope="module")
def C(built):
    from trimem_gb300 import capi
    return capi


def test_batch_matches_single_meshes(C):
    reps = _replicas()
    b = C.Batch([(p, f) for p, f, _ in reps], [C.params(**prm) for _, _, prm in reps])
    assert b.n_total % 256 == 0 and list(b.offsets[:-1] % 256) == [0] * len(reps)
    # size classes: 162 / 642 / 2,562 vertices, each with its tuned block sizes
    cls = b.tuning()
    assert [c[:2] for c in cls] == [(b.offsets[0], b.offsets[1]), (b.offsets[1], b.offsets[3]),
                                     (b.offsets[3], b.offsets[4])]
    assert all(bs in (64, 128, 256, 512) for c in cls for bs in c[2:])
    eb, gb = b.energy(with_grad=True)
    for r, (p, f, prm) in enumerate(reps):
        m = C.Mesh(p, f)
        e = C.Energy(m, C.params(**prm))
        e.set_stencil_precision(1)
        es, gs = e.gradient(m, with_energy=True)
        assert abs(eb[r] - es) <= 1e-12 * abs(es), (r, eb[r], es)
        assert np.linalg.norm(gb[r] - gs) <= 1e-12 * np.linalg.norm(gs), r
        # and the FP32-stencil error against the FP64 oracle stays small
        eo = O.Energy(O.Mesh(p, f), O.default_params(**prm)).energy(O.Mesh(p, f))
        assert abs(eb[r] - eo) <= 1e-5 * abs(eo), r


def test_batch_with_verlet_lists_matches_single_meshes(C):
    """The same replicas with Verlet lists (src/nlists/verlet_list.h): each
    replica's energy and gradient equal its single-mesh evaluation with a
    Verlet list, and a batch cannot mix the two kinds of list."""
    reps = [(p, f, dict(prm, n_search=1)) for p, f, prm in _replicas()]
    b = C.Batch([(p, f) for p, f, _ in reps], [C.params(**prm) for _, _, prm in reps])
    eb, gb = b.energy(with_grad=True)
    for r, (p, f, prm) in enumerate(reps):
        m = C.Mesh(p, f)
        e = C.Energy(m, C.params(**prm))
        e.set_stencil_precision(1)
        es, gs = e.gradient(m, with_energy=True)
        assert abs(eb[r] - es) <= 1e-12 * abs(es), (r, eb[r], es)
        assert np.linalg.norm(gb[r] - gs) <= 1e-12 * np.linalg.norm(gs), r
    eo = O.Energy(O.Mesh(reps[3][0], reps[3][1]), O.default_params(**reps[3][2]))
    assert abs(eb[3] - eo.energy(O.Mesh(reps[3][0], reps[3][1]))) <= 1e-5 * abs(eb[3])
    mixed = [C.params(**prm) for _, _, prm in _replicas()]
    mixed[1] = C.params(**reps[1][2])
    with pytest.raises(RuntimeError):
        C.Batch([(p, f) for p, f, _ in reps], mixed)
    # HMC steps on the Verlet batch: finite, deterministic
    acc = b.hmc(4, 5, 1e-6, seed=3)
    b2 = C.Batch([(p, f) for p, f, _ in reps], [C.params(**prm) for _, _, prm in reps])
    acc2 = b2.hmc(4, 5, 1e-6, seed=3)
    assert np.array_equal(acc, acc2)
    for x, x2 in zip(b.positions(), b2.positions()):
        assert np.array_equal(x, x2) and np.isfinite(x).all()


def test_batch_hmc_graph_replay_is_deterministic(C):
    reps = _replicas()
    runs = []
    for use_graph in (False, True):
        b = C.Batch([(p, f) for p, f, _ in reps], [C.params(**prm) for _, _, prm in reps])
        acc = b.hmc(6, 5, 1e-6, seed=11, use_graph=use_graph)
        runs.append((acc, b.positions()))
    assert np.array_equal(runs[0][0], runs[1][0])
    for x0, x1 in zip(runs[0][1], runs[1][1]):
        assert np.array_equal(x0, x1)
    assert runs[0][0].sum() > 0  # small steps are accepted
    # the positions moved and stay finite
    x_init = [p for p, _, _ in reps]
    assert any(np.abs(x - xi).max() > 0 for x, xi in zip(runs[1][1], x_init))
    assert all(np.isfinite(x).all() for x in runs[1][1])


def test_batch_hmc_refresh_changes_no_result(C):
    """Rebuilding the neighbour list between steps only changes which path
    finds the pairs (near rows, candidate rows or the cell walk), all in the
    reference's pair order: positions and decisions are identical."""
    reps = _replicas()
    runs = []
    for refresh in (0, 1, 2):
        b = C.Batch([(p, f) for p, f, _ in reps], [C.params(**prm) for _, _, prm in reps])
        acc = b.hmc(6, 5, 2e-6, seed=5, refresh=refresh)
        runs.append((acc, b.positions()))
    for acc, xs in runs[1:]:
        assert np.array_equal(acc, runs[0][0])
        for x0, x1 in zip(runs[0][1], xs):
            assert np.array_equal(x0, x1)
