"""The committed equilibrated chain state (trimem_gb300/data/chain_state_L7.npz,
written by python -m trimem_gb300.mc.equilibrate): it belongs to the
163,842-vertex benchmark membrane's energy, holds a closed triangulation of
that mesh, and is refused for any other energy."""
import numpy as np

from trimem_gb300 import workloads
from trimem_gb300.mc.equilibrate import STATE_L7, load_state, workload_key


def test_committed_state_matches_the_benchmark_workload():
    p, f, prm = workloads.very_large_mesh()
    st = load_state(prm, len(p))
    assert st is not None, STATE_L7
    x, fv = st["x"], st["faces"]
    assert x.shape == p.shape and x.dtype == np.float64 and np.isfinite(x).all()
    assert fv.shape == f.shape and fv.min() == 0 and fv.max() == len(p) - 1
    # a closed triangulation of the sphere: every edge in two faces, Euler 2
    e = np.sort(np.concatenate([fv[:, [0, 1]], fv[:, [1, 2]], fv[:, [2, 0]]]), axis=1)
    ue, cnt = np.unique(e, axis=0, return_counts=True)
    assert (cnt == 2).all()
    assert len(p) - len(ue) + len(fv) == 2
    assert np.bincount(ue.ravel(), minlength=len(p)).min() >= 3
    # reference properties of the input sphere (area, volume, curvature, ...)
    assert st["initial"].shape == (6,) and st["initial"][0] > 0 and st["initial"][1] > 0
    info = st["info"]
    assert info["steps"] >= 30000 and info["warm_dt"] > 0
    assert len(info["bending_block_means"]) == info["steps"] // info["block_steps"]


def test_state_is_refused_for_another_energy():
    p, f, prm = workloads.very_large_mesh()
    other = dict(prm, volume_frac=0.75)
    assert not np.array_equal(workload_key(prm, len(p)), workload_key(other, len(p)))
    assert load_state(other, len(p)) is None
    assert load_state(prm, len(p) - 1) is None
