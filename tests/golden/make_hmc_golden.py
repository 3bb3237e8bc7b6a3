"""Recreates tests/golden/hmc_icosahedron.json from the reference's test file.

The reference pins plain HMC (tests/test_sampling.py:14-27 and :38-61) on the
vertices of trimesh's icosahedron with the quadratic energy x.x/2,
np.random.seed(42), time_step 0.1 and the default 100 integration steps.
trimesh is not installed, so the start positions are recovered here from the
golden output: velocity Verlet on x.x/2 maps every coordinate linearly,
x_L = a x_0 + b p, so for each of the 2^10 accept/reject patterns the start
x_0 follows from ref_hmc by one division.  The pattern whose x_0 rows are the
twelve unit vectors of an icosahedron and whose forward run (with this
package's HMC, which recomputes every accept decision) reproduces ref_hmc to
1e-14 is kept.  Run with the environment variable TRIMEM_REFERENCE set to
the root of a trimem checkout (the folder holding tests/test_sampling.py).
"""
import ast
import itertools
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from trimem_gb300.meshgen import hull_faces  # noqa: E402

REF = os.environ.get("TRIMEM_REFERENCE")


def read_ref_hmc():
    if not REF:
        raise SystemExit("set TRIMEM_REFERENCE to the root of a trimem checkout")
    src = open(os.path.join(REF, "tests", "test_sampling.py")).read()
    m = re.search(r"ref_hmc\s*=\s*np\.array\(\s*(\[.*?\])\s*\)", src, flags=re.S)
    return np.array(ast.literal_eval(m.group(1)))


def vv_map(dt, L):
    """2x2 matrix of L velocity-Verlet steps for force -x, unit mass."""
    M = np.eye(2)
    step = np.array([[1 - dt * dt / 2, dt], [-dt + dt**3 / 4, 1 - dt * dt / 2]])
    for _ in range(L):
        M = step @ M
    return M


def run(x0, steps=10):
    np.random.seed(42)
    x, _ = O.hmc_chain(x0.copy(), lambda x: 0.5 * x.ravel().dot(x.ravel()), lambda x: x,
                       n_steps=steps, dt=0.1, n_leapfrog=100)
    return x


def main():
    ref = read_ref_hmc()
    dt, L, nsteps = 0.1, 100, 10
    M = vv_map(dt, L)
    a, b = M[0, 0], M[0, 1]
    np.random.seed(42)
    ps = []
    for _ in range(nsteps):
        ps.append(np.random.normal(size=ref.shape))
        np.random.uniform()
    best = None
    for pat in itertools.product([0, 1], repeat=nsteps):
        off = np.zeros_like(ref)
        scale = 1.0
        for k in range(nsteps):
            if pat[k]:
                off = a * off + b * ps[k]
                scale *= a
        x0 = (ref - off) / scale
        r = np.linalg.norm(x0, axis=1)
        err = np.abs(r - 1).max()
        if best is None or err < best[0]:
            best = (err, pat, x0)
    err, pat, x0 = best
    assert err < 1e-10, err
    out = run(x0)
    dev = float(np.linalg.norm(out - ref))
    assert dev < 1e-14, dev
    faces = hull_faces(x0)
    assert len(faces) == 20
    json.dump({"x0": x0.tolist(), "faces": faces.tolist(), "ref_hmc": ref.tolist(), "accept_pattern": pat,
               "forward_error": dev}, open(os.path.join(HERE, "hmc_icosahedron.json"), "w"), indent=1)
    print("accept pattern", pat, "max | |x0|-1 |", err, "forward error", dev)


if __name__ == "__main__":
    main()
