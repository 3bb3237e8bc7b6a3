"""Trajectory writers (no GPU): the reference's xyz text format and part
enumeration (src/trimem/mc/output/xyz.py, _common.py), and VTK
UnstructuredGrid files named like the reference's vtu writer."""
import numpy as np

from trimem_gb300 import meshgen
from trimem_gb300.mc.output import VtuWriter, XyzWriter, read_vtu


def test_xyz_frames_and_parts(tmp_path):
    p, f = meshgen.icosphere(1)
    w = XyzWriter(tmp_path / "traj")
    w.write_points_cells(p, f)
    w.write_points_cells(p + 1.0, f)
    assert w.fname.name == "traj.p0.xyz"
    lines = w.fname.read_text().splitlines()
    n = len(p)
    assert lines[0] == str(n) and lines[1] == "#" and lines[n + 2] == str(n)
    first = lines[2].split("\t")
    assert first[0] == "C" and np.allclose([float(v) for v in first[1:]], p[0], atol=1e-6)
    assert len(lines) == 2 * (n + 2)
    # a second writer with the same prefix opens the next part
    assert XyzWriter(tmp_path / "traj").fname.name == "traj.p1.xyz"


def test_vtu_round_trip(tmp_path):
    import torch

    p, f = meshgen.jittered_icosphere(2, seed=4)
    w = VtuWriter(tmp_path / "mesh")
    f0 = w.write_points_cells(p, f)
    f1 = w.write_points_cells(torch.tensor(p) * 2.0, f)  # tensors are accepted
    assert (f0.name, f1.name) == ("mesh.0.p0.vtu", "mesh.1.p0.vtu")
    q, c = read_vtu(f0)
    assert np.array_equal(q, p) and np.array_equal(c, f)  # repr() keeps every bit
    q1, _ = read_vtu(f1)
    assert np.array_equal(q1, 2.0 * p)
    assert VtuWriter(tmp_path / "mesh").part == ".p1"
