"""State wrapper around :class:`trimem_gb300.core.TriMesh`
(src/trimem/mc/mesh.py in the reference)."""
import copy

import numpy as np


def _core():
    from .. import load_core
    return load_core()


class Mesh:
    """Vertices ``x`` (a view of the mesh's positions; assignment copies in
    place) and faces ``f``."""

    def __init__(self, points=None, cells=None):
        m = _core()
        if points is not None and cells is not None:
            self.trimesh = m.TriMesh(points, cells)
        else:
            self.trimesh = m.TriMesh()

    @property
    def x(self):
        return self.trimesh.points()

    @x.setter
    def x(self, values):
        np.copyto(self.x, values)

    @property
    def f(self):
        return self.trimesh.fv_indices()

    def copy(self):
        return copy.deepcopy(self)


def read_trimesh(filename):
    """Mesh read from ``filename`` (OFF, OBJ or STL)."""
    mesh = Mesh.__new__(Mesh)
    mesh.trimesh = _core().read_mesh(filename)
    return mesh
