"""Synthetic triangle meshes (numpy only).

``icosphere(level)`` subdivides the regular icosahedron ``level`` times,
projecting new vertices onto the unit sphere: 10*4**level + 2 vertices,
20*4**level faces, faces oriented outwards.  ``rect`` and ``tube`` build the
planar grid and the open cylinder the reference's test-suite uses
(tests/util.py:5-69 in the reference): same vertex numbering and the same
diagonal per grid cell, so per-vertex known answers (e.g. the neighbour counts
of vertex 151 of ``rect(20, 20)``) carry over.
"""
import numpy as np

_PHI = (1.0 + 5.0 ** 0.5) / 2.0


def icosahedron():
    """Unit icosahedron: (12, 3) float64 vertices, (20, 3) int32 faces."""
    v = []
    for a in (-1.0, 1.0):
        for b in (-_PHI, _PHI):
            v.append((0.0, a, b))
            v.append((a, b, 0.0))
            v.append((b, 0.0, a))
    v = np.asarray(v, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, hull_faces(v)


def hull_faces(v):
    """Outward-oriented faces of a convex polyhedron whose edges all have the
    minimal vertex distance (the icosahedron)."""
    n = len(v)
    d = np.linalg.norm(v[:, None, :] - v[None, :, :], axis=2)
    lmin = d[d > 0].min()
    adj = np.abs(d - lmin) < 1e-9 * lmin
    faces = []
    for i in range(n):
        for j in range(i + 1, n):
            if not adj[i, j]:
                continue
            for k in range(j + 1, n):
                if adj[i, k] and adj[j, k]:
                    a, b, c = i, j, k
                    nrm = np.cross(v[b] - v[a], v[c] - v[a])
                    if np.dot(nrm, v[a] + v[b] + v[c]) < 0:
                        b, c = c, b
                    faces.append((a, b, c))
    return np.asarray(faces, dtype=np.int32)


def icosphere(level, radius=1.0):
    """Subdivided icosahedron on a sphere of ``radius``."""
    v, f = icosahedron()
    verts = [tuple(x) for x in v]
    faces = f.tolist()
    for _ in range(int(level)):
        mid = {}

        def midpoint(a, b):
            key = (a, b) if a < b else (b, a)
            idx = mid.get(key)
            if idx is None:
                p = (np.asarray(verts[a]) + np.asarray(verts[b])) * 0.5
                p /= np.linalg.norm(p)
                idx = len(verts)
                verts.append(tuple(p))
                mid[key] = idx
            return idx

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.asarray(verts, dtype=np.float64) * radius, np.asarray(faces, dtype=np.int32)


def rect(nx, ny):
    """Planar unit-square grid, vertex index = iy*nx + ix, in the z=0 plane."""
    x = np.linspace(0.0, 1.0, nx)
    y = np.linspace(0.0, 1.0, ny)
    gx, gy = np.meshgrid(x, y)
    pts = np.stack([gx.ravel(), gy.ravel(), np.zeros(nx * ny)], axis=1)
    faces = []
    for r in range(ny - 1):
        base = r * nx
        for c in range(nx - 1):
            faces.append((base + c, base + c + 1, base + c + 1 + nx))
        for c in range(nx - 1):
            faces.append((base + c + nx, base + c, base + c + 1 + nx))
    return pts, np.asarray(faces, dtype=np.int32)


def tube(length=1.0, radius=1.0, segments=30):
    """Open cylinder around the y axis; rings of ``segments`` vertices."""
    mesh_size = 2.0 * np.pi * radius / segments
    nring = int(length // mesh_size) + 1
    ang = np.linspace(0.0, 2.0 * np.pi, segments + 1)[:-1]
    ys = np.linspace(-length / 2.0, length / 2.0, nring)
    pts = np.array([(np.cos(a) * radius, y, np.sin(a) * radius) for y in ys for a in ang])
    faces = []
    for r in range(nring - 1):
        o = r * segments
        for s in range(segments):
            faces.append((o + s, o + s + segments, o + (s + 1) % segments))
        for s in range(segments):
            faces.append((o + (s + 1) % segments, o + s + segments, o + (s + 1) % segments + segments))
    return pts, np.asarray(faces, dtype=np.int32)


def mean_edge_length(points, faces):
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    e = np.unique(np.sort(e, axis=1), axis=0)
    return float(np.linalg.norm(points[e[:, 0]] - points[e[:, 1]], axis=1).mean())


# mean edge length of the level-4 unit icosphere
L4_MEAN_EDGE = 0.07549909830150697


def jittered_icosphere(level, sigma_rel=0.01 / L4_MEAN_EDGE, seed=0):
    """Icosphere with Gaussian vertex jitter of ``sigma_rel`` times the mean
    edge length: sigma 0.01 at level 4 and the same relative jitter (13% of
    the mean edge) at every other level."""
    p, f = icosphere(level)
    l = mean_edge_length(p, f)
    rng = np.random.default_rng(seed)
    return p + rng.normal(0.0, sigma_rel * l, size=p.shape), f
