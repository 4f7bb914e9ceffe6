"""Particle surface meshes for the retarded BEM path.

``trisphere`` mirrors ``Particles/particleshapes/trisphere.m:18-61``: it loads
the stored minimum-energy point set closest in size to ``n`` (the table ships
as ``data/tables.npz``), triangulates it, and scales it to the requested
diameter.  The reference triangulates by a stereographic projection plus a
planar Delaunay triangulation (``misc/sphtriangulate.m``); for points on a
sphere that triangulation is the convex hull of the points, which is what is
computed here (same triangles, different face order).  Faces are oriented so
that ``(v1 - v2) x (v3 - v2)`` — the normal of ``norm_flat.m:36-38`` — points
outwards.

``fibsphere`` is this project's own deterministic mesher for sizes beyond the
stored sets (the largest has 1444 points): a Fibonacci spiral of points on the
sphere, triangulated the same way.  ``n_faces = 2 * n_points - 4``.

Faces are returned as ``int64 [n, 4]`` 0-based vertex indices with ``-1`` in
the 4th column for triangles (the reference uses NaN there).
"""
import os

import numpy as np

_TABLES = None


def tables():
    global _TABLES
    if _TABLES is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tables.npz")
        _TABLES = dict(np.load(path))
    return _TABLES


def _hull_faces(unit):
    from scipy.spatial import ConvexHull
    hull = ConvexHull(unit)
    faces = np.asarray(hull.simplices, dtype=np.int64)
    v1, v2, v3 = unit[faces[:, 0]], unit[faces[:, 1]], unit[faces[:, 2]]
    nvec = np.cross(v1 - v2, v3 - v2)
    cen = (v1 + v2 + v3) / 3
    flip = np.sum(nvec * cen, 1) < 0
    faces[flip] = faces[flip][:, ::-1]
    # deterministic order: sort faces by their smallest vertex index tuple
    rolled = np.array([np.roll(f, -int(np.argmin(f))) for f in faces])
    order = np.lexsort((rolled[:, 2], rolled[:, 1], rolled[:, 0]))
    faces = rolled[order]
    return np.hstack([faces, -np.ones((faces.shape[0], 1), np.int64)])


def trisphere(n, diameter=1.0):
    """Sphere from the stored point set closest to ``n`` points (trisphere.m)."""
    t = tables()
    sizes = t["sphere_sizes"]
    nsav = int(sizes[np.argmin(np.abs(sizes - n))])
    pts = t["sphere%d" % nsav].astype(np.float64)
    faces = _hull_faces(pts / np.linalg.norm(pts, axis=1)[:, None])
    v1 = 0.5 * pts * diameter
    verts = 0.5 * diameter * v1 / np.sqrt(np.sum(v1 * v1, 1))[:, None]
    return verts, faces


def fibsphere(n_faces, diameter=1.0, center=(0.0, 0.0, 0.0)):
    """Deterministic sphere with ``n_faces`` (even) flat triangles."""
    npts = n_faces // 2 + 2
    i = np.arange(npts, dtype=np.float64) + 0.5
    z = 1 - 2 * i / npts
    r = np.sqrt(np.maximum(0.0, 1 - z * z))
    golden = np.pi * (3 - np.sqrt(5.0))
    phi = golden * i
    unit = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    faces = _hull_faces(unit)
    verts = 0.5 * diameter * unit + np.asarray(center, dtype=np.float64)[None, :]
    return verts, faces


def sphere(n_faces, diameter=1.0, center=(0.0, 0.0, 0.0)):
    """``trisphere`` when a stored set gives exactly ``n_faces``, else ``fibsphere``."""
    npts = n_faces // 2 + 2
    sizes = tables()["sphere_sizes"]
    if npts in set(int(s) for s in sizes):
        v, f = trisphere(npts, diameter)
        return v + np.asarray(center, dtype=np.float64)[None, :], f
    return fibsphere(n_faces, diameter, center)
