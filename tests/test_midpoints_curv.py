"""Curved-element nodes from the approximate curvature (midpoints.m key
'curv': refine.m, vertex_neighbours.m, edge_tangents.m,
make_halfway_vertices.m) on the host: the package's vectorised version
against the oracle's loop restatement, and known answers.

Known answers (no reference outputs exist for this path): on a regular planar
triangle grid the tangents run along the edges and the Bezier midpoints of
interior edges are the edge midpoints (1e-13); on a sphere the new nodes lie
closer to the sphere than the flat midpoints and the curved area is closer to
4 pi R^2; every edge node is shared by the two faces of a closed surface.
"""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


def cases():
    return {"sphere": shapes.trisphere(256, 20.0),
            "rod": shapes.trirod(10.0, 40.0, (15, 5, 11)),
            "cube": shapes.tricube(8, 40.0, 0.25),
            "fibsphere": shapes.fibsphere(600, 30.0)}


@pytest.mark.parametrize("name", ["sphere", "rod", "cube", "fibsphere"])
def test_package_matches_oracle(name):
    v, f = cases()[name]
    v2, f2 = shapes.midpoints_curv(v, f)
    w2, g2 = R.midpoints_curv(v, f)
    assert np.array_equal(f2, g2)
    assert v2.shape == w2.shape
    assert np.max(np.abs(v2 - w2)) <= 1e-13 * np.max(np.abs(w2))
    assert np.array_equal(v2[:v.shape[0]], np.asarray(v, float))


def test_neighbour_fans_match_oracle():
    v, f = shapes.trirod(10.0, 40.0, (15, 5, 11))
    tri, _ = shapes._split_triangles(f)
    assert shapes._neighbour_fans(tri, v.shape[0]) == R.vertex_neighbours(tri, v.shape[0])
    # an open patch: boundary vertices open their fans at the boundary
    g = planar_grid(5)
    tri = g[1][:, :3]
    fo, fp = R.vertex_neighbours(tri, g[0].shape[0]), shapes._neighbour_fans(tri, g[0].shape[0])
    assert fo == fp
    for fan in fp:
        assert len(fan) == len(set(fan))


def planar_grid(k):
    pts = np.array([[i + 0.5 * j, np.sqrt(3) / 2 * j, 0.0] for j in range(k) for i in range(k)])
    faces = []
    for j in range(k - 1):
        for i in range(k - 1):
            a, b, c, d = j * k + i, j * k + i + 1, (j + 1) * k + i, (j + 1) * k + i + 1
            faces += [[a, b, c, -1], [b, d, c, -1]]
    return pts, np.array(faces, np.int64)


def test_planar_grid_interior_edges_are_straight():
    k = 7
    v, f = planar_grid(k)
    v2, f2 = shapes.midpoints_curv(v, f)
    assert np.all(v2[:, 2] == 0.0)
    interior = np.zeros(v.shape[0], bool)
    for j in range(1, k - 1):
        interior[j * k + 1:j * k + k - 1] = True
    checked = 0
    for row in f2:
        for e, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
            if interior[row[a]] and interior[row[b]]:
                mid = 0.5 * (v[row[a]] + v[row[b]])
                assert np.max(np.abs(v2[row[4 + e]] - mid)) < 1e-13
                checked += 1
    assert checked > 20


def test_sphere_nodes_closer_than_flat():
    v, f = shapes.trisphere(256, 20.0)
    v2, _ = shapes.midpoints_curv(v, f)
    w2, _ = shapes.midpoints_flat(v, f)
    dc = np.abs(np.linalg.norm(v2[v.shape[0]:], axis=1) - 10.0).max()
    df = np.abs(np.linalg.norm(w2[v.shape[0]:], axis=1) - 10.0).max()
    assert dc < df / 3, (dc, df)
    p = m.particle(v, f)
    exact = 4 * np.pi * 100.0
    a_curv = p.midpoints("curv").area.sum()
    assert abs(a_curv - exact) < abs(p.area.sum() - exact) / 3


@pytest.mark.parametrize("name", ["sphere", "rod"])
def test_closed_surface_nodes_shared(name):
    v, f = cases()[name]
    _, f2 = shapes.midpoints_curv(v, f)
    quad = f2[:, 3] >= 0
    edge_nodes = np.concatenate([f2[~quad, 4:7].ravel(), f2[quad, 4:8].ravel()])
    _, counts = np.unique(edge_nodes, return_counts=True)
    assert np.all(counts == 2)
    # quadrilateral centre nodes are the diagonal's own nodes
    if quad.any():
        _, cc = np.unique(f2[quad, 8], return_counts=True)
        assert np.all(cc == 1) and not np.isin(f2[quad, 8], edge_nodes).any()


def test_particle_mirror():
    v, f = shapes.trirod(10.0, 40.0, (15, 5, 11))
    p = m.particle(v, f)
    q = p.midpoints("curv")
    assert q.interp == "curv" and q.faces2.shape == (p.n, 9)
    assert p.midpoints("flat").interp == "flat"
    assert m.curved(p).interp == "curv"
    # curved.m keeps the nodes a particle carries unless a key is given
    assert np.array_equal(m.curved(q).verts2, q.verts2)
    c = m.curved(p, "curv")
    assert np.array_equal(c.verts2, q.verts2) and np.array_equal(c.faces2, q.faces2)
    exact = np.pi * 10 * 30 + 4 * np.pi * 25
    assert abs(q.area.sum() - exact) < abs(p.area.sum() - exact) / 5
    with pytest.raises(ValueError):
        p.midpoints("smooth")


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_perturbed_and_open_meshes_match_oracle(seed):
    """Seeded random vertex perturbations (irregular fans, odd valences) and
    an open cap of a sphere (boundary vertices open their fans)."""
    rng = np.random.default_rng(seed)
    v, f = shapes.trisphere(144, 20.0)
    v = v + rng.normal(scale=0.3, size=v.shape)
    for verts, faces in ((v, f), (v, f[np.all(v[f[:, :3], 2] > -2.0, axis=1)])):
        v2, f2 = shapes.midpoints_curv(verts, faces)
        w2, g2 = R.midpoints_curv(verts, faces)
        assert np.array_equal(f2, g2)
        assert np.max(np.abs(v2 - w2)) <= 1e-13 * np.max(np.abs(w2))
