"""Particle transforms of the mirror (Particles/@particle rot.m, scale.m,
flip.m, flipfaces.m) on flat and curved elements: rotations move centroids
and normals and keep areas, scaling scales areas, flipfaces reverses the
normals, flip mirrors the particle with the normals kept outward.  For
curved quadrilaterals the split into two 6-node triangles follows the corner
order (norm_curv.m takes the basis from the first, quad_curv.m sums both), so
flipfaces moves the split to the other diagonal: their flipped normals are
antiparallel to 2e-3 and their areas agree to 1e-3, not exactly.  That is
the reference's behaviour too."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes


def particles():
    v, f = shapes.trirod(10.0, 40.0, (15, 5, 11))
    p = m.particle(v, f)
    return {"flat": p, "curved": p.midpoints("curv")}


@pytest.mark.parametrize("kind", ["flat", "curved"])
def test_rotation(kind):
    p = particles()[kind]
    q = p.rot(90, [0, 1, 0])
    # rot.m's expm(-angle J) on row vectors: 90 degrees about y maps (x, y, z) -> (z, y, -x)
    r = np.array([[0, 0, -1], [0, 1, 0], [1, 0, 0]], float)
    assert np.allclose(q.pos, p.pos @ r, atol=1e-12)
    assert np.allclose(q.nvec, p.nvec @ r, atol=1e-12)
    assert np.allclose(q.area, p.area, rtol=1e-12)
    assert np.allclose(p.rot(30).rot(-30).pos, p.pos, atol=1e-12)


@pytest.mark.parametrize("kind", ["flat", "curved"])
def test_scale_flip(kind):
    p = particles()[kind]
    assert np.allclose(p.scale(2.0).area, 4 * p.area, rtol=1e-12)
    assert np.allclose(p.scale([1, 1, 2]).pos[:, 2], 2 * p.pos[:, 2], atol=1e-12)
    ff = p.flipfaces()
    tol, atol = (1e-12, 1e-12) if kind == "flat" else (2e-3, 1e-3)
    assert np.min(np.sum(ff.nvec * -p.nvec, 1)) > 1 - tol
    assert np.allclose(ff.area, p.area, rtol=atol)
    fl = p.flip(1)
    mirror = np.array([-1.0, 1.0, 1.0])
    if kind == "flat":
        assert np.allclose(fl.pos, p.pos * mirror, atol=1e-12)
    assert np.min(np.sum(fl.nvec * (p.nvec * mirror), 1)) > 1 - tol    # still outward
    assert np.allclose(fl.area, p.area, rtol=atol)
    assert np.allclose(fl.flip(1).pos, p.pos, atol=1e-12)


def test_shape_particles():
    rod = m.trirod(10.0, 40.0, (15, 5, 11))
    v, f = shapes.trirod(10.0, 40.0, (15, 5, 11))
    assert np.array_equal(rod.faces, f) and np.allclose(rod.verts, v)
    assert abs(rod.midpoints("curv").area.sum() - (np.pi * 10 * 30 + 4 * np.pi * 25)) < 2.0
    cube = m.tricube(8, 40.0, 0.25, op={"interp": "flat"})
    assert cube.n == shapes.tricube(8, 40.0, 0.25)[1].shape[0]
    assert np.all(np.sum(cube.nvec * cube.pos, 1) > 0)          # outward normals


def test_sphere_segments():
    """trispheresegment.m: a full sphere from the (phi, theta^2) grid of the
    dipole demos has outward normals, merged seam and poles (30 x 30 cells,
    the pole cells triangles) and, with curved elements, the sphere's area
    to 1e-4; a quarter segment and the triangle variant are outward too."""
    full = m.trispheresegment(2 * np.pi * np.linspace(0, 1, 31), np.pi * np.linspace(0, 1, 31) ** 2, 4.0)
    assert full.n == 900 and np.sum(full.faces[:, 3] < 0) == 60
    assert np.all(np.sum(full.nvec * full.pos, 1) > 0)
    assert np.allclose(np.linalg.norm(full.verts2, axis=1), 2.0, atol=1e-12)
    curved = m.trispheresegment(2 * np.pi * np.linspace(0, 1, 31), np.pi * np.linspace(0, 1, 31) ** 2, 4.0,
                                op={"interp": "curv"})
    assert abs(curved.area.sum() - 16 * np.pi) < 1e-4 * 16 * np.pi
    quarter = m.trispheresegment(np.linspace(0, np.pi / 2, 10), np.pi * np.linspace(0, 1, 15) ** 2, 10.0)
    assert np.all(np.sum(quarter.nvec * quarter.pos, 1) > 0)
    tri = m.trispheresegment(2 * np.pi * np.linspace(0, 1, 13), np.pi * np.linspace(0, 1, 9), 4.0, triangles=True)
    assert np.all(tri.faces[:, 3] < 0) and np.all(np.sum(tri.nvec * tri.pos, 1) > 0)
