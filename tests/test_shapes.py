"""Particle meshers: the hemispherically capped rod (trirod.m) and the cube with
rounded edges (tricube.m) at the face counts of the workloads, checked for a
closed surface (every edge shared by two faces), outward normals and the
analytic area / volume of the capsule."""
from collections import Counter

import numpy as np
import pytest

from mnpbem_gb300 import shapes


def edge_counts(faces):
    c = Counter()
    for f in faces:
        idx = [int(i) for i in f if i >= 0]
        for a, b in zip(idx, idx[1:] + idx[:1]):
            c[tuple(sorted((a, b)))] += 1
    return set(c.values())


def face_frame(verts, faces):
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    p = R.Particle(verts, faces, q)
    return p.pos, p.nvec, p.area


@pytest.mark.parametrize("n,nfaces", [((41, 11, 31), 2000), ((51, 11, 31), 2500)])
def test_rod_counts_and_closure(n, nfaces):
    v, f = shapes.trirod(10.0, 40.0, n)
    assert f.shape == (nfaces, 4)
    assert edge_counts(f) == {2}
    pos, nvec, area = face_frame(v, f)
    assert np.all(np.sum(nvec * pos, 1) > 0)
    vol = np.sum(area * np.sum(pos * nvec, 1)) / 3
    assert abs(area.sum() - (np.pi * 10 * 30 + np.pi * 100)) / (np.pi * 400) < 0.01
    assert abs(vol - (np.pi * 25 * 30 + 4 / 3 * np.pi * 125)) / 2880 < 0.01


def test_rounded_cube():
    e = shapes.rounding_to_e(40.0, 4.0)
    v, f = shapes.tricube(23, 40.0, e)
    assert f.shape == (2904, 4)
    assert edge_counts(f) == {2}
    pos, nvec, area = face_frame(v, f)
    assert np.all(np.sum(nvec * pos, 1) > 0)
    assert np.allclose(np.abs(v).max(0), 20.0)
    # a rounded cube has less area than the sharp one, more than the inscribed sphere
    assert 4 * np.pi * 400 < area.sum() < 9600


def test_triangle_split():
    v, f = shapes.trirod(10.0, 40.0, (21, 6, 11), triangles=True)
    assert np.all(f[:, 3] == -1)
    assert edge_counts(f) == {2}
