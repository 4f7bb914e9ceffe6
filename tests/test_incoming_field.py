"""Incoming plane-wave fields (@planewaveret/field.m) on the host: the
package's closed form against the oracle's restatement at the faces of a
dimer (one medium per sphere: only the faces bordering the embedding medium
get the wave), and the plane-wave relations |e| = |pol|, e . dir = 0,
h = nb dir x e; a meshfield passes given fields through, reshaped."""
import numpy as np

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


def test_plane_wave_field_matches_oracle():
    v, f = shapes.trisphere(60, 10.0)
    p1, p2 = m.particle(v, f), m.particle(v + [0, 0, 12.0], f)
    drude = m.epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV")
    cp = m.comparticle([m.epsconst(1.77), drude, drude], [p1, p2], [[2, 1], [3, 1]], 1, 2)
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [1 / np.sqrt(2), 0, 1 / np.sqrt(2)]])
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    ocp = R.ComParticle([R.EpsConst(1.77), R.drude_eps(), R.drude_eps()],
                        [R.Particle(p1.verts, p1.faces, q), R.Particle(p2.verts, p2.faces, q)],
                        np.array([[2, 1], [3, 1]]), [True, True])
    pw = R.PlaneWaveRet(exc.pol, exc.dir, R.Particle(*shapes.trisphere(256, 2.0), q))
    for inout in (1, 2):
        got = exc.field(cp, 600.0, inout)
        we, wh = pw.field(ocp, 600.0, inout)
        assert np.max(np.abs(got.e - we)) < 1e-14 and np.max(np.abs(got.h - wh)) < 1e-14
    got = exc.field(cp, 600.0, 2)
    nb = np.sqrt(1.77)
    assert np.allclose(np.linalg.norm(got.e, axis=1), 1.0, atol=1e-14)
    for i in range(2):
        assert np.max(np.abs(got.e[:, :, i] @ exc.dir[i])) < 1e-14
        assert np.allclose(got.h[:, :, i], nb * np.cross(exc.dir[i], got.e[:, :, i]), atol=1e-14)
    assert not np.any(exc.field(cp, 600.0, 1).e)        # no face has medium 1 inside


def test_meshfield_passes_fields_through():
    mf = m.meshfield.__new__(m.meshfield)
    mf.shape = (4, 5)
    e = np.arange(20 * 3 * 2).reshape(20, 3, 2) + 0j
    ee, hh = mf(m.compstruct(None, 600.0, e=e, h=2 * e))
    assert ee.shape == (4, 5, 3, 2) and np.array_equal(ee.reshape(20, 3, 2), e)
    assert np.array_equal(hh.reshape(20, 3, 2), 2 * e)
