"""Fields at points off the boundary on the host: the oracle's point fields
(Greenfun/@compgreenret/field.m over a compoint) approach the far field of
spectrumret/farfield.m as the distance grows (E r exp(-ikr) -> e_far with an
O(1/(kr)) remainder), and the media of points follow compoint's rule."""
import numpy as np

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


def test_point_fields_approach_far_field():
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    v, f = shapes.trisphere(144, 20.0)
    cp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(v, f, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    enei = 520.0
    _, _, sols, _ = R.solve_spectrum(cp, pw, [enei])
    s = sols[0]
    dirs = np.array([[0, 0, 1.0], [1.0, 0, 0], [0.6, 0, 0.8]])
    ef, hf, k = pw.farfield(cp, s, dirs)
    errs = []
    for r in (1e4, 1e5):
        e, h = R.point_fields(cp, dirs * r, [1, 1, 1], enei, s["sig1"], s["sig2"], s["h1"], s["h2"])
        sc = r * np.exp(-1j * k * r)
        errs.append((np.max(np.abs(e * sc - ef)) / np.max(np.abs(ef)), np.max(np.abs(h * sc - hf)) / np.max(np.abs(hf))))
    assert errs[1][0] < 5e-3 and errs[1][1] < 5e-3, errs
    assert errs[1][0] < 0.2 * errs[0][0], errs        # the remainder falls like 1 / r


def test_point_media():
    p = m.trisphere(144, 20.0)
    cp = m.comparticle([m.epsconst(1.0), m.epsconst(2.0)], [p], [[2, 1]], 1)
    pts = np.array([[0, 0, 0], [0, 0, 5.0], [0, 0, 15.0], [30.0, 0, 0]])
    assert list(m.point_media(cp, pts)) == [2, 2, 1, 1]
