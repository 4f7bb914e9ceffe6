"""GPU fields at points off the boundary (mnpbem_fields / meshfield) against
the oracle's restatement of compgreenret field.m over a compoint, on the same
surface charges (from the GPU FP64 solve): points outside (near the surface,
inside the RelCutoff refinement zone, and far away) and inside a 284-face
sphere, flat and curved elements.  Tolerance 1e-10 (relative to the largest
field of the set)."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

from test_gpu_parity import drude, rel, record

pytestmark = pytest.mark.gpu


def points():
    rng = np.random.default_rng(5)
    u = rng.standard_normal((40, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    radii = np.concatenate([np.full(10, 10.4), np.full(10, 11.5), np.full(10, 40.0), np.full(10, 4.0)])
    return u * radii[:, None]


@pytest.mark.parametrize("interp", ["flat", "curv"])
def test_fields_match_oracle(gpu_lib, interp):
    from oracle import mnpbem_ref as R
    p = m.trisphere(144, 20.0, {"interp": interp})
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    sig = bem.mldivide(exc(cp, 540.0))
    pts = points()
    emesh = m.meshfield(bem, pts)
    assert list(emesh.medium) == [1] * 30 + [2] * 10
    e, h = emesh(sig)
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    op = R.Particle.curved(p.verts2, p.faces2, q) if interp == "curv" else R.Particle(p.verts, p.faces, q)
    ocp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [op], [[2, 1]], [True])
    eo, ho = R.point_fields(ocp, pts, emesh.medium, 540.0, sig.sig1, sig.sig2, sig.h1, sig.h2)
    errs = {"e": rel(e, eo), "h": rel(h, ho), "e_near": rel(e[:10], eo[:10]), "e_inside": rel(e[30:], eo[30:])}
    rows, _, _, _ = R.point_refinement(ocp, pts)
    errs["refined_pairs"] = int(rows.size)
    record("fields_" + interp, **errs)
    assert errs["refined_pairs"] > 0
    for k in ("e", "h", "e_near", "e_inside"):
        assert errs[k] < 1e-10, (k, errs)
