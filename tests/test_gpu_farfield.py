"""GPU far fields of the surface charges (mnpbem_farfield, spectrumret
farfield.m) against the oracle's restatement on the same charges: the
284-face sphere and the two-sphere dimer, two polarisations, on the 508
directions of the sphere at infinity and in the propagation directions
(1e-12 of the largest entry); the extinction from those far fields equals
the solver's own (optical theorem, 1e-12)."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

from test_gpu_parity import rel, record
from test_gpu_surface import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["sphere", "dimer"])
def test_farfield_matches_oracle(gpu_lib, name):
    from oracle import mnpbem_ref as R
    cp = dict(cases())[name]
    enei = 600.0
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    sig = bem.mldivide(exc(cp, enei))
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    parts = [R.Particle(pp.verts, pp.faces, q) for pp in cp.p]
    eps = [R.EpsConst(1.77)] + [R.drude_eps()] * (len(cp.eps) - 1)
    ocp = R.ComParticle(eps, parts, cp.inout, [bool(c) for c in cp.closed])
    pw = R.PlaneWaveRet(exc.pol, exc.dir, R.Particle(*shapes.trisphere(256, 2.0), q))
    osig = {"enei": enei, "sig1": sig.sig1, "sig2": sig.sig2, "h1": sig.h1, "h2": sig.h2}
    errs = {}
    for key, dirs in (("inf", exc.spec.nvec), ("dir", exc.dir)):
        ff = exc.spec.farfield(bem, sig, dirs)
        we, wh, k = pw.farfield(ocp, osig, np.asarray(dirs, float))
        errs["e_" + key], errs["h_" + key] = rel(ff.e, we), rel(ff.h, wh)
    ff = exc.spec.farfield(bem, sig, exc.dir)
    ext = np.array([4 * np.pi / k * np.imag(np.conj(exc.pol[i]) @ ff.e[i, :, i]) for i in range(2)]).real
    errs["ext"] = rel(ext, sig.ext)
    record("farfield_" + name, **errs)
    for kk, v in errs.items():
        assert v < 1e-12, (kk, v)
