"""Differential scattering (``[sca, dsca] = exc.sca(sig)``) on the host: the
package's flux arithmetic over far fields, with the far fields supplied by
the oracle's restatement of farfield.m (the GPU far fields are checked
against the same restatement in test_gpu_farfield.py).  The area-weighted
sum of dsca must equal the oracle's scattering cross section (1e-13)."""
import numpy as np

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


class _Solver:
    """Stands in for a bemret: carries the particle for eps_media."""

    def __init__(self, p):
        self.p = p


def test_dsca_sums_to_oracle_sca(monkeypatch):
    v, f = shapes.trisphere(60, 10.0)
    drude = m.epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV")
    cp = m.comparticle([m.epsconst(1.77), drude], [m.particle(v, f)], [[2, 1]], 1)
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    ocp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(v, f, q)], [[2, 1]], [True])
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    pw = R.PlaneWaveRet(exc.pol, exc.dir, R.Particle(exc.spec.pinfty.verts, exc.spec.pinfty.faces, q))
    enei = 520.0
    ext, sca, sols, _ = R.solve_spectrum(ocp, pw, [enei])
    osig = sols[0]
    sig = m.compstruct(cp, enei, sig1=osig["sig1"], sig2=osig["sig2"], h1=osig["h1"], h2=osig["h2"])

    def fake_farfield(bem, s, dir=None):
        e, h, _ = pw.farfield(ocp, osig, exc.spec.nvec)
        return m.compstruct(cp, enei, e=e, h=h)
    monkeypatch.setattr(exc.spec, "farfield", fake_farfield)
    got, dsca = exc.dscattering(_Solver(cp), sig)
    assert dsca.dsca.shape == (exc.spec.nvec.shape[0], 2)
    assert np.max(np.abs(got - sca[0])) < 1e-13 * np.max(np.abs(sca[0]))
    assert np.allclose(exc.spec.area @ dsca.dsca, got, rtol=1e-14, atol=0)
