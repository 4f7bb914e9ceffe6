"""Dipole excitation on the host (Simulation/retarded/@dipoleret): the
product's potentials (potential.m:14-117) equal the oracle's, and the oracle's
decay rates reach the free-space limit far from the particle (total 1 to
2e-3; radiative 1 to the 1.2 % area error of the 508-face sphere at infinity)
and respect the mirror symmetry of a sphere."""
import numpy as np

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


def setup():
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    v, f = shapes.trisphere(144, 20.0)
    ocp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(v, f, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    return q, ocp, R.Particle(vi, fi, q)


def test_potentials_match_oracle():
    q, ocp, pinf = setup()
    drude = m.epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV")
    cp = m.comparticle([m.epsconst(1.77), drude], [m.trisphere(144, 20.0)], [[2, 1]], 1)
    pos = [[0, 0, 15.0], [12.0, 0, 3.0]]
    d = m.dipoleret(cp, pos)
    exc = d(cp, 540.0)
    od = R.DipoleRet(pos, d.dip, d.medium, pinf)
    oexc = od.potential(ocp, 540.0)
    for k in ("phi1", "phi1p", "phi2", "phi2p", "a1", "a1p", "a2", "a2p"):
        ref = oexc[k]
        scale = max(np.max(np.abs(ref)), 1e-300)
        assert np.max(np.abs(getattr(exc, k) - ref)) / scale < 1e-13, k
    assert list(d.medium) == [1, 1] and d.ncol == 6


def test_oracle_decay_rates_free_space_limit():
    _, ocp, pinf = setup()
    dip = np.zeros((2, 3, 2))
    dip[:, :, 0], dip[:, :, 1] = [1, 0, 0], [0, 0, 1]
    d = R.DipoleRet([[0, 0, 400.0], [0, 0, -400.0]], dip, [1, 1], pinf)
    sig = R.BemRet(ocp).solve(d.potential(ocp, 520.0))
    tot, rad = d.decayrate(ocp, sig)
    assert np.max(np.abs(tot - 1)) < 2e-3, tot
    assert np.max(np.abs(rad - 1)) < 0.02, rad
    assert np.allclose(tot[0], tot[1], rtol=1e-6) and np.allclose(rad[0], rad[1], rtol=1e-6)
