"""GPU dipole excitation against the oracle: surface charges from external
potentials (mnpbem_solve_potentials; excitation.m + mldivide.m) and the total
and radiative decay rates (decayrate.m) of dipoles 5 nm and 20 nm from a
284-face sphere.  Tolerances: FP64 charges 1e-10, mixed 1e-8; decay rates
(FP64 solve) 1e-9."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

from test_gpu_parity import drude, rel, record

pytestmark = pytest.mark.gpu


def test_dipole_charges_and_decay_rates(gpu_lib):
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    p = m.trisphere(144, 20.0)
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    ocp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(p.verts, p.faces, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pos = [[0, 0, 15.0], [0, 30.0, 0]]
    dip = m.dipoleret(cp, pos)                      # x, y, z at both positions: 6 columns
    od = R.DipoleRet(pos, dip.dip, dip.medium, R.Particle(vi, fi, q))
    enei = 540.0
    osig = R.BemRet(ocp).solve(od.potential(ocp, enei))
    otot, orad = od.decayrate(ocp, osig)
    errs = {}
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        bem = m.bemsolver(cp, m.bemoptions(precision=prec))
        sig = bem.mldivide(dip(cp, enei))
        for k in ("sig1", "sig2", "h1", "h2"):
            errs[k + "_" + prec] = rel(getattr(sig, k), osig[k])
        if prec == "fp64":
            tot, rad, rad0 = dip.decayrate(bem, sig)
            errs["tot"], errs["rad"] = rel(tot, otot), rel(rad, orad)
            assert rad0.shape == tot.shape and np.all(tot > 1)
        for k in ("sig1", "sig2", "h1", "h2"):
            assert errs[k + "_" + prec] < tol, (k, prec, errs)
    record("dipole", **errs, tot_max=float(np.max(otot)))
    assert errs["tot"] < 1e-9 and errs["rad"] < 1e-9, errs
