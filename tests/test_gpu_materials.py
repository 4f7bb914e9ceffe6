"""GPU parity with a tabulated dielectric function (epstable('gold.dat'),
Johnson and Christy): a 144-face gold sphere, d = 20 nm, in vacuum, x-polarised
plane wave along +z at 450, 520 and 600 nm, through the C ABI against the
oracle with its own spline of the same table (FP64 1e-10, mixed 1e-8), and
within 10 % of Mie for these flat faces (the oracle itself is 3.5 - 7 % off)."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import materials, shapes

from test_gpu_parity import rel, record

pytestmark = pytest.mark.gpu


def test_gold_table_sphere(gpu_lib):
    from oracle import mnpbem_ref as Ro
    tab = np.load(materials.os.path.join(materials.os.path.dirname(materials.__file__),
                                         "data", "epstables.npz"))["gold"]
    v, f = shapes.trisphere(144, 20.0)
    cp = m.comparticle([m.epsconst(1.0), m.epstable("gold.dat")], [m.particle(v, f)], [[2, 1]], 1)
    t = shapes.tables()
    q = Ro.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    gold = Ro.EpsTable(tab)
    ocp = Ro.ComParticle([Ro.EpsConst(1.0), gold], [Ro.Particle(v, f, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = Ro.PlaneWaveRet([1, 0, 0], [0, 0, 1], Ro.Particle(vi, fi, q))
    enei = [450.0, 520.0, 600.0]
    oext, osca, _, _ = Ro.solve_spectrum(ocp, pw, enei)
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    r = m.bemsolver(cp, m.bemoptions(precision="fp64")).spectrum(exc, enei)
    rm = m.bemsolver(cp, m.bemoptions(precision="mixed")).spectrum(exc, enei)
    mie, _ = Ro.mie_ext_sca(gold, Ro.EpsConst(1.0), 20.0, enei)
    e = {"ext_fp64": rel(r["ext"], oext), "sca_fp64": rel(r["sca"], osca),
         "ext_mixed": rel(rm["ext"], oext), "sca_mixed": rel(rm["sca"], osca),
         "mie": float(np.max(np.abs(r["ext"][:, 0] - mie) / mie))}
    record("gold_table_sphere", **e)
    assert e["ext_fp64"] < 1e-10 and e["sca_fp64"] < 1e-10, e
    assert e["ext_mixed"] < 1e-8 and e["sca_mixed"] < 1e-8, e
    assert e["mie"] < 0.1, e
