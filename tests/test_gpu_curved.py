"""GPU parity for curved boundary elements (interp = 'curv'; 6-node triangles,
9-node quadrilaterals: norm_curv.m, quad_curv.m, quadpol_curv.m) against the
FP64 oracle, through the C ABI (mnpbem_geom_create_curved).

Case: the 508-face sphere with its edge midpoints on the sphere (trisphere.m
curved nodes), d = 20 nm, Drude metal in eps = 1.77.  Tolerances as for flat
elements: geometry 1e-13, near coefficients 1e-12, self coefficients 1e-9,
FP64 matrices 1e-10, FP64 cross sections 1e-10, mixed precision 1e-8.  A rod
of quadrilaterals with flat midpoints must reproduce the flat solution
(1e-6: the cap quadrilaterals are not parallelograms), a triangulated sphere
with flat midpoints to 1e-10, and the curved sphere must sit within 2 % of Mie near the plasmon
resonance where the flat one is 10 % off.
"""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

from test_gpu_parity import drude, rel, record

pytestmark = pytest.mark.gpu


def oracle(cp):
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    parts = [R.Particle.curved(pp.verts2, pp.faces2, q) if pp.curved else R.Particle(pp.verts, pp.faces, q)
             for pp in cp.p]
    ocp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], parts, cp.inout, [bool(c) for c in cp.closed])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    return R, ocp, pw


@pytest.fixture(scope="module")
def sphere(gpu_lib):
    p = m.trisphere(256, 20.0, {"interp": "curv"})
    return m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)


def test_curved_geometry_and_refinement(sphere):
    cp = sphere
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    R, ocp, _ = oracle(cp)
    g = R.CompGreenRet(ocp)
    r = bem.refinement()
    errs = {k: rel(r[k], getattr(ocp, k)) for k in ("pos", "nvec", "tvec1", "tvec2", "area")}
    assert np.array_equal(r["row"], g.g.rows) and np.array_equal(r["col"], g.g.cols)
    diag = r["row"] == r["col"]
    for o in range(6):
        sg, sf = np.max(np.abs(g.g.g[:, o])), np.max(np.abs(g.g.f[:, :, o]))
        errs["g%d_self" % o] = float(np.max(np.abs(r["g"][diag, o] - g.g.g[diag, o])) / sg)
        errs["f%d_self" % o] = float(np.max(np.abs(r["f"][diag, :, o] - g.g.f[diag, :, o])) / sf)
        errs["g%d_near" % o] = float(np.max(np.abs(r["g"][~diag, o] - g.g.g[~diag, o])) / sg)
        errs["f%d_near" % o] = float(np.max(np.abs(r["f"][~diag, :, o] - g.g.f[~diag, :, o])) / sf)
    record("curved_refinement", **errs)
    for k, v in errs.items():
        tol = 1e-9 if "self" in k else (1e-12 if "near" in k else 1e-13)
        assert v < tol, (k, v)


def test_curved_assembly_and_solve(sphere):
    cp = sphere
    R, ocp, pw = oracle(cp)
    enei = [480.0, 520.0]
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    want = R.BemRet(ocp).matrices(520.0)
    got = bem.matrices(520.0, "fp64")
    e = {nm: rel(a, b) for nm, a, b in zip(("G1", "H1", "G2", "H2"), got, want)}
    oext, osca, _, _ = R.solve_spectrum(ocp, pw, enei)
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    r = bem.spectrum(exc, enei)
    e["ext_fp64"], e["sca_fp64"] = rel(r["ext"], oext), rel(r["sca"], osca)
    rm = m.bemsolver(cp, m.bemoptions(precision="mixed")).spectrum(exc, enei)
    e["ext_mixed"], e["sca_mixed"] = rel(rm["ext"], oext), rel(rm["sca"], osca)
    record("curved_solve", **e)
    for nm in ("G1", "H1", "G2", "H2"):
        assert e[nm] < 1e-10, (nm, e[nm])
    assert e["ext_fp64"] < 1e-10 and e["sca_fp64"] < 1e-10, e
    assert e["ext_mixed"] < 1e-8 and e["sca_mixed"] < 1e-8, e
    # physics: curved elements against Mie at the plasmon resonance
    from oracle import mnpbem_ref as Ro
    mie, _ = Ro.mie_ext_sca(Ro.drude_eps(), Ro.EpsConst(1.77), 20.0, [520.0])
    flat = m.bemsolver(m.comparticle([m.epsconst(1.77), drude()], [m.trisphere(256, 20.0)], [[2, 1]], 1),
                       m.bemoptions(precision="fp64")).spectrum(exc, [520.0])
    ec, ef = abs(r["ext"][1, 0] - mie[0]) / mie[0], abs(flat["ext"][0, 0] - mie[0]) / mie[0]
    record("curved_vs_mie", curved=float(ec), flat=float(ef))
    assert ec < 0.02 and ef > 0.05, (ec, ef)


def test_flat_midpoints_reproduce_flat_solution(gpu_lib):
    # triangles: curved elements through flat midpoints are the flat elements
    v, f = shapes.trisphere(144, 20.0)
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    rs = {}
    for interp in ("flat", "curv"):
        cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v, f, {"interp": interp})], [[2, 1]], 1)
        rs[interp] = m.bemsolver(cp, m.bemoptions(precision="fp64")).spectrum(exc, [520.0, 650.0])
    e = {"ext": rel(rs["curv"]["ext"], rs["flat"]["ext"]), "sca": rel(rs["curv"]["sca"], rs["flat"]["sca"])}
    record("curved_flat_midpoints_sphere", **e)
    assert e["ext"] < 1e-10 and e["sca"] < 1e-10, e
    v, f = shapes.trirod(10.0, 40.0, (15, 5, 11))
    exc = m.planewave([0, 0, 1], [1, 0, 0])
    res = {}
    for interp in ("flat", "curv"):
        p = m.particle(v, f, {"interp": interp})
        cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
        res[interp] = m.bemsolver(cp, m.bemoptions(precision="fp64")).spectrum(exc, [600.0, 700.0])
    # the quadrilaterals of the caps are not parallelograms: their rule-18
    # points move slightly (totriangles_curv.m uses the centre as a mid-node)
    e = {"ext": rel(res["curv"]["ext"], res["flat"]["ext"]), "sca": rel(res["curv"]["sca"], res["flat"]["sca"])}
    record("curved_flat_midpoints_rod", **e)
    assert e["ext"] < 1e-6 and e["sca"] < 1e-6, e     # measured 3e-8


def test_gradient_rejects_curved(sphere):
    bem = m.bemsolver(sphere, m.bemoptions(precision="fp64"))
    with pytest.raises(m._lib.MnpbemError) as err:
        bem.ext_gradient(m.planewave([1, 0, 0], [0, 0, 1]), 600.0)
    assert err.value.status == 7     # UNSUPPORTED


def test_curvature_midpoints_rod(gpu_lib):
    """Rod whose curved nodes come from midpoints(p, 'curv') (refine.m): the
    GPU solve on the package's nodes against the oracle on the nodes of its
    own restatement (FP64 1e-10, mixed 1e-8)."""
    from oracle import mnpbem_ref as Ro
    v, f = shapes.trirod(10.0, 40.0, (15, 5, 11))
    p = m.particle(v, f).midpoints("curv")
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    t = shapes.tables()
    q = Ro.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    w2, g2 = Ro.midpoints_curv(v, f)
    ocp = Ro.ComParticle([Ro.EpsConst(1.77), Ro.drude_eps()], [Ro.Particle.curved(w2, g2, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = Ro.PlaneWaveRet([0, 0, 1], [1, 0, 0], Ro.Particle(vi, fi, q))
    enei = [600.0, 700.0]
    oext, osca, _, _ = Ro.solve_spectrum(ocp, pw, enei)
    exc = m.planewave([0, 0, 1], [1, 0, 0])
    r = m.bemsolver(cp, m.bemoptions(precision="fp64")).spectrum(exc, enei)
    rm = m.bemsolver(cp, m.bemoptions(precision="mixed")).spectrum(exc, enei)
    e = {"ext_fp64": rel(r["ext"], oext), "sca_fp64": rel(r["sca"], osca),
         "ext_mixed": rel(rm["ext"], oext), "sca_mixed": rel(rm["sca"], osca)}
    record("curved_curvature_midpoints_rod", **e)
    assert e["ext_fp64"] < 1e-10 and e["sca_fp64"] < 1e-10, e
    assert e["ext_mixed"] < 1e-8 and e["sca_mixed"] < 1e-8, e
