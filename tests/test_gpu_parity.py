"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Cases: the 508-face sphere of the committed fixture (C1 geometry), a 284-face
sphere solved live by the oracle, and a sphere dimer with separate media for
the two particles (block-diagonal G1, dense G2).  Tolerances (max |diff| /
max |ref| unless stated):
  geometry 1e-13; near-pair refinement coefficients 1e-12; self-element
  coefficients 1e-9 (the polar rule puts points 0.5e-6 element radii from the
  centroid, where r = |centroid - point| loses ~9 digits to cancellation in any
  FP64 evaluation of the reference formula); FP64 matrices 1e-10; FP64 bemret
  matrices 1e-9; FP64 solution fields 1e-9 and cross sections 1e-10;
  complex64 assembly 2e-6; double-single assembly (hi + lo) against the FP64
  pass 1e-13; mixed precision (complex64 inversion + FP64 refinement) cross
  sections 1e-8.
Measured errors are appended as JSON lines to the file named by the
environment variable ``MNPBEM_PARITY_LOG`` when it is set.
"""
import json
import os

import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DRUDE = (10.0, 9.065, 0.0708)


def drude():
    e0, wp, g = DRUDE
    return m.epsfun(lambda w: e0 - wp ** 2 / (w * (w + 1j * g)), "eV")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def record(name, **vals):
    path = os.environ.get("MNPBEM_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"test": name, **vals}) + "\n")


@pytest.fixture(scope="module")
def c1(gpu_lib):
    d = np.load(os.path.join(GOLD, "c1_sphere508.npz"))
    p = m.particle(d["verts"], d["faces"])
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    return d, cp


def oracle_setup(cp):
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    parts = [R.Particle(pp.verts, pp.faces, q) for pp in cp.p]
    eps = [R.EpsConst(1.77)] + [R.drude_eps(*DRUDE) for _ in range(len(cp.eps) - 1)]
    ocp = R.ComParticle(eps, parts, cp.inout, [bool(c) for c in cp.closed])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    return R, ocp, pw


def test_geometry_and_refinement_parity(c1):
    d, cp = c1
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    R, ocp, _ = oracle_setup(cp)
    g = R.CompGreenRet(ocp)
    r = bem.refinement()
    assert rel(r["pos"], ocp.pos) < 1e-13 and rel(r["nvec"], ocp.nvec) < 1e-13
    assert rel(r["tvec1"], ocp.tvec1) < 1e-13 and rel(r["tvec2"], ocp.tvec2) < 1e-13
    assert rel(r["area"], ocp.area) < 1e-13
    assert r["row"].size == g.g.ind.size == int(d["nref"])
    assert np.array_equal(r["row"], g.g.rows) and np.array_equal(r["col"], g.g.cols)
    diag = r["row"] == r["col"]
    errs = {}
    # errors relative to the largest coefficient of the same order over all
    # refined elements (some self-element orders are exactly zero or pure
    # rounding noise around zero, e.g. f[:, :, 1] and f[:, :, 3])
    for o in range(6):
        sg, sf = np.max(np.abs(g.g.g[:, o])), np.max(np.abs(g.g.f[:, :, o]))
        errs["g%d_self" % o] = float(np.max(np.abs(r["g"][diag, o] - g.g.g[diag, o])) / sg)
        errs["f%d_self" % o] = float(np.max(np.abs(r["f"][diag, :, o] - g.g.f[diag, :, o])) / sf)
        errs["g%d_near" % o] = float(np.max(np.abs(r["g"][~diag, o] - g.g.g[~diag, o])) / sg)
        errs["f%d_near" % o] = float(np.max(np.abs(r["f"][~diag, :, o] - g.g.f[~diag, :, o])) / sf)
    record("refinement", **errs)
    for k, v in errs.items():
        assert v < (1e-9 if "self" in k else 1e-12), (k, v)


@pytest.mark.parametrize("enei", [450.0, 620.0])
def test_assembly_parity(c1, enei):
    d, cp = c1
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    R, ocp, _ = oracle_setup(cp)
    ob = R.BemRet(ocp)
    want = ob.matrices(enei)
    got = bem.matrices(enei, "fp64")
    got32 = bem.matrices(enei, "fp32")
    names = ("G1", "H1", "G2", "H2")
    e64 = {nm: rel(a, b) for nm, a, b in zip(names, got, want)}
    e32 = {nm + "_c64": rel(a, b) for nm, a, b in zip(names, got32, want)}
    record("assembly_%g" % enei, **e64, **e32)
    for nm, v in e64.items():
        assert v < 1e-10, (nm, v)
    for (nm, v), a in zip(e32.items(), got32):
        assert a.dtype == np.complex64 and v < 2e-6, (nm, v)
    # mixed-precision pass (double-single far field): hi + lo against the FP64 pass
    gotmx = bem.matrices(enei, "mixed")
    emx = {nm + "_ds": rel(a, b) for nm, a, b in zip(names, gotmx, got)}
    record("assembly_ds_%g" % enei, **emx)
    for nm, v in emx.items():
        assert v < 1e-13, (nm, v)


def test_bem_matrices_fp64(c1):
    d, cp = c1
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    R, ocp, _ = oracle_setup(cp)
    ob = R.BemRet(ocp)
    ob.initmat(520.0)
    got = bem.bem_matrices(520.0, "fp64")
    errs = {name: rel(got[name], getattr(ob, name)) for name in ("G1i", "G2i", "Sigma1", "Deltai", "Sigmai")}
    record("bem_matrices_fp64", **errs)
    for name, v in errs.items():
        assert v < 1e-9, (name, v)
    gm = bem.bem_matrices(520.0, "mixed")
    errs = {name: rel(gm[name], getattr(ob, name)) for name in ("G1i", "G2i", "Sigma1", "Deltai", "Sigmai")}
    record("bem_matrices_mixed_c64", **errs)
    for name, v in errs.items():   # TF32 tensor-core products: ~1e-3 before refinement
        assert v < 2e-2, (name, v)


def test_solve_fp64_matches_fixture(c1):
    d, cp = c1
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    sig = bem.mldivide(exc(cp, float(d["enei_sig"])))
    errs = {key: rel(getattr(sig, key), d[key]) for key in ("sig1", "sig2", "h1", "h2")}
    r = bem.spectrum(exc, d["enei"])
    errs["ext"] = rel(r["ext"][:, 0], d["ext"])
    errs["sca"] = rel(r["sca"][:, 0], d["sca"])
    record("solve_fp64_c1", **errs)
    for key in ("sig1", "sig2", "h1", "h2"):
        assert errs[key] < 1e-9, (key, errs[key])
    assert errs["ext"] < 1e-10 and errs["sca"] < 1e-10, errs
    # physics: the same discretisation error against Mie as the oracle
    assert np.median(np.abs(r["ext"][:, 0] - d["mie_ext"]) / d["mie_ext"]) < 0.05


def test_solve_mixed_matches_fixture(c1):
    d, cp = c1
    bem = m.bemsolver(cp, m.bemoptions(precision="mixed"))
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    r = bem.spectrum(exc, d["enei"])
    errs = {"ext": rel(r["ext"][:, 0], d["ext"]), "sca": rel(r["sca"][:, 0], d["sca"]),
            "max_iters": int(r["ir_iters"].max()), "max_resid": float(r["ir_resid"].max())}
    record("solve_mixed_c1", **errs)
    assert errs["ext"] < 1e-8 and errs["sca"] < 1e-8, errs
    assert np.all(r["ir_iters"] >= 1) and np.all(r["ir_resid"] < 1e-9)


def test_live_oracle_two_polarisations(gpu_lib):
    p = m.trisphere(144, 30.0)
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    R, ocp, _ = oracle_setup(cp)
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]], R.Particle(vi, fi, q))
    enei = [480.0, 590.0]
    oext, osca, sols, _ = R.solve_spectrum(ocp, pw, enei)
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        bem = m.bemsolver(cp, m.bemoptions(precision=prec))
        r = bem.spectrum(exc, enei, fields=True)
        errs = {"ext": rel(r["ext"], oext), "sca": rel(r["sca"], osca),
                "sig2": rel(r["sig2"][1], sols[1]["sig2"]), "h1": rel(r["h1"][1], sols[1]["h1"])}
        record("live_two_pol_" + prec, **errs)
        assert errs["ext"] < tol and errs["sca"] < tol, (prec, errs)
        assert errs["sig2"] < 10 * tol and errs["h1"] < 10 * tol, (prec, errs)


def test_dimer_block_structure(gpu_lib):
    d = np.load(os.path.join(GOLD, "dimer_sphere116.npz"))
    p1, p2 = m.particle(d["verts1"], d["faces1"]), m.particle(d["verts2"], d["faces2"])
    cp = m.comparticle([m.epsconst(1.77), drude(), drude()], [p1, p2], [[2, 1], [3, 1]], 1, 2)
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        bem = m.bemsolver(cp, m.bemoptions(precision=prec))
        assert bem.sizes()[1] == int(d["nref"])
        r = bem.spectrum(exc, d["enei"])
        errs = {"ext": rel(r["ext"][:, 0], d["ext"]), "sca": rel(r["sca"][:, 0], d["sca"])}
        record("dimer_" + prec, **errs)
        assert errs["ext"] < tol and errs["sca"] < tol, (prec, errs)
    G1, H1, G2, H2 = bem.matrices(550.0)
    n1 = p1.n
    assert np.all(G1[:n1, n1:] == 0) and np.all(G1[n1:, :n1] == 0)   # con{1,1} block-diagonal
    assert np.all(G2[:n1, n1:] != 0)                                  # con{2,2} full


def test_error_status(gpu_lib):
    p = m.trisphere(60, 10.0)
    cp = m.comparticle([m.epsconst(1.77), drude()], [p], [[2, 1]], 1)
    bem = m.bemsolver(cp)
    with pytest.raises(m._lib.MnpbemError) as e:
        bem.spectrum(m.planewave([1, 0, 0], [0, 0, 1], medium=3), [500.0])
    assert e.value.status == 1
    with pytest.raises(m._lib.MnpbemError):
        bem.spectrum(m.planewave([1, 0, 0], [0, 0, 1]), [-5.0])


def test_concurrent_lanes_match_serial(gpu_lib):
    """Wavelengths in flight on several lanes give the results of one lane.

    1200-face sphere (tensor-core path with 256-wide Gauss-Jordan steps), two
    polarisations, seven wavelengths; the second call on three lanes replays
    the graphs captured by the first."""
    v, f = shapes.fibsphere(1200, 30.0)
    cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v, f)], [[2, 1]], 1)
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    enei = np.linspace(450.0, 700.0, 7)
    bem = m.bemsolver(cp, m.bemoptions(precision="mixed", lanes=1))
    ref = bem.spectrum(exc, enei, fields=True)
    bem.set_lanes(3)
    for rep in range(2):
        r = bem.spectrum(exc, enei, fields=True)
        errs = {"ext": rel(r["ext"], ref["ext"]), "sca": rel(r["sca"], ref["sca"]),
                "sig2": rel(r["sig2"], ref["sig2"]), "h1": rel(r["h1"], ref["h1"])}
        record("lanes3_vs_1_rep%d" % rep, **errs)
        assert errs["ext"] < 1e-12 and errs["sca"] < 1e-12, errs
        assert errs["sig2"] < 1e-10 and errs["h1"] < 1e-10, errs
        assert np.all(np.abs(r["ir_iters"] - ref["ir_iters"]) <= 1)


def test_tensor_core_inversions_at_1200_faces(gpu_lib):
    """n >= 1024: 256-wide Gauss-Jordan steps whose pivot blocks are inverted
    on a CTA cluster and whose updates run on the tensor cores (TF32).  The
    complex64 bemret matrices agree with the FP64 ones to TF32 accuracy, and
    the refined cross sections with the FP64 path to 1e-8."""
    v, f = shapes.fibsphere(1200, 30.0)
    cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v, f)], [[2, 1]], 1)
    b64 = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    bmx = m.bemsolver(cp, m.bemoptions(precision="mixed"))
    M64 = b64.bem_matrices(560.0)
    Mmx = bmx.bem_matrices(560.0)
    errs = {k: rel(Mmx[k], M64[k]) for k in M64}
    record("bem_matrices_mixed_vs_fp64_1200", **errs)
    for k, e in errs.items():
        assert e < 2e-2, (k, errs)
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    enei = [480.0, 560.0, 640.0]
    r64 = b64.spectrum(exc, enei)
    rmx = bmx.spectrum(exc, enei)
    e = {"ext": rel(rmx["ext"], r64["ext"]), "sca": rel(rmx["sca"], r64["sca"]),
         "iters": rmx["ir_iters"].tolist()}
    record("solve_mixed_vs_fp64_1200", **e)
    assert e["ext"] < 1e-8 and e["sca"] < 1e-8, e


def test_batch_of_uneven_particles_matches_single_solves(gpu_lib):
    """mnpbem_solve_batch: a sphere, a capped rod (quadrilaterals) and a rounded
    cube of different face counts, two polarisations, solved together give
    the results of one mnpbem_solve per particle; the FP64 rod also agrees with
    the oracle solved live."""
    v1, f1 = shapes.fibsphere(300, 30.0)
    v2, f2 = shapes.trirod(10.0, 40.0, (17, 5, 9))
    v3, f3 = shapes.tricube(7, 40.0, shapes.rounding_to_e(40.0, 4.0))
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    enei = np.linspace(450.0, 800.0, 5)
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-12)):
        bems = []
        for v, f in ((v1, f1), (v2, f2), (v3, f3)):
            cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v, f)], [[2, 1]], 1)
            bems.append(m.bemsolver(cp, m.bemoptions(precision=prec)))
        single = [b.spectrum(exc, enei) for b in bems]
        batch = m.spectrum_batch([(b, exc, enei) for b in bems])
        for k, (a, b) in enumerate(zip(batch, single)):
            errs = {"ext": rel(a["ext"], b["ext"]), "sca": rel(a["sca"], b["sca"])}
            record("batch_vs_single_%s_%d" % (prec, k), **errs)
            assert errs["ext"] < tol and errs["sca"] < tol, (prec, k, errs)
    # the rod (quadrilateral faces) against the live oracle, FP64
    cp = m.comparticle([m.epsconst(1.77), drude()], [m.particle(v2, f2)], [[2, 1]], 1)
    R, ocp, _ = oracle_setup(cp)
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]], R.Particle(vi, fi, q))
    oext, osca, _, _ = R.solve_spectrum(ocp, pw, enei[:2])
    r = m.bemsolver(cp, m.bemoptions(precision="fp64")).spectrum(exc, enei[:2])
    errs = {"ext": rel(r["ext"], oext), "sca": rel(r["sca"], osca)}
    record("rod_quads_fp64_vs_oracle", **errs)
    assert errs["ext"] < 1e-10 and errs["sca"] < 1e-10, errs
