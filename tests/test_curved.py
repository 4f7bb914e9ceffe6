"""Curved boundary elements (interp = 'curv') on the host: oracle restatement
of norm_curv.m / quad_curv.m / quadpol_curv.m / totriangles_curv.m, the host
mirror of the particle, and the C ABI's argument checks (no GPU needed).

Known answers: curved elements through flat midpoints reproduce the flat
elements (centroids, normals, areas and both quadrature rules to 1e-13; the
tangent basis inside the plane is a different but equally orthonormal choice);
a sphere with midpoints on the sphere has its area within 1e-4 of 4 pi R^2
(flat faces: 1.2 % short) and its extinction near the plasmon resonance within
2 % of Mie (flat: 10 %).
"""
import ctypes

import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


def quad():
    t = shapes.tables()
    return R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))


def rod():
    return shapes.trirod(10.0, 40.0, (15, 5, 11))


@pytest.mark.parametrize("shape", ["sphere", "rod"])
def test_flat_midpoints_reproduce_flat_elements(shape):
    q = quad()
    v, f = shapes.trisphere(144, 20.0) if shape == "sphere" else rod()
    pf = R.Particle(v, f, q)
    v2, f2 = R.midpoints_flat(v, f)
    pc = R.Particle.curved(v2, f2, q)
    for k in ("pos", "nvec", "area"):
        assert np.max(np.abs(getattr(pf, k) - getattr(pc, k))) < 1e-13, k
    # orthonormal bases
    for t1, t2, nv in ((pc.tvec1, pc.tvec2, pc.nvec),):
        assert np.allclose(np.sum(t1 * t2, 1), 0, atol=1e-14) and np.allclose(np.sum(t1 * nv, 1), 0, atol=1e-14)
    idx = np.arange(pf.n)
    a, b = pf.quad_points(idx), pc.quad_points(idx)
    assert np.array_equal(a[2], b[2])
    # per-element weight sums are the areas in both; the points coincide on
    # triangles (a quadrilateral's 6-node halves use its centre as the third
    # mid-node, totriangles_curv.m:25-27, which is the diagonal's midpoint only
    # for parallelograms)
    sa, sb = np.bincount(a[2], a[1]), np.bincount(b[2], b[2] * 0 + b[1])
    assert np.max(np.abs(sa - sb)) < 1e-13
    tri = np.isin(a[2], np.nonzero(pf.faces[:, 3] < 0)[0]) & (np.arange(a[2].size) < idx.size * q.w.size)
    assert np.max(np.abs(a[0][tri] - b[0][tri])) < 1e-13 and np.max(np.abs(a[1][tri] - b[1][tri])) < 1e-14
    a, b = pf.quadpol_points(idx), pc.quadpol_points(idx)
    assert np.max(np.abs(a[0] - b[0])) < 1e-13 and np.max(np.abs(a[1] - b[1])) < 1e-14


def test_curved_sphere_area():
    q = quad()
    v, f = shapes.trisphere(256, 20.0)
    v2, f2 = shapes.trisphere_curved(256, 20.0)
    exact = 4 * np.pi * 10.0 ** 2
    flat = R.Particle(v, f, q).area.sum()
    curv = R.Particle.curved(v2, f2, q).area.sum()
    assert abs(curv - exact) / exact < 1e-4
    assert abs(flat - exact) / exact > 1e-2


def test_host_particle_matches_oracle():
    q = quad()
    p = m.trisphere(256, 20.0, {"interp": "curv"})
    po = R.Particle.curved(p.verts2, p.faces2, q)
    for k in ("pos", "nvec", "area", "tvec1", "tvec2"):
        assert np.max(np.abs(getattr(p, k) - getattr(po, k))) < 1e-13, k
    v, f = rod()
    pr = m.particle(v, f, {"interp": "curv"})          # flat midpoints
    prf = m.particle(v, f)
    for k in ("pos", "nvec", "area"):
        assert np.max(np.abs(getattr(pr, k) - getattr(prf, k))) < 1e-13, k
    # the compound of a curved and a flat particle is curved as a whole
    cp = m.comparticle([m.epsconst(1.0), m.epsconst(2.0)], [p, prf.shift([40.0, 0, 0])], [[2, 1], [2, 1]], 1, 2)
    assert cp.curved and cp.faces2.shape == (cp.n, 9)


def test_midpoints_match_oracle():
    for v, f in (shapes.trisphere(144, 20.0), rod()):
        a2, b2 = shapes.midpoints_flat(v, f)
        c2, d2 = R.midpoints_flat(v, f)
        assert np.array_equal(b2 >= 0, d2 >= 0)
        used = b2 >= 0
        assert np.max(np.abs(a2[np.where(used, b2, 0)] - c2[np.where(used, d2, 0)])) == 0.0


def test_curved_sphere_closer_to_mie():
    q = quad()
    v, f = shapes.trisphere(256, 20.0)
    v2, f2 = shapes.trisphere_curved(256, 20.0)
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    lam = [520.0]
    mie, _ = R.mie_ext_sca(R.drude_eps(), R.EpsConst(1.77), 20.0, lam)
    errs = {}
    for name, part in (("flat", R.Particle(v, f, q)), ("curv", R.Particle.curved(v2, f2, q))):
        cp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [part], [[2, 1]], [True])
        ext, _, _, _ = R.solve_spectrum(cp, pw, lam)
        errs[name] = abs(ext[0, 0] - mie[0]) / mie[0]
    assert errs["curv"] < 0.02 and errs["flat"] > 0.05, errs


def test_curved_create_rejects_bad_nodes():
    from mnpbem_gb300 import _lib
    lib = _lib.load()
    v2, f2 = shapes.trisphere_curved(60, 10.0)
    bad = f2.copy()
    bad[3, 5] = -1                     # a triangle without its edge-23 midpoint
    p = m.trisphere(60, 10.0)
    qd = p.quad
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (qd.x, qd.y, qd.w, qd.x3, qd.y3, qd.w3, qd.x4, qd.y4, qd.w4)]
    Q = _lib.Quad(arrs[0].size, _lib.dptr(arrs[0]), _lib.dptr(arrs[1]), _lib.dptr(arrs[2]),
                  arrs[3].size, _lib.dptr(arrs[3]), _lib.dptr(arrs[4]), _lib.dptr(arrs[5]),
                  arrs[6].size, _lib.dptr(arrs[6]), _lib.dptr(arrs[7]), _lib.dptr(arrs[8]))
    opts = _lib.Options(3.0, 0.0, 5, 0)
    pn = np.array([f2.shape[0]], np.int64)
    io = np.array([2, 1], np.int32)
    cl = np.array([1], np.int32)
    h = ctypes.c_void_p()
    v2 = np.ascontiguousarray(v2)
    bad = np.ascontiguousarray(bad, dtype=np.int64)
    st = lib.mnpbem_geom_create_curved(_lib.dptr(v2), v2.shape[0], bad.ctypes.data_as(_lib.c_int64_p),
                                       bad.shape[0], 1, pn.ctypes.data_as(_lib.c_int64_p),
                                       io.ctypes.data_as(_lib.c_int32_p), cl.ctypes.data_as(_lib.c_int32_p),
                                       ctypes.byref(Q), ctypes.byref(opts), ctypes.byref(h))
    assert st == _lib.INVALID_ARG if hasattr(_lib, "INVALID_ARG") else st == 1
    assert b"invalid node index" in lib.mnpbem_last_error()
