"""CPU tests of the FP64 oracle against independent known answers.

MNPBEM ships no tests or golden outputs for this path, so the oracle is pinned
by mathematics and physics: exactness of the quadrature rules, Legendre-Gauss-
Lobatto nodes, the Fuchs-Liu closed-surface sum rule, consistency of the direct
bemret solve with the full BEM operator, energy conservation of Mie theory and
convergence of BEM to Mie theory, plus regression against the committed
fixtures made by ``tests/golden/make_golden.py``.
"""
import math
import os

import numpy as np
import pytest

from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def quad():
    t = shapes.tables()
    return R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))


def sphere_setup(npts=144, diameter=20.0):
    q = quad()
    v, f = shapes.trisphere(npts, diameter)
    p = R.Particle(v, f, q)
    eps = [R.EpsConst(1.77), R.drude_eps()]
    cp = R.ComParticle(eps, [p], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    return cp, pw, eps


def test_rule18_exact_to_degree_11():
    q = quad()
    for a in range(12):
        for b in range(12 - a):
            exact = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
            got = 0.5 * np.sum(q.w * q.x ** a * q.y ** b)
            assert abs(got - exact) < 1e-15 * max(1.0, 1 / exact)


def test_lglnodes_known_values():
    x, w = R.lglnodes(2)
    assert np.allclose(x, [1, 0, -1], atol=1e-15)
    assert np.allclose(w, [1 / 3, 4 / 3, 1 / 3], atol=1e-15)
    x, w = R.lglnodes(7)
    assert x.size == 8 and abs(w.sum() - 2) < 1e-14
    # exact for polynomials of degree 2n-1
    for d in range(14):
        assert abs(np.sum(w * x ** d) - (2 / (d + 1) if d % 2 == 0 else 0)) < 1e-13


def test_polar_rules():
    q = quad()
    assert q.x3.size == 144 and q.x4.size == 192
    assert abs(q.w3.sum() - 1) < 1e-14 and abs(q.w4.sum() - 4) < 1e-13
    # centroid of the unit triangle and of [-1, 1]^2
    assert abs(np.sum(q.w3 * q.x3) - 1 / 3) < 1e-6 and abs(np.sum(q.w3 * q.y3) - 1 / 3) < 1e-6
    assert abs(np.sum(q.w4 * q.x4)) < 1e-12 and abs(np.sum(q.w4 * q.y4)) < 1e-12


def test_sum_rule_closed_surface():
    cp, pw, eps = sphere_setup(60, 10.0)
    g = R.CompGreenRet(cp)
    n = cp.n
    F0 = g.g.eval_F_indexed(np.repeat(np.arange(n), n), np.tile(np.arange(n), n), 0.0).real.reshape(n, n)
    colsum = (cp.area[:, None] * F0).sum(0) / cp.area
    assert np.max(np.abs(colsum + 2 * np.pi)) < 1e-12


def test_refinement_pattern_density():
    cp, pw, eps = sphere_setup(256, 20.0)
    ir = R.refinematrix(cp)
    assert np.all(np.diag(ir) == 2)
    assert 35 < np.count_nonzero(ir) / cp.n < 50


def test_direct_solve_satisfies_full_operator():
    cp, pw, eps = sphere_setup(144, 20.0)
    bem = R.BemRet(cp)
    exc = pw.potential(cp, 560.0)
    sig = bem.solve(exc)
    phi, a, alpha, De = bem.excitation(exc)
    rp, ra, rD, ral = bem.afun(sig["sig1"], sig["h1"], sig["sig2"], sig["h2"])
    scale = max(np.abs(a).max(), np.abs(alpha).max(), np.abs(De).max())
    for got, want in ((rp, phi), (ra, a), (rD, De), (ral, alpha)):
        assert np.max(np.abs(got - want)) < 1e-10 * scale


def test_mie_lossless_energy_conservation():
    # a lossless sphere scatters all it removes: ext == sca
    ext, sca = R.mie_ext_sca(R.EpsConst(4.0), R.EpsConst(1.0), 100.0, [400.0, 600.0])
    assert np.allclose(ext, sca, rtol=1e-10)
    # small-sphere (Rayleigh) limit of extinction for a lossy sphere
    ein, eb, d, lam = R.EpsConst(-2.0 + 0.5j), R.EpsConst(1.0), 1.0, 500.0
    ext, sca = R.mie_ext_sca(ein, eb, d, [lam])
    k = 2 * np.pi / lam
    alpha = 4 * np.pi * (d / 2) ** 3 * ((-2.0 + 0.5j) - 1) / ((-2.0 + 0.5j) + 2)
    assert abs(ext[0] - k * np.imag(alpha)) / ext[0] < 1e-3


def test_bem_converges_to_mie():
    errs = []
    for npts in (144, 256):
        cp, pw, eps = sphere_setup(npts, 20.0)
        ext, sca, _, _ = R.solve_spectrum(cp, pw, [600.0])
        mext, _ = R.mie_ext_sca(eps[1], eps[0], 20.0, [600.0])
        errs.append(abs(ext[0, 0] - mext[0]) / mext[0])
    assert errs[1] < errs[0] < 0.1


def test_oracle_matches_committed_fixture():
    d = np.load(os.path.join(GOLD, "c1_sphere508.npz"))
    q = quad()
    p = R.Particle(d["verts"], d["faces"], q)
    eps = [R.EpsConst(1.77), R.drude_eps()]
    cp = R.ComParticle(eps, [p], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    sel = [0, 17, 39]
    ext, sca, _, _ = R.solve_spectrum(cp, pw, d["enei"][sel])
    assert np.allclose(ext[:, 0], d["ext"][sel], rtol=1e-11)
    assert np.allclose(sca[:, 0], d["sca"][sel], rtol=1e-11)
    # the committed Mie values and the BEM spectrum agree to the discretisation
    # error of 508 flat faces: same resonance, a few per cent off it
    assert abs(int(np.argmax(d["ext"])) - int(np.argmax(d["mie_ext"]))) <= 1
    assert np.median(np.abs(d["ext"] - d["mie_ext"]) / d["mie_ext"]) < 0.05


@pytest.mark.parametrize("n", [60, 256])
def test_trisphere_mesh(n):
    v, f = shapes.trisphere(n, 2.0)
    assert f.shape[0] == 2 * n - 4
    assert np.all(f[:, 3] == -1)
    p = R.Particle(v, f, quad())
    assert np.all(np.sum(p.nvec * p.pos, 1) > 0)       # outward normals
    assert 0 < (4 * np.pi - p.area.sum()) / (4 * np.pi) < 0.1   # flat faces lie inside
