"""Fields and potentials on the boundary (compgreenret field.m / potential.m
on the particle itself): known answers of the oracle restatement, which the
GPU parity test then uses.

* n . H1p equals the H1 of the matrix assembly (and H2p, H2): the Cartesian
  derivative reuses the pinned refined coefficients (1e-14);
* the potentials of a bemret solution are continuous across the boundary,
  phi1 = phi2 + phi_ext and a1 = a2 + a_ext, which are the BEM equations
  G1 sig1 = G2 sig2 + phi2 and G1 h1 = G2 h2 + a2 (1e-13);
* the normal component of D = eps E is continuous at every face, which the
  bemret conditions (Garcia de Abajo and Howie, Eqs. 15, 18) impose on the
  discrete fields (1e-12); the tangential E is continuous only up to the
  discretisation error (below 2e-3 on a 284-face sphere).
"""
import numpy as np
import pytest

from mnpbem_gb300 import shapes
from oracle import mnpbem_ref as R


@pytest.fixture(scope="module")
def solved():
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    v, f = shapes.trisphere(144, 20.0)
    cp = R.ComParticle([R.EpsConst(1.77), R.drude_eps()], [R.Particle(v, f, q)], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]], R.Particle(vi, fi, q))
    enei = 520.0
    _, _, sols, bem = R.solve_spectrum(cp, pw, [enei])
    return cp, bem, pw.potential(cp, enei), sols[0], enei


def test_cartesian_derivative_matches_assembly(solved):
    cp, bem, _, _, enei = solved
    for a, key, hk in ((0, "H1p", "H1"), (1, "H2p", "H2")):
        Hp, H = bem.g.eval_p(a, a, key, enei), bem.g.eval(a, a, hk, enei)
        assert np.max(np.abs(np.einsum("ic,icj->ij", cp.nvec, Hp) - H)) < 1e-14 * np.max(np.abs(H))
    assert np.isscalar(bem.g.eval_p(0, 1, "H1p", enei))     # no medium shared: block 0


def test_potentials_continuous(solved):
    cp, bem, exc, sig, enei = solved
    args = (bem.g, enei, sig["sig1"], sig["sig2"], sig["h1"], sig["h2"])
    phi1, _, a1, _ = R.surface_potential(*args, inout=1)
    phi2, _, a2, _ = R.surface_potential(*args, inout=2)
    assert np.max(np.abs(phi1 - phi2)) < 1e-13 * np.max(np.abs(phi1))
    assert np.max(np.abs(a1 - (a2 + exc["a2"]))) < 1e-13 * np.max(np.abs(a1))


def test_normal_displacement_continuous(solved):
    cp, bem, exc, sig, enei = solved
    args = (bem.g, enei, sig["sig1"], sig["sig2"], sig["h1"], sig["h2"])
    e1, h1 = R.surface_field(*args, inout=1)
    e2, h2 = R.surface_field(*args, inout=2)
    e2 = e2 + 1j * 2 * np.pi / enei * exc["a2"]          # incoming plane wave E = i k0 a
    nv = cp.nvec[:, :, None]
    eps1, eps2 = cp.eps[1](enei)[0], cp.eps[0](enei)[0]
    dn1, dn2 = eps1 * np.sum(nv * e1, 1), eps2 * np.sum(nv * e2, 1)
    assert np.max(np.abs(dn1 - dn2)) < 1e-12 * np.max(np.abs(dn2))
    tan = lambda e: e - nv * np.sum(nv * e, 1, keepdims=True)      # noqa: E731
    assert np.max(np.abs(tan(e1) - tan(e2))) < 2e-3 * np.max(np.abs(e2))
    assert e1.shape == h1.shape == (cp.n, 3, 2)
