"""GPU parity of the fields and potentials on the boundary itself
(mnpbem_surface_fields: compgreenret field.m / potential.m as bemret.field
and bemret.potential call them) against the oracle on the same surface
charges: a 284-face sphere (flat and curved elements) and a two-sphere dimer
with one medium per sphere, two polarisations, inside and outside.
Tolerance 1e-10 of the largest entry, that of the FP64 matrices: the
singular self coefficient g0 of flat elements (a sum over the polar points
around the centroid) differs from the oracle's by about 1e-11 of the largest
G entry, which the G-based outputs (phi, a, E, H: measured 1e-13 - 4.3e-12)
inherit; the H-based ones (phip, ap) agree to 1e-14, and with curved
elements every output agrees to 1e-14.  The GPU fields must
also keep the normal D continuous (1e-10)."""
import os

import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

from test_gpu_parity import GOLD, drude, rel, record

pytestmark = pytest.mark.gpu


def oracle_greens(cp):
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    parts = [R.Particle.curved(pp.verts2, pp.faces2, q) if pp.curved else R.Particle(pp.verts, pp.faces, q)
             for pp in cp.p]
    eps = [R.EpsConst(1.77)] + [R.drude_eps()] * (len(cp.eps) - 1)
    ocp = R.ComParticle(eps, parts, cp.inout, [bool(c) for c in cp.closed])
    return R, R.BemRet(ocp).g


def cases():
    yield "sphere", m.comparticle([m.epsconst(1.77), drude()], [m.trisphere(144, 20.0)], [[2, 1]], 1)
    yield "curved", m.comparticle([m.epsconst(1.77), drude()],
                                  [m.trisphere(144, 20.0, {"interp": "curv"})], [[2, 1]], 1)
    d = np.load(os.path.join(GOLD, "dimer_sphere116.npz"))
    p1, p2 = m.particle(d["verts1"], d["faces1"]), m.particle(d["verts2"], d["faces2"])
    yield "dimer", m.comparticle([m.epsconst(1.77), drude(), drude()], [p1, p2], [[2, 1], [3, 1]], 1, 2)


@pytest.mark.parametrize("name", ["sphere", "curved", "dimer"])
def test_surface_fields_and_potentials_match_oracle(gpu_lib, name):
    cp = dict(cases())[name]
    enei = 540.0
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]])
    sig = bem.mldivide(exc(cp, enei))
    R, g = oracle_greens(cp)
    args = (g, enei, sig.sig1, sig.sig2, sig.h1, sig.h2)
    errs = {}
    for inout in (1, 2):
        f = bem.field(sig, inout)
        pot = bem.potential(sig, inout)
        we, wh = R.surface_field(*args, inout=inout)
        wphi, wphip, wa, wap = R.surface_potential(*args, inout=inout)
        s = str(inout)
        errs["e%d" % inout], errs["h%d" % inout] = rel(f.e, we), rel(f.h, wh)
        errs["phi%d" % inout] = rel(getattr(pot, "phi" + s), wphi)
        errs["phip%d" % inout] = rel(getattr(pot, "phi" + s + "p"), wphip)
        errs["a%d" % inout] = rel(getattr(pot, "a" + s), wa)
        errs["ap%d" % inout] = rel(getattr(pot, "a" + s + "p"), wap)
    record("surface_fields_" + name, **errs)
    for k, v in errs.items():
        assert v < 1e-10, (k, v)
    # normal D continuity of the GPU fields (plane wave outside: E_inc = i k0 a)
    e1, e2 = bem.field(sig, 1).e, bem.field(sig, 2).e
    k0 = 2 * np.pi / enei
    inc = np.zeros_like(e2)
    for ip in range(2):
        pol, dr = np.array(exc.pol[ip], float), np.array(exc.dir[ip], float)
        inc[:, :, ip] = pol[None, :] * np.exp(1j * k0 * np.sqrt(1.77) * (cp.pos @ dr))[:, None]
    eps_in = np.array([cp.eps[i - 1](enei)[0] for i in np.repeat(cp.inout[:, 0], [q.n for q in cp.p])])
    nv = cp.nvec[:, :, None]
    dn1 = eps_in[:, None] * np.sum(nv * e1, 1)
    dn2 = 1.77 * np.sum(nv * (e2 + inc), 1)
    assert rel(dn1, dn2) < 1e-10, rel(dn1, dn2)


def test_mtimes_inverts_mldivide(gpu_lib):
    """bem * (bem \\ exc) gives the potentials of the charges on both sides
    (mtimes.m), which with the external ones are continuous across the
    boundary: phi1 = phi2, a1 = a2 + a_ext for a plane wave from outside."""
    cp = dict(cases())["sphere"]
    bem = m.bemsolver(cp, m.bemoptions(precision="fp64"))
    exc = m.planewave([1, 0, 0], [0, 0, 1])
    enei = 560.0
    sig = bem.mldivide(exc(cp, enei))
    phi = bem * sig
    pot2 = bem.potential(sig, 2)
    assert np.array_equal(phi.a2, pot2.a2) and np.array_equal(phi.phi2p, pot2.phi2p)
    k0 = 2 * np.pi / enei
    a_ext = (np.array([1.0, 0, 0])[None, :] * np.exp(1j * k0 * np.sqrt(1.77) * cp.pos[:, 2])[:, None]
             / (1j * k0))[:, :, None]
    assert rel(phi.phi1, phi.phi2) < 1e-10
    assert rel(phi.a1, phi.a2 + a_ext) < 1e-10
