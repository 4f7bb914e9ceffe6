"""Generate the golden fixtures of the GPU parity tests from the FP64 oracle.

    python tests/golden/make_golden.py

Writes (all inputs are deterministic; no random numbers):

* ``c1_sphere508.npz`` — sphere of diameter 20 nm from the stored 256-point
  set (508 flat triangles), Drude metal eps(w) = 10 - 9.065^2 / (w (w + 0.0708 i))
  (w in eV) in eps = 1.77, x-polarised plane wave along +z, 40 wavelengths
  400..800 nm: oracle extinction / scattering, Mie extinction / scattering,
  and the oracle surface charges and currents at 520 nm.
* ``dimer_sphere116.npz`` — two spheres of diameter 10 nm (60-point set, 116
  faces each) with a 2 nm gap along x, separate media for the two metals,
  polarisation along the dimer axis: oracle ext / sca at 3 wavelengths.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mnpbem_gb300 import shapes  # noqa: E402
from oracle import mnpbem_ref as R  # noqa: E402


def quad():
    t = shapes.tables()
    return R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))


def c1():
    q = quad()
    v, f = shapes.trisphere(256, 20.0)
    p = R.Particle(v, f, q)
    eps = [R.EpsConst(1.77), R.drude_eps()]
    cp = R.ComParticle(eps, [p], [[2, 1]], [True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    enei = np.linspace(400, 800, 40)
    ext, sca, sols, bem = R.solve_spectrum(cp, pw, enei)
    mext, msca = R.mie_ext_sca(eps[1], eps[0], 20.0, enei)
    sig = bem.solve(pw.potential(cp, 520.0))
    np.savez_compressed(os.path.join(HERE, "c1_sphere508.npz"), verts=v, faces=f, enei=enei,
                        ext=ext[:, 0], sca=sca[:, 0], mie_ext=mext, mie_sca=msca, enei_sig=520.0,
                        sig1=sig["sig1"], sig2=sig["sig2"], h1=sig["h1"], h2=sig["h2"],
                        nref=bem.g.g.ind.size)
    print("c1: nref", bem.g.g.ind.size, "ext[0..3]", ext[:3, 0])


def dimer():
    q = quad()
    v1, f1 = shapes.sphere(116, 10.0, center=(-6.0, 0, 0))
    v2, f2 = shapes.sphere(116, 10.0, center=(6.0, 0, 0))
    p1, p2 = R.Particle(v1, f1, q), R.Particle(v2, f2, q)
    eps = [R.EpsConst(1.77), R.drude_eps(), R.drude_eps()]
    cp = R.ComParticle(eps, [p1, p2], [[2, 1], [3, 1]], [True, True])
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([1, 0, 0], [0, 0, 1], R.Particle(vi, fi, q))
    enei = np.array([450.0, 550.0, 700.0])
    ext, sca, sols, bem = R.solve_spectrum(cp, pw, enei)
    np.savez_compressed(os.path.join(HERE, "dimer_sphere116.npz"), verts1=v1, faces1=f1, verts2=v2,
                        faces2=f2, enei=enei, ext=ext[:, 0], sca=sca[:, 0], nref=bem.g.g.ind.size)
    print("dimer: nref", bem.g.g.ind.size, "ext", ext[:, 0])


if __name__ == "__main__":
    c1()
    dimer()
