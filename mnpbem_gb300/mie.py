"""Mie theory for spheres in the retarded case (Mie/@mieret, Mie/miesolver.m),
the analytic check MNPBEM users compare a BEM spectrum against.

Coefficients a_l, b_l of miecoefficients.m from the Riccati-Bessel functions
of riccatibessel.m (psi_l(z) = z j_l(z), xi_l(z) = z h_l(z) with their
derivatives through z f_{l-1} - l f_l), for l = 1 .. lmax (lmax = 20 as
@mieret/private/init.m); cross sections of extinction.m / scattering.m:
    ext = 2 pi / k^2 sum (2l + 1) Re(a_l + b_l),
    sca = 2 pi / k^2 sum (2l + 1) (|a_l|^2 + |b_l|^2),
k the wavenumber in the embedding medium.  The embedding medium is taken at
the wavelength itself (the reference evaluates a constant one at 0).
Closed-form series on the host: nothing here is O(faces).
"""
import numpy as np


def _riccati(z, lmax):
    """j_l, h_l (spherical, first kind) and z f_{l-1} - l f_l for l = 1..lmax."""
    from scipy.special import spherical_jn, spherical_yn
    l = np.arange(0, lmax + 1)
    j = spherical_jn(l, z)
    h = j + 1j * spherical_yn(l, z)
    lv = l[1:]
    return j[1:], h[1:], z * j[:-1] - lv * j[1:], z * h[:-1] - lv * h[1:]


class mieret:
    """Mie solver for a sphere of ``diameter`` (nm) with dielectric functions
    ``epsin`` inside and ``epsout`` outside (MNPBEM's dielectric-function
    objects: ``eps, k = eps_obj(enei)``)."""

    def __init__(self, epsin, epsout, diameter, lmax=20):
        self.epsin, self.epsout, self.diameter, self.lmax = epsin, epsout, float(diameter), int(lmax)

    def coefficients(self, enei):
        """``k`` and the Mie coefficients ``a, b [lmax]`` at one wavelength."""
        epsb = complex(np.asarray(self.epsout(np.array([enei]))[0]).ravel()[0])
        k = 2 * np.pi / enei * np.sqrt(epsb)
        epsr = complex(np.asarray(self.epsin(np.array([enei]))[0]).ravel()[0]) / epsb
        nr = np.sqrt(epsr)
        x = k * self.diameter / 2
        j1, _, zjp1, _ = _riccati(nr * x, self.lmax)
        j2, h2, zjp2, zhp2 = _riccati(x + 0j, self.lmax)
        a = (nr ** 2 * j1 * zjp2 - j2 * zjp1) / (nr ** 2 * j1 * zhp2 - h2 * zjp1)
        b = (j1 * zjp2 - j2 * zjp1) / (j1 * zhp2 - h2 * zjp1)
        return k, a, b

    def _sum(self, enei, which):
        enei = np.atleast_1d(np.asarray(enei, dtype=np.float64))
        out = np.zeros(enei.size)
        w = 2 * np.arange(1, self.lmax + 1) + 1
        for i, lam in enumerate(enei):
            k, a, b = self.coefficients(float(lam))
            s = np.real(a + b) if which == "ext" else np.abs(a) ** 2 + np.abs(b) ** 2
            out[i] = np.real(2 * np.pi / k ** 2 * np.sum(w * s))
        return out

    def extinction(self, enei):
        return self._sum(enei, "ext")

    def scattering(self, enei):
        return self._sum(enei, "sca")

    def absorption(self, enei):
        return self.extinction(enei) - self.scattering(enei)

    ext, sca, abs = extinction, scattering, absorption


def miesolver(epsin, epsout, diameter, op=None, **kw):
    """Factory of Mie/miesolver.m for sim = 'ret' (the only case built)."""
    op = dict(op or {}, **kw)
    if op.get("sim", "ret") != "ret":
        raise ValueError("only the retarded Mie solver (sim = 'ret') is available")
    return mieret(epsin, epsout, diameter, op.get("lmax", 20))
