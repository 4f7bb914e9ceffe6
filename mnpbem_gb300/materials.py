"""Dielectric functions with MNPBEM's calling convention ``[eps, k] = obj(enei)``.

``enei`` is the light wavelength in vacuum (nm); ``k = 2 pi / enei * sqrt(eps)``
with the principal square root.  Mirrors ``Material/@epsconst``,
``Material/@epsdrude`` (presets of ``@epsdrude/init.m``), ``Material/@epstable``
and ``Material/epsfun.m``; ``EV2NM`` is ``Misc/units.m:2``.
"""
import os

import numpy as np

EV2NM = 1.0 / 8.0655477e-4


class epsconst:
    """Constant dielectric function (Material/@epsconst)."""

    def __init__(self, eps):
        self.eps = complex(eps)

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=np.float64)
        eps = np.full(enei.shape, self.eps, dtype=np.complex128)
        return eps, 2 * np.pi / enei * np.sqrt(eps)

    def __repr__(self):
        return "epsconst(%r)" % (self.eps,)


class epsdrude:
    """Drude dielectric function eps0 - wp^2 / (w (w + i gammad)), w in eV.

    ``epsdrude('Au' | 'Ag' | 'Al')`` uses the presets of @epsdrude/init.m;
    ``epsdrude(eps0=..., wp=..., gammad=...)`` sets the parameters directly.
    """

    def __init__(self, name=None, eps0=None, wp=None, gammad=None):
        if name is not None:
            hartree = 27.2116
            tunit = 0.66 / hartree
            key = name.lower()
            if key in ("au", "gold"):
                rs, e0, gd = 3.0, 10.0, tunit / 10
            elif key in ("ag", "silver"):
                rs, e0, gd = 3.0, 3.3, tunit / 30
            elif key in ("al", "aluminum"):
                rs, e0, gd = 2.07, 1.0, 1.06 / hartree
            else:
                raise ValueError("Material name unknown")
            density = 3 / (4 * np.pi * rs ** 3)
            self.eps0, self.wp, self.gammad = e0, np.sqrt(4 * np.pi * density) * hartree, gd * hartree
        else:
            if eps0 is None or wp is None or gammad is None:
                raise ValueError("epsdrude needs a material name or eps0, wp and gammad")
            self.eps0, self.wp, self.gammad = float(eps0), float(wp), float(gammad)
        self.name = name

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=np.float64)
        w = EV2NM / enei
        eps = self.eps0 - self.wp ** 2 / (w * (w + 1j * self.gammad))
        return eps, 2 * np.pi / enei * np.sqrt(eps)


class epsfun:
    """User dielectric function of wavelength ('nm') or photon energy ('eV')."""

    def __init__(self, fun, key="nm"):
        if key not in ("nm", "eV"):
            raise ValueError("key must be 'nm' or 'eV'")
        self.fun, self.key = fun, key

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=np.float64)
        arg = enei if self.key == "nm" else EV2NM / enei
        eps = np.asarray(self.fun(arg), dtype=np.complex128)
        return eps, 2 * np.pi / enei * np.sqrt(eps)


_EPSTABLES = None


def _shipped_table(name):
    global _EPSTABLES
    if _EPSTABLES is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "epstables.npz")
        _EPSTABLES = dict(np.load(path))
    key = name[:-4] if name.endswith(".dat") else name
    return _EPSTABLES.get(key)


class epstable:
    """Tabulated dielectric function (Material/@epstable/epstable.m:13-40,
    subsref.m:15-31).

    ``finp`` is a text file with ``ene n k`` per line (photon energy in eV,
    refractive index and extinction coefficient; ``%`` starts a comment) or
    the name of a table MNPBEM ships: ``gold.dat``, ``silver.dat`` (Johnson
    and Christy), ``goldpalik.dat``, ``silverpalik.dat``, ``copperpalik.dat``
    (Palik).  n and k are interpolated by cubic not-a-knot splines over the
    wavelength ``EV2NM / ene`` (MATLAB's ``spline``; the table is ordered by
    wavelength first), and ``eps = (n + i k)^2``.  Wavelengths outside the
    table raise ``ValueError`` (subsref.m:19-20 asserts the range)."""

    def __init__(self, finp):
        from scipy.interpolate import CubicSpline
        tab = _shipped_table(os.path.basename(finp)) if not os.path.isfile(finp) else None
        if tab is None:
            if not os.path.isfile(finp):
                raise FileNotFoundError("epstable: no table %r" % (finp,))
            rows = []
            with open(finp) as fh:
                for line in fh:
                    line = line.split("%")[0].strip()
                    if line:
                        rows.append([float(t) for t in line.split()[:3]])
            tab = np.asarray(rows, dtype=np.float64).reshape(-1, 3)
        if tab.shape[0] < 4:
            raise ValueError("epstable: a table needs at least 4 rows")
        enei = EV2NM / tab[:, 0]
        order = np.argsort(enei)
        if np.any(np.diff(enei[order]) <= 0):
            raise ValueError("epstable: photon energies must be distinct")
        self.finp = finp
        self.enei = enei
        self._n = CubicSpline(enei[order], tab[order, 1], bc_type="not-a-knot")
        self._k = CubicSpline(enei[order], tab[order, 2], bc_type="not-a-knot")

    def __call__(self, enei):
        enei = np.asarray(enei, dtype=np.float64)
        if enei.size and (enei.min() < self.enei.min() or enei.max() > self.enei.max()):
            raise ValueError("epstable: wavelength outside the table (%.1f - %.1f nm)"
                             % (self.enei.min(), self.enei.max()))
        eps = (self._n(enei) + 1j * self._k(enei)) ** 2
        return eps, 2 * np.pi / enei * np.sqrt(eps)

    def __repr__(self):
        return "epstable(%r)" % (self.finp,)
