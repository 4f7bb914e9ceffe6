"""Tabulated dielectric functions (Material/@epstable): the package's
``epstable`` against the oracle's own not-a-knot spline restatement on every
shipped table, and known answers: the table values at the tabulated
wavelengths, exact reproduction of cubic n(lambda), k(lambda), the comment
style of the table files and the range check."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import materials
from oracle import mnpbem_ref as R

NAMES = ["gold", "silver", "goldpalik", "silverpalik", "copperpalik"]


def table(name):
    return np.load(materials.os.path.join(materials.os.path.dirname(materials.__file__),
                                          "data", "epstables.npz"))[name]


@pytest.mark.parametrize("name", NAMES)
def test_package_matches_oracle(name):
    tab = table(name)
    got, want = m.epstable(name + ".dat"), R.EpsTable(tab)
    lo, hi = want.enei.min(), want.enei.max()
    enei = np.concatenate([np.linspace(lo, hi, 301), [lo, hi]])
    e1, k1 = got(enei)
    e2, k2 = want(enei)
    assert np.max(np.abs(e1 - e2) / np.abs(e2)) < 1e-11
    assert np.max(np.abs(k1 - k2) / np.abs(k2)) < 1e-11


@pytest.mark.parametrize("name", ["gold", "goldpalik"])
def test_table_points(name):
    tab = table(name)
    eps, k = m.epstable(name + ".dat")(m.EV2NM / tab[:, 0])
    want = (tab[:, 1] + 1j * tab[:, 2]) ** 2
    assert np.max(np.abs(eps - want) / np.abs(want)) < 1e-13
    assert np.allclose(k, 2 * np.pi / (m.EV2NM / tab[:, 0]) * np.sqrt(want), rtol=1e-13, atol=0)


def test_cubic_reproduced_and_file_format(tmp_path):
    lam = np.linspace(300.0, 900.0, 9) + np.array([0, 7, -3, 11, 0, -8, 5, 2, 0])
    n = 0.2 + 1e-3 * lam - 2e-6 * lam ** 2 + 1.5e-9 * lam ** 3
    k = 3.0 - 4e-3 * lam + 1e-6 * lam ** 2 + 2e-9 * lam ** 3
    ene = m.EV2NM / lam
    path = tmp_path / "cubic.dat"
    with open(path, "w") as fh:
        fh.write("% a cubic table\n%  Energy (eV)  n   k\n")
        for row in zip(ene[::-1], n[::-1], k[::-1]):
            fh.write("%.17g\t%.17g\t%.17g   %% trailing comment\n" % row)
    t = np.linspace(lam.min(), lam.max(), 97)
    want = (0.2 + 1e-3 * t - 2e-6 * t ** 2 + 1.5e-9 * t ** 3
            + 1j * (3.0 - 4e-3 * t + 1e-6 * t ** 2 + 2e-9 * t ** 3)) ** 2
    for eps in (m.epstable(str(path))(t)[0], R.EpsTable(np.stack([ene, n, k], 1))(t)[0]):
        assert np.max(np.abs(eps - want) / np.abs(want)) < 1e-11


def test_range_and_missing_file():
    g = m.epstable("gold.dat")
    with pytest.raises(ValueError):
        g([150.0])
    with pytest.raises(ValueError):
        g([520.0, 2500.0])
    with pytest.raises(FileNotFoundError):
        m.epstable("unobtainium.dat")
