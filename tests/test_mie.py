"""Mie solver of the package (mieret / miesolver) against the oracle's
restatement (which uses Bessel functions of half-integer order where the
package uses spherical Bessel functions), for a Drude sphere and a tabulated
gold sphere: 1e-10; ext = sca + abs; the quasistatic limit of a small
sphere, ext = k Im(alpha) with alpha = 4 pi a^3 (eps - epsb) / (eps + 2 epsb)."""
import numpy as np
import pytest

import mnpbem_gb300 as m
from oracle import mnpbem_ref as R

ENEI = np.linspace(400.0, 800.0, 21)


@pytest.mark.parametrize("metal", ["drude", "gold"])
def test_matches_oracle(metal):
    if metal == "drude":
        eps_in, o_in = m.epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV"), R.drude_eps()
    else:
        eps_in = m.epstable("gold.dat")
        o_in = R.EpsTable(np.load(m.materials.os.path.join(
            m.materials.os.path.dirname(m.materials.__file__), "data", "epstables.npz"))["gold"])
    mie = m.miesolver(eps_in, m.epsconst(1.77), 30.0)
    ext, sca = R.mie_ext_sca(o_in, R.EpsConst(1.77), 30.0, ENEI)
    assert np.max(np.abs(mie.ext(ENEI) - ext) / np.abs(ext)) < 1e-10
    assert np.max(np.abs(mie.sca(ENEI) - sca) / np.abs(sca)) < 1e-10
    assert np.allclose(mie.abs(ENEI), mie.ext(ENEI) - mie.sca(ENEI), rtol=0, atol=1e-12 * ext.max())


def test_quasistatic_limit():
    eps = m.epsconst(-2.0 + 0.3j)
    mie = m.mieret(eps, m.epsconst(1.0), 2.0)        # 2 nm sphere at 600 nm
    k = 2 * np.pi / 600.0
    alpha = 4 * np.pi * 1.0 ** 3 * (-3.0 + 0.3j) / (-2.0 + 0.3j + 2.0)
    assert abs(mie.ext(600.0)[0] - k * alpha.imag) < 1e-3 * k * alpha.imag
    with pytest.raises(ValueError):
        m.miesolver(eps, m.epsconst(1.0), 2.0, sim="stat")
