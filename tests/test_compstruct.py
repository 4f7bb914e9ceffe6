"""compstruct arithmetic (Particles/@compstruct plus.m, minus.m, uminus.m,
mtimes.m): fields present in both operands are added, fields of one are
kept, a scalar multiplies every field."""
import numpy as np

import mnpbem_gb300 as m


def test_plus_minus_times():
    a = m.compstruct(None, 500.0, phi1=np.array([1.0, 2.0]), a1=np.ones((2, 3)))
    b = m.compstruct(None, 500.0, phi1=np.array([0.5, 0.5]), phi2=np.array([3.0, 4.0]))
    c = a + b
    assert np.array_equal(c.phi1, [1.5, 2.5]) and np.array_equal(c.phi2, [3.0, 4.0])
    assert np.array_equal(c.a1, np.ones((2, 3)))
    assert np.array_equal(a.phi1, [1.0, 2.0])                 # operands unchanged
    d = a - b
    assert np.array_equal(d.phi1, [0.5, 1.5]) and np.array_equal(d.phi2, [-3.0, -4.0])
    e = 2j * a
    assert np.array_equal(e.phi1, [2j, 4j]) and (a * 2j).a1[0, 0] == 2j
    assert np.array_equal((-a).a1, -np.ones((2, 3)))
    assert c.enei == 500.0
