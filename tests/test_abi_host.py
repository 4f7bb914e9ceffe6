"""CPU tests: the C-ABI library builds, loads and exports every symbol that
``include/*.h`` declares; argument validation and the host-side mirror of
MNPBEM's interface (materials, particles, options) behave like the reference.
No compute call reaches a GPU here.
"""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names.update(re.findall(r"MNPBEM_API\s+[\w\s\*]+?\b(mnpbem_\w+)\s*\(", src))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from mnpbem_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_api():
    names = declared_symbols()
    for must in ("mnpbem_geom_create", "mnpbem_solve", "mnpbem_assemble", "mnpbem_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.mnpbem_version().startswith(b"mnpbem-gb300")


def test_python_binding_covers_header(lib):
    from mnpbem_gb300 import _lib
    for name in declared_symbols():
        assert name in _lib.SIGNATURES, name


def test_invalid_arguments_rejected_before_any_device_call(lib):
    from mnpbem_gb300 import _lib
    h = ctypes.c_void_p()
    st = lib.mnpbem_geom_create(None, 0, None, 0, 0, None, None, None, None, None, ctypes.byref(h))
    assert st == 1 and b"invalid" in lib.mnpbem_last_error()
    # faces referring to a vertex that does not exist
    verts = np.zeros((3, 3))
    faces = np.array([[0, 1, 5, -1]], dtype=np.int64)
    pn = np.array([1], dtype=np.int64)
    inout = np.array([2, 1], dtype=np.int32)
    x = np.zeros(3)
    q = _lib.Quad(3, _lib.dptr(x), _lib.dptr(x), _lib.dptr(x), 3, _lib.dptr(x), _lib.dptr(x),
                  _lib.dptr(x), 0, None, None, None)
    st = lib.mnpbem_geom_create(_lib.dptr(verts), 3, faces.ctypes.data_as(_lib.c_int64_p), 1, 1,
                                pn.ctypes.data_as(_lib.c_int64_p), inout.ctypes.data_as(_lib.c_int32_p),
                                None, ctypes.byref(q), None, ctypes.byref(h))
    assert st == 1 and b"vertex" in lib.mnpbem_last_error()
    assert lib.mnpbem_geom_destroy(None) == 0
    assert lib.mnpbem_solve(None, None, 0, None, None, 0, 0, None, None) == 1
    assert lib.mnpbem_solve_batch(None, 0, 0, None) == 1
    assert lib.mnpbem_geom_set_lanes(None, 2) == 1
    assert lib.mnpbem_ext_gradient(None, None, 0, 500.0, None, 0, 0, None, None, None) == 1
    assert lib.mnpbem_surface_fields(None, 500.0, None, 0, 1, 2, *([None] * 10)) == 1
    assert lib.mnpbem_farfield(None, 500.0, None, 0, 1, 1, None, 1, *([None] * 6)) == 1
    assert lib.mnpbem_geom_stat(None, b"block_cond_max", None) == 1
    assert lib.mnpbem_selftest_bounded_wait(0, 0) == 1          # limit out of range
    assert lib.mnpbem_selftest_bounded_wait(0, 2000000) == 1


def test_materials():
    from mnpbem_gb300 import EV2NM, epsconst, epsdrude, epsfun
    e, k = epsconst(1.77)([500.0, 600.0])
    assert np.allclose(e, 1.77) and np.allclose(k, 2 * np.pi / np.array([500, 600]) * np.sqrt(1.77))
    f = epsfun(lambda w: 10 - 9.065 ** 2 / (w * (w + 0.0708j)), "eV")
    e, k = f(np.array([620.0]))
    w = EV2NM / 620.0
    assert np.allclose(e, 10 - 9.065 ** 2 / (w * (w + 0.0708j)))
    au = epsdrude("Au")
    assert abs(au.eps0 - 10) < 1e-12 and abs(au.wp - 9.0705) < 2e-3 and abs(au.gammad - 0.066) < 1e-3
    e, k = au(500.0)
    assert np.isclose(k, 2 * np.pi / 500 * np.sqrt(e))


def test_particles_and_options():
    import mnpbem_gb300 as m
    op = m.bemoptions(sim="ret", interp="flat")
    assert op["RelCutoff"] == 3 and op["order"] == 5
    p = m.trisphere(144, 10.0)
    assert p.n == 284 and np.all(np.sum(p.nvec * p.pos, 1) > 0)
    cp = m.comparticle([m.epsconst(1.0), m.epsdrude("Au")], [p, p.shift([12, 0, 0])],
                       [[2, 1], [2, 1]], 1, 2, op=op)
    assert cp.n == 568 and list(cp.closed) == [1, 1]
    assert cp.eps_media([500.0, 600.0]).shape == (2, 2)
    with pytest.raises(ValueError):
        m.comparticle([m.epsconst(1.0)], [p], [[2, 1]])
    with pytest.raises(ValueError):
        m.planewave([1, 0, 0], [1, 0, 0])
    exc = m.planewave([[1, 0, 0], [0, 1, 0]], [[0, 0, 1], [0, 0, 1]], op)
    assert exc.npol == 2 and exc.spec.pinfty.n == 508
    q = m.quadface()
    assert q.x.size == 28 and q.x3.size == 144 and q.x4.size == 192


def test_fibsphere_counts():
    from mnpbem_gb300 import shapes
    for nf in (1000, 4000):
        v, f = shapes.fibsphere(nf, 50.0)
        assert f.shape[0] == nf
        cen = v[f[:, :3]].mean(1)
        nv = np.cross(v[f[:, 0]] - v[f[:, 1]], v[f[:, 2]] - v[f[:, 1]])
        assert np.all(np.sum(nv * cen, 1) > 0)


def test_autotune_settings_lookup(tmp_path, monkeypatch):
    import json
    from mnpbem_gb300 import autotune
    f = tmp_path / "tuned.json"
    f.write_text(json.dumps({"4000": {"options": {"lanes": 6, "tc_stages": 4, "gj_block": 256}},
                             "24000": {"options": {"lanes": 3}}}))
    monkeypatch.setattr(autotune, "TUNED", str(f))
    assert autotune.settings_for(3000, "mixed") == {"lanes": 6, "tc_stages": 4, "gj_block": 256}
    assert autotune.settings_for(20000, "mixed") == {"lanes": 3}
    assert autotune.settings_for(500, "mixed") == {}          # nothing within a factor of 2
    assert autotune.settings_for(4000, "fp64") == {}


def test_set_option_validation(lib):
    assert lib.mnpbem_geom_set_option(None, b"lanes", 2) == 1
