"""Adjoint gradient of the extinction cross section (mnpbem_ext_gradient).

1. The CUDA adjoint equals the FP64 oracle adjoint (oracle/adjoint_ref.py,
   itself checked against central finite differences on the CPU) on a sphere
   and a triangulated rod, for the extinction and the scattering cross
   section: vertex gradient and d/d eps to 1e-8 relative (max |diff| / max |ref|).
2. On the capped rod 10 x 40 nm with ~2000 triangles at 650 nm, polarised
   along the axis: directional derivatives along random vertex displacements
   agree with central finite differences of the library's own FP64 solve
   (step 1e-4 nm, refinement pattern unchanged) to 1e-4 relative, and
   d/d eps with finite differences in Re eps and Im eps to 1e-4.
3. torch.autograd.gradcheck through the autograd wrapper on a small sphere.
"""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

pytestmark = pytest.mark.gpu
EPS_IN = complex(-8.5, 0.9)


def solver(v, f, eps=EPS_IN):
    cp = m.comparticle([m.epsconst(1.77), m.epsconst(eps)], [m.particle(v, f)], [[2, 1]], 1)
    return m.bemsolver(cp, m.bemoptions(precision="fp64"))


@pytest.mark.parametrize("shape,which", [("sphere", "ext"), ("rod", "ext"), ("sphere", "sca"), ("rod", "sca")])
def test_gradient_matches_oracle_adjoint(gpu_lib, shape, which):
    from oracle import adjoint_ref as A
    from oracle import mnpbem_ref as R
    if shape == "sphere":
        v, f = shapes.trisphere(32, 10.0)
        pol, dirv = [1.0, 0, 0], [0, 0, 1.0]
    else:
        v, f = shapes.trirod(6.0, 16.0, (9, 4, 5), triangles=True)
        pol, dirv = [0, 0, 1.0], [1.0, 0, 0]
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    vi, fi = shapes.trisphere(256, 2.0)
    J0, gv0, ge0, _ = A.cross_section_gradient(v, f, q, 1.77, EPS_IN, 520.0, pol, dirv, which,
                                               R.Particle(vi, fi, q))
    val, gv, ge = solver(v, f).cross_section_gradient(m.planewave([pol], [dirv]), 520.0, 0, which)
    assert abs(val - J0) / abs(J0) < 1e-10
    assert np.max(np.abs(gv - gv0)) / np.max(np.abs(gv0)) < 1e-8
    assert abs(ge - ge0) / abs(ge0) < 1e-8


def test_gradient_rod_2000_faces_vs_finite_differences(gpu_lib):
    v, f = shapes.trirod(10.0, 40.0, (25, 7, 32), triangles=True)
    assert abs(f.shape[0] - 2000) < 40
    pol, dirv, enei = [0, 0, 1.0], [1.0, 0, 0], 650.0
    exc = m.planewave([pol], [dirv])
    ext, gv, ge = solver(v, f).ext_gradient(exc, enei)
    rng = np.random.default_rng(7)
    h = 1e-4
    for trial in range(3):
        dv = rng.standard_normal(v.shape)
        dv /= np.linalg.norm(dv)
        jp = solver(v + h * dv, f).spectrum(exc, [enei])["ext"][0, 0]
        jm = solver(v - h * dv, f).spectrum(exc, [enei])["ext"][0, 0]
        fd = (jp - jm) / (2 * h)
        ad = float(np.sum(gv * dv))
        assert abs(ad - fd) / abs(fd) < 1e-4, (trial, ad, fd)
    he = 1e-4
    fr = (solver(v, f, EPS_IN + he).spectrum(exc, [enei])["ext"][0, 0]
          - solver(v, f, EPS_IN - he).spectrum(exc, [enei])["ext"][0, 0]) / (2 * he)
    fi = (solver(v, f, EPS_IN + 1j * he).spectrum(exc, [enei])["ext"][0, 0]
          - solver(v, f, EPS_IN - 1j * he).spectrum(exc, [enei])["ext"][0, 0]) / (2 * he)
    assert abs(ge.real - fr) / abs(fr) < 1e-4 and abs(ge.imag - fi) / abs(fi) < 1e-4, (ge, fr, fi)


def test_scattering_gradient_rod_vs_finite_differences(gpu_lib):
    v, f = shapes.trirod(10.0, 40.0, (25, 7, 32), triangles=True)
    pol, dirv, enei = [0, 0, 1.0], [1.0, 0, 0], 650.0
    exc = m.planewave([pol], [dirv])
    sca, gv, ge = solver(v, f).cross_section_gradient(exc, enei, 0, "sca")
    rng = np.random.default_rng(11)
    dv = rng.standard_normal(v.shape)
    dv /= np.linalg.norm(dv)
    h = 1e-4
    jp = solver(v + h * dv, f).spectrum(exc, [enei])["sca"][0, 0]
    jm = solver(v - h * dv, f).spectrum(exc, [enei])["sca"][0, 0]
    fd = (jp - jm) / (2 * h)
    assert abs(float(np.sum(gv * dv)) - fd) / abs(fd) < 1e-4


@pytest.mark.parametrize("which", ["extinction", "scattering"])
def test_autograd_gradcheck(gpu_lib, which):
    torch = pytest.importorskip("torch")
    from mnpbem_gb300 import autograd
    cross_section = getattr(autograd, which)
    v, f = shapes.trisphere(32, 10.0)
    verts = torch.tensor(v, dtype=torch.float64, requires_grad=True)
    eps = torch.tensor([EPS_IN.real, EPS_IN.imag], dtype=torch.float64, requires_grad=True)
    fn = lambda vv, ee: cross_section(vv, ee, f, 520.0)
    # the scattering cross section is ~1e-3 of the extinction on this 10 nm sphere
    atol = 1e-6 if which == "extinction" else 1e-9
    assert torch.autograd.gradcheck(fn, (verts, eps), eps=1e-5, atol=atol, rtol=1e-4, nondet_tol=1e-12)


@pytest.mark.parametrize("which", ["ext", "sca"])
def test_mixed_precision_gradient_matches_fp64(gpu_lib, which):
    """complex64 forward / transposed solves with FP64-class refinement give
    the FP64 gradient on the 2016-face rod to 1e-7 (max |diff| / max |ref|)."""
    v, f = shapes.trirod(10.0, 40.0, (25, 7, 32), triangles=True)
    exc = m.planewave([[0, 0, 1.0]], [[1.0, 0, 0]])
    b = solver(v, f)
    v64, g64, e64 = b.cross_section_gradient(exc, 650.0, 0, which, "fp64")
    vmx, gmx, emx = b.cross_section_gradient(exc, 650.0, 0, which, "mixed")
    assert abs(vmx - v64) / abs(v64) < 1e-9
    assert np.max(np.abs(gmx - g64)) / np.max(np.abs(g64)) < 1e-7
    assert abs(emx - e64) / abs(e64) < 1e-7
