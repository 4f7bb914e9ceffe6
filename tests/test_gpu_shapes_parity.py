"""GPU parity on the benchmark geometries against the FP64 oracle solved live.

The direct solve factors G1, G2 and Sigma into block LDU factors (G1 per
diagonal block when the particles' media do not couple) and inverts Delta by
Gauss-Jordan, each diagonal block inverted with partial pivoting inside the
block (64-wide CUDA-core blocks) or by the 256-wide cluster kernel
(tensor-core path, 1024 faces and more).  The oracle inverts with LAPACK
(partial pivoting over whole columns), as initmat.m's inv does.

Cases (all above 1024 faces, so the mixed path runs on the tensor cores): the
capped rod of the gradient configuration (10 x 40 nm, 2016 triangles,
polarisation along the axis, 650 nm); the rod with quadrilaterals (1224
faces); the rounded cube (40 nm edge, 4 nm rounding, 1350 faces); sphere
dimers (d = 50 nm, 2 x 600 faces) with 2 nm and 1 nm gaps, whose G1 is
factored in two blocks.
Tolerances on ext and sca (relative): FP64 1e-10, mixed precision
(complex64 / TF32 factors with FP64-class refinement to 1e-10) 1e-8; the FP64
surface charges 1e-9 (max |diff| / max |ref|).
"""
import numpy as np
import pytest

import mnpbem_gb300 as m
from mnpbem_gb300 import shapes

pytestmark = pytest.mark.gpu
DRUDE = (10.0, 9.065, 0.0708)


def drude():
    e0, wp, g = DRUDE
    return m.epsfun(lambda w: e0 - wp ** 2 / (w * (w + 1j * g)), "eV")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def solve_both(parts, inout, pol, dirv, enei):
    """(GPU results per precision, oracle results) for one wavelength.

    The refinement pattern (refinematrix.m: (d - rad_j) / rad_i < 3 with d from
    pdist2.m's |a|^2 + |b|^2 - 2 a.b) is decided by the last bits of d for
    pairs at exactly the cutoff, which regular grids (the flat sides of the
    cube) have; the reference's own pattern there depends on its BLAS.  Pairs
    on which the library's pattern and the oracle's differ must lie within
    1e-9 of the cutoff, and the oracle then solves with the library's pattern."""
    from oracle import mnpbem_ref as R
    t = shapes.tables()
    q = R.QuadFace((t["rule18_x"], t["rule18_y"], t["rule18_w"]))
    ocp = R.ComParticle([R.EpsConst(1.77)] + [R.drude_eps(*DRUDE) for _ in parts],
                        [R.Particle(v, f, q) for v, f in parts], inout, [True] * len(parts))
    cp = m.comparticle([m.epsconst(1.77)] + [drude() for _ in parts], [m.particle(v, f) for v, f in parts],
                       inout, *range(1, len(parts) + 1))
    exc = m.planewave([pol], [dirv])
    got = {}
    for prec in ("fp64", "mixed"):
        bem = m.bemsolver(cp, m.bemoptions(precision=prec, lanes=1))
        got[prec] = (bem.spectrum(exc, [enei], fields=True), bem)
    # the library's refinement pattern against the oracle's
    r = got["fp64"][1].refinement()
    pat = np.zeros((cp.n, cp.n), np.int8)
    pat[r["row"], r["col"]] = np.where(r["row"] == r["col"], 2, 1)
    opat = R.refinematrix(ocp)
    diff = np.argwhere(pat != opat)
    if diff.size:
        pos, rad = ocp.pos, ocp.bradius()
        d = np.linalg.norm(pos[diff[:, 0]] - pos[diff[:, 1]], axis=1)
        idist = (d - rad[diff[:, 1]]) / rad[diff[:, 0]]
        assert np.all(np.abs(idist - 3.0) < 1e-9), idist
    vi, fi = shapes.trisphere(256, 2.0)
    pw = R.PlaneWaveRet([pol], [dirv], R.Particle(vi, fi, q))
    ob = R.BemRet(ocp, pattern=pat)
    sig = ob.solve(pw.potential(ocp, enei))
    oext, osca = pw.extinction(ocp, sig), pw.scattering(ocp, sig)
    return got, (np.ravel(oext), np.ravel(osca), sig)


def check(got, want, nblocks=None):
    oext, osca, sig = want
    r64, b64 = got["fp64"]
    rmx, bmx = got["mixed"]
    assert rel(r64["ext"][0], oext) < 1e-10 and rel(r64["sca"][0], osca) < 1e-10
    assert rel(r64["sig2"][0], sig["sig2"]) < 1e-9 and rel(r64["h2"][0], sig["h2"]) < 1e-9
    assert rel(rmx["ext"][0], oext) < 1e-8 and rel(rmx["sca"][0], osca) < 1e-8
    for b in (b64, bmx):
        assert b.stat("block_cond_max") > 0
        if nblocks:
            assert b.stat("g1_blocks") == nblocks


def test_capped_rod_of_the_gradient_configuration(gpu_lib):
    v, f = shapes.trirod(10.0, 40.0, (25, 7, 32), triangles=True)
    assert f.shape[0] == 2016
    got, want = solve_both([(v, f)], [[2, 1]], [0, 0, 1.0], [1.0, 0, 0], 650.0)
    check(got, want, 1)


def test_rod_with_quadrilaterals(gpu_lib):
    v, f = shapes.trirod(10.0, 40.0, (25, 9, 36))     # 1224 faces, 1176 of them quadrilaterals
    assert np.sum(f[:, 3] >= 0) > 1000
    got, want = solve_both([(v, f)], [[2, 1]], [0, 0, 1.0], [1.0, 0, 0], 640.0)
    check(got, want)


def test_rounded_cube(gpu_lib):
    v, f = shapes.tricube(16, 40.0, shapes.rounding_to_e(40.0, 4.0))   # 1350 faces
    got, want = solve_both([(v, f)], [[2, 1]], [1.0, 0, 0], [0, 0, 1.0], 600.0)
    check(got, want)


@pytest.mark.parametrize("gap", [2.0, 1.0])
def test_sphere_dimer_with_narrow_gap(gpu_lib, gap):
    nf = 600
    c = 25.0 + gap / 2
    parts = [shapes.fibsphere(nf, 50.0, center=(-c, 0.0, 0.0)), shapes.fibsphere(nf, 50.0, center=(c, 0.0, 0.0))]
    got, want = solve_both(parts, [[2, 1], [3, 1]], [1.0, 0, 0], [0, 0, 1.0], 700.0)
    check(got, want, 2)
